// Host-side immersed-boundary geometry: the input producer for the pressure
// solve.  In the reference this layer (set_boundary, IBM/BOUNDARY_SET.F90:8-51)
// stays on the host and feeds the solver iblank, the ghost-cell list and the
// image-point interpolation coefficients.  This file restates it in C++ for
// closed triangulated surfaces (UNSTRUCTURED_SURFACE bodies):
//   - icosphere surface generation (stands in for unstruc_surface_in.dat,
//     IBM/BOUNDARY_MARKER_INIT.F90:209-247),
//   - iblank by directional (scan-line) fill of cell centres enclosed by the
//     surface (the fill step of IBM/BOUNDARY_IBLANK_FAST.F90:2-501), then the
//     reference's clean-up passes for a solid body (IBM/BOUNDARY_SET.F90:267-410),
//   - ghost marks and the ordered ghost list (IBM/GCM_SET_BOUNDARY.F90:49-118),
//   - body intercept by the reference's selection rules (the first element
//     whose normal projection passes the area test, else an edge foot from the
//     closest marker, over the three closest markers;
//     IBM/GCM_INTERCEPT_KERNELS_UNSTRUC.F90:26-398), with the reference's
//     inward element normals (IBM/BOUNDARY_SET_ARCLENGTH_NORM.F90:69-165,200-320),
//   - image point, stencil cell search and the Neumann Vandermonde inverse
//     (IBM/GCM_SET_BOUNDARY.F90:124-494, LU with partial pivoting in place of
//     DGETRF/DGETRI from IBM/Lapack_VICAR.F90).
// Arrays are Fortran column-major with lower bound 0, as in the reference.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <utility>
#include <vector>

namespace {

struct V3 { double x, y, z; };
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator*(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }

inline size_t fidx(int nx, int ny, int i, int j, int k)
{
    return (size_t)i + (size_t)(nx + 2) * ((size_t)j + (size_t)(ny + 2) * (size_t)k);
}

// The reference's surface conventions (IBM/BOUNDARY_SET_ARCLENGTH_NORM.F90:
// 69-165, 200-320): element normals point INTO the body, n = (p2 - p1) x
// (p3 - p2) / |.| over the nodes in inward order, centroid (p1 + p2 + p3) / 3.
// A closed surface given outward (positive signed volume, as fsi_geom_icosphere
// writes it) is read with nodes 2 and 3 swapped, as determine_norm_dir_unstruc
// reorders it.
struct Surface {
    int nv = 0, nt = 0;
    const double *verts = nullptr;
    std::vector<int> nodes;               // (3, nt), inward order
    std::vector<V3> nrm;                  // inward unit normals
    std::vector<std::vector<int>> vtri;   // marker -> its elements, ascending
    V3 p(int m) const { return V3{verts[3 * m], verts[3 * m + 1], verts[3 * m + 2]}; }
    int node(int e, int q) const { return nodes[3 * (size_t)e + q]; }
};

Surface make_surface(int nv, const double *verts, int nt, const int32_t *tris)
{
    Surface s;
    s.nv = nv; s.nt = nt; s.verts = verts;
    double vol6 = 0.0;
    for (int t = 0; t < nt; ++t) {
        V3 a = s.p(tris[3 * t]), b = s.p(tris[3 * t + 1]), c = s.p(tris[3 * t + 2]);
        vol6 += dot(a, cross(b, c));
    }
    const bool outward = vol6 > 0.0;
    s.nodes.resize(3 * (size_t)nt);
    for (int t = 0; t < nt; ++t) {
        s.nodes[3 * (size_t)t] = tris[3 * t];
        s.nodes[3 * (size_t)t + 1] = outward ? tris[3 * t + 2] : tris[3 * t + 1];
        s.nodes[3 * (size_t)t + 2] = outward ? tris[3 * t + 1] : tris[3 * t + 2];
    }
    s.nrm.resize(nt);
    s.vtri.assign(nv, {});
    for (int t = 0; t < nt; ++t) {
        V3 p1 = s.p(s.node(t, 0)), p2 = s.p(s.node(t, 1)), p3 = s.p(s.node(t, 2));
        V3 a = p2 - p1, b = p3 - p2;
        V3 n{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
        double mag = std::sqrt(n.x * n.x + n.y * n.y + n.z * n.z);
        s.nrm[t] = V3{n.x / mag, n.y / mag, n.z / mag};
        for (int q = 0; q < 3; ++q) s.vtri[s.node(t, q)].push_back(t);
    }
    return s;
}

// The angle between a and b as the reference's vector_angle takes it
// (IBM/AMODULES.F90:968-988): acos of the cosine, 0 or pi outside (-1, 1).
double vec_angle(V3 a, V3 b)
{
    auto len = [](V3 v) { double s = 0.0; s = s + v.x * v.x; s = s + v.y * v.y; s = s + v.z * v.z; return std::sqrt(s); };
    double c = dot(a, b) / (len(a) * len(b));
    if (c < 1.0 && c > -1.0) return std::acos(c);
    return c > 0.0 ? 0.0 : 4.0 * std::atan(1.0);
}

// Normal projection of p onto element e's plane and the Heron-area test of
// check_BIInsideTriangle (IBM/BOUNDARY_IBLANK_FAST.F90:1028-1159): inside when
// |area(124) + area(234) + area(314) - area(123)| < 1e-4 area(123).
bool project_inside(const Surface &s, int e, V3 p, V3 &bi)
{
    const V3 n = s.nrm[e];
    const V3 p1 = s.p(s.node(e, 0)), p2 = s.p(s.node(e, 1)), p3 = s.p(s.node(e, 2));
    double plane = -n.x * p1.x - n.y * p1.y - n.z * p1.z;
    double d = -(n.x * p.x + n.y * p.y + n.z * p.z + plane);
    bi = V3{p.x + n.x * d, p.y + n.y * d, p.z + n.z * d};
    auto side = [](V3 a, V3 b) {
        return std::sqrt((a.x - b.x) * (a.x - b.x) + (a.y - b.y) * (a.y - b.y) + (a.z - b.z) * (a.z - b.z));
    };
    double s12 = side(p2, p1), s23 = side(p3, p2), s31 = side(p1, p3);
    double s14 = side(bi, p1), s24 = side(bi, p2), s34 = side(bi, p3);
    auto heron = [](double a, double b, double c) {
        double h = 0.5 * (a + b + c);
        return std::sqrt(h * (h - a) * (h - b) * (h - c));
    };
    double a123 = heron(s12, s23, s31);
    double diff = heron(s12, s24, s14) + heron(s23, s24, s34) + heron(s31, s34, s14) - a123;
    return std::fabs(diff) < 1.0e-4 * a123;
}

// Body intercept of the point p (GCM_calc_bodyIntercept_Unstruc,
// IBM/GCM_INTERCEPT_KERNELS_UNSTRUC.F90:26-398).  For each of the three
// closest markers: the first of its elements (ascending) whose normal
// projection passes the inside test gives the intercept; failing that, the
// element whose outward normal makes the smallest angle with (p - marker)
// (last of equals) is taken and the intercept is the nearer foot on its two
// edges that leave the marker, clamped to the marker.  Of the three
// candidates the nearest (first of equals) wins.
void body_intercept(const Surface &s, V3 p, V3 &bi, int &elem)
{
    int best[3] = {-1, -1, -1};
    double bd[3] = {1e300, 1e300, 1e300};
    for (int m = 0; m < s.nv; ++m) {
        V3 q = s.p(m);
        double dx = q.x - p.x, dy = q.y - p.y, dz = q.z - p.z;
        double d = dx * dx + dy * dy + dz * dz;
        for (int r = 0; r < 3; ++r)
            if (d < bd[r]) {
                for (int u = 2; u > r; --u) { bd[u] = bd[u - 1]; best[u] = best[u - 1]; }
                bd[r] = d; best[r] = m;
                break;
            }
    }
    V3 cand[3];
    int cel[3];
    for (int c = 0; c < 3; ++c) {
        const int mk = best[c];
        const V3 cv = s.p(mk);
        int ce = -1;
        bool found = false;
        double angMin = 1.0e16;
        V3 b{0, 0, 0};
        for (int e : s.vtri[mk]) {
            V3 t;
            if (project_inside(s, e, p, t)) { b = t; ce = e; found = true; break; }
            double ang = vec_angle(p - cv, -1.0 * s.nrm[e]);
            if (ang <= angMin) { angMin = ang; ce = e; b = t; }
        }
        if (!found) {
            int a = s.node(ce, 0), bb = s.node(ce, 1), cc = s.node(ce, 2), na, nb;
            if (a == mk) { na = bb; nb = cc; }
            else if (bb == mk) { na = cc; nb = a; }
            else { na = a; nb = bb; }
            const V3 v01 = p - cv;
            double dmin = 1.0e16;
            V3 ei = cv;
            for (int edge = 0; edge < 2; ++edge) {
                V3 v12 = s.p(edge == 0 ? na : nb) - cv;
                double mag = std::sqrt(v12.x * v12.x + v12.y * v12.y + v12.z * v12.z);
                double inv = 1.0 / mag;
                v12 = V3{v12.x * inv, v12.y * inv, v12.z * inv};
                double pl = v01.x * v12.x + v01.y * v12.y + v01.z * v12.z;
                V3 t = (pl < 0.0 || pl > mag) ? cv : V3{cv.x + pl * v12.x, cv.y + pl * v12.y, cv.z + pl * v12.z};
                double d = (t.x - p.x) * (t.x - p.x) + (t.y - p.y) * (t.y - p.y) + (t.z - p.z) * (t.z - p.z);
                if (d < dmin) { dmin = d; ei = t; }
            }
            b = ei;
        }
        cand[c] = b;
        cel[c] = ce;
    }
    int w = 0;
    double dw = 0.0;
    for (int c = 0; c < 3; ++c) {
        V3 r = cand[c] - p;
        double d = r.x * r.x + r.y * r.y + r.z * r.z;
        if (c == 0 || d < dw) { dw = d; w = c; }
    }
    bi = cand[w];
    elem = cel[w];
}

// In-place inverse of an 8x8 column-major matrix by LU with partial pivoting.
bool inv8(double *A)
{
    const int n = 8;
    int piv[8];
    for (int k = 0; k < n; ++k) {
        int p = k;
        double mx = std::fabs(A[k + n * k]);
        for (int i = k + 1; i < n; ++i)
            if (std::fabs(A[i + n * k]) > mx) { mx = std::fabs(A[i + n * k]); p = i; }
        piv[k] = p;
        if (mx == 0.0) return false;
        if (p != k)
            for (int j = 0; j < n; ++j) std::swap(A[k + n * j], A[p + n * j]);
        for (int i = k + 1; i < n; ++i) {
            A[i + n * k] /= A[k + n * k];
            for (int j = k + 1; j < n; ++j) A[i + n * j] -= A[i + n * k] * A[k + n * j];
        }
    }
    // invert U then solve inv(A) * L = inv(U), undo pivots (the DGETRI scheme)
    for (int j = 0; j < n; ++j) {
        A[j + n * j] = 1.0 / A[j + n * j];
        double ajj = -A[j + n * j];
        double tmp[8];
        for (int i = 0; i < j; ++i) tmp[i] = A[i + n * j];
        for (int i = 0; i < j; ++i) {
            double s = 0.0;
            for (int l = i; l < j; ++l) s += A[i + n * l] * tmp[l];
            A[i + n * j] = s;
        }
        for (int i = 0; i < j; ++i) A[i + n * j] *= ajj;
    }
    for (int j = n - 2; j >= 0; --j) {
        double work[8];
        for (int i = j + 1; i < n; ++i) { work[i] = A[i + n * j]; A[i + n * j] = 0.0; }
        for (int i = 0; i < n; ++i) {
            double s = 0.0;
            for (int l = j + 1; l < n; ++l) s += A[i + n * l] * work[l];
            A[i + n * j] -= s;
        }
    }
    for (int j = n - 2; j >= 0; --j) {
        int jp = piv[j];
        if (jp != j)
            for (int i = 0; i < n; ++i) std::swap(A[i + n * j], A[i + n * jp]);
    }
    return true;
}

} // namespace

extern "C" {

// Icosahedron subdivided nsub times and projected onto a sphere; outward-oriented
// triangles.  nsub = 4 gives 2562 vertices and 5120 triangles.  Returns 0, or -1
// if the capacities are too small (the required counts are still written).
int fsi_geom_icosphere(int nsub, double radius, double cx, double cy, double cz,
                       double *verts, int cap_verts, int32_t *tris, int cap_tris,
                       int *nv_out, int *nt_out)
{
    const double t = (1.0 + std::sqrt(5.0)) / 2.0;
    std::vector<V3> v = {{-1, t, 0}, {1, t, 0}, {-1, -t, 0}, {1, -t, 0}, {0, -1, t}, {0, 1, t},
                         {0, -1, -t}, {0, 1, -t}, {t, 0, -1}, {t, 0, 1}, {-t, 0, -1}, {-t, 0, 1}};
    std::vector<int> f = {0, 11, 5, 0, 5, 1, 0, 1, 7, 0, 7, 10, 0, 10, 11, 1, 5, 9, 5, 11, 4,
                          11, 10, 2, 10, 7, 6, 7, 1, 8, 3, 9, 4, 3, 4, 2, 3, 2, 6, 3, 6, 8,
                          3, 8, 9, 4, 9, 5, 2, 4, 11, 6, 2, 10, 8, 6, 7, 9, 8, 1};
    for (auto &p : v) { double s = 1.0 / std::sqrt(dot(p, p)); p = s * p; }
    for (int s = 0; s < nsub; ++s) {
        std::map<std::pair<int, int>, int> mid;
        auto midpoint = [&](int a, int b) {
            auto key = std::make_pair(std::min(a, b), std::max(a, b));
            auto it = mid.find(key);
            if (it != mid.end()) return it->second;
            V3 m = 0.5 * (v[a] + v[b]);
            double sc = 1.0 / std::sqrt(dot(m, m));
            v.push_back(sc * m);
            int id = (int)v.size() - 1;
            mid[key] = id;
            return id;
        };
        std::vector<int> g;
        g.reserve(f.size() * 4);
        for (size_t q = 0; q < f.size(); q += 3) {
            int a = f[q], b = f[q + 1], c = f[q + 2];
            int ab = midpoint(a, b), bc = midpoint(b, c), ca = midpoint(c, a);
            int add[12] = {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca};
            g.insert(g.end(), add, add + 12);
        }
        f.swap(g);
    }
    int nv = (int)v.size(), nt = (int)(f.size() / 3);
    *nv_out = nv;
    *nt_out = nt;
    if (nv > cap_verts || nt > cap_tris) return -1;
    for (int i = 0; i < nv; ++i) {
        verts[3 * i] = cx + radius * v[i].x;
        verts[3 * i + 1] = cy + radius * v[i].y;
        verts[3 * i + 2] = cz + radius * v[i].z;
    }
    for (int i = 0; i < nt; ++i) {
        V3 a = v[f[3 * i]], b = v[f[3 * i + 1]], c = v[f[3 * i + 2]];
        bool outward = dot(cross(b - a, c - a), a + b + c) > 0;
        tris[3 * i] = f[3 * i];
        tris[3 * i + 1] = outward ? f[3 * i + 1] : f[3 * i + 2];
        tris[3 * i + 2] = outward ? f[3 * i + 2] : f[3 * i + 1];
    }
    return 0;
}

// iblank(i,j,k) = 1 for cell centres enclosed by the closed surface, i,j,k in
// 1..n?-1; ghost layers stay 0.  Scan lines along x: a centre is inside when an
// odd number of surface crossings lie to its left.  Crossings are found with a
// half-open rule on the (y,z) projection so that a line through a shared edge
// or vertex is counted once.  Returns the number of solid cells.
long fsi_geom_iblank(int nx, int ny, int nz, const double *x, const double *y, const double *z,
                     int nv, const double *verts, int nt, const int32_t *tris, int8_t *iblank)
{
    (void)nv;
    std::vector<double> xc(nx + 1), yc(ny + 1), zc(nz + 1);
    for (int i = 0; i <= nx; ++i) xc[i] = 0.5 * (x[i] + x[i + 1]);
    for (int j = 0; j <= ny; ++j) yc[j] = 0.5 * (y[j] + y[j + 1]);
    for (int k = 0; k <= nz; ++k) zc[k] = 0.5 * (z[k] + z[k + 1]);
    size_t nf = (size_t)(nx + 2) * (size_t)(ny + 2) * (size_t)(nz + 2);
    std::memset(iblank, 0, nf);
    long nsolid = 0;
    std::vector<double> hits;
    for (int k = 1; k <= nz - 1; ++k)
        for (int j = 1; j <= ny - 1; ++j) {
            const double py = yc[j], pz = zc[k];
            hits.clear();
            for (int t = 0; t < nt; ++t) {
                const double *a = verts + 3 * tris[3 * t], *b = verts + 3 * tris[3 * t + 1],
                             *c = verts + 3 * tris[3 * t + 2];
                double ymin = std::min({a[1], b[1], c[1]}), ymax = std::max({a[1], b[1], c[1]});
                double zmin = std::min({a[2], b[2], c[2]}), zmax = std::max({a[2], b[2], c[2]});
                if (py < ymin || py > ymax || pz < zmin || pz > zmax) continue;
                // barycentric test in the (y,z) plane with a half-open edge rule
                auto edge = [&](const double *p, const double *q) {
                    return (q[1] - p[1]) * (pz - p[2]) - (q[2] - p[2]) * (py - p[1]);
                };
                double e0 = edge(a, b), e1 = edge(b, c), e2 = edge(c, a);
                auto owns = [](double e, const double *p, const double *q) {
                    if (e != 0.0) return e > 0.0;
                    // tie-break: edges whose direction points to +y, or to +z when flat in y
                    double dy = q[1] - p[1], dz = q[2] - p[2];
                    return dy > 0.0 || (dy == 0.0 && dz < 0.0);
                };
                bool pos = owns(e0, a, b) && owns(e1, b, c) && owns(e2, c, a);
                bool neg = owns(-e0, b, a) && owns(-e1, c, b) && owns(-e2, a, c);
                if (!pos && !neg) continue;
                double area = e0 + e1 + e2;
                if (area == 0.0) continue;
                double xh = (e1 * a[0] + e2 * b[0] + e0 * c[0]) / area;
                hits.push_back(xh);
            }
            if (hits.empty()) continue;
            std::sort(hits.begin(), hits.end());
            for (int i = 1; i <= nx - 1; ++i) {
                int left = (int)(std::lower_bound(hits.begin(), hits.end(), xc[i]) - hits.begin());
                if (left & 1) iblank[fidx(nx, ny, i, j, k)] = 1;
            }
        }
    // The clean-up passes set_internal_boundary runs on a solid body
    // (IBM/BOUNDARY_SET.F90:267-410), in its order.  find_isolatedIblank (:440-499):
    // a solid cell with no other solid cell in its 3x3x3 block (clipped to the
    // interior) turns fluid.  find_iblankHoles (:502-602) acts under SSM only.
    const int nxc = nx - 1, nyc = ny - 1, nzc = nz - 1;
    for (int k = 1; k <= nzc; ++k)
        for (int j = 1; j <= nyc; ++j)
            for (int i = 1; i <= nxc; ++i) {
                if (iblank[fidx(nx, ny, i, j, k)] != 1) continue;
                int solid = 0;
                for (int c = std::max(k - 1, 1); c <= std::min(k + 1, nzc); ++c)
                    for (int b = std::max(j - 1, 1); b <= std::min(j + 1, nyc); ++b)
                        for (int a = std::max(i - 1, 1); a <= std::min(i + 1, nxc); ++a)
                            solid += iblank[fidx(nx, ny, a, b, c)];
                if (solid <= 1) iblank[fidx(nx, ny, i, j, k)] = 0;
            }
    // fill_cell (IBM/SSM_SET_BC.F90:1425-1511): a fluid cell whose solid
    // neighbour faces it across a flagged face closes.  Under GCM the level-1
    // flags are set_outer_iup's (IBM/BOUNDARY_SET.F90:54-130): the low face of
    // the first cell and the high face of the last cell of every line.  One
    // pass per direction, x then y then z, updating in place.
    const int dims[3] = {nxc, nyc, nzc};
    for (int axis = 0; axis < 3; ++axis)
        for (int k = 1; k <= nzc; ++k)
            for (int j = 1; j <= nyc; ++j)
                for (int i = 1; i <= nxc; ++i) {
                    int8_t &cell = iblank[fidx(nx, ny, i, j, k)];
                    if (cell != 0) continue;
                    const int pos = axis == 0 ? i : axis == 1 ? j : k;
                    const int8_t lo = iblank[fidx(nx, ny, i - (axis == 0), j - (axis == 1), k - (axis == 2))];
                    const int8_t hi = iblank[fidx(nx, ny, i + (axis == 0), j + (axis == 1), k + (axis == 2))];
                    if ((lo == 1 && pos == dims[axis]) || (hi == 1 && pos == 1)) cell = 1;
                }
    for (size_t o = 0; o < nf; ++o) nsolid += iblank[o];
    return nsolid;
}

// Ghost marks: solid cells with a fluid 6-neighbour, neighbour indices clamped
// to the interior (IBM/GCM_SET_BOUNDARY.F90:49-73).  Writes ghostCellMark and the
// ordered list (k, j, i ascending, :106-118).  Returns nGhost, or -1 when the
// list capacity is too small.
int fsi_geom_ghost_list(int nx, int ny, int nz, const int8_t *iblank, int8_t *ghost,
                        int cap, int32_t *iG, int32_t *jG, int32_t *kG)
{
    size_t nf = (size_t)(nx + 2) * (size_t)(ny + 2) * (size_t)(nz + 2);
    std::memset(ghost, 0, nf);
    int count = 0;
    for (int k = 1; k <= nz - 1; ++k)
        for (int j = 1; j <= ny - 1; ++j)
            for (int i = 1; i <= nx - 1; ++i) {
                int iM = std::max(i - 1, 1), iP = std::min(i + 1, nx - 1);
                int jM = std::max(j - 1, 1), jP = std::min(j + 1, ny - 1);
                int kM = std::max(k - 1, 1), kP = std::min(k + 1, nz - 1);
                int b = iblank[fidx(nx, ny, i, j, k)];
                if (b * iblank[fidx(nx, ny, iM, j, k)] == 0 || b * iblank[fidx(nx, ny, iP, j, k)] == 0 ||
                    b * iblank[fidx(nx, ny, i, jM, k)] == 0 || b * iblank[fidx(nx, ny, i, jP, k)] == 0 ||
                    b * iblank[fidx(nx, ny, i, j, kM)] == 0 || b * iblank[fidx(nx, ny, i, j, kP)] == 0) {
                    if (b == 1) ghost[fidx(nx, ny, i, j, k)] = 1;
                }
            }
    for (int k = 1; k <= nz - 1; ++k)
        for (int j = 1; j <= ny - 1; ++j)
            for (int i = 1; i <= nx - 1; ++i)
                if (ghost[fidx(nx, ny, i, j, k)] == 1) {
                    if (count < cap) { iG[count] = i; jG[count] = j; kG[count] = k; }
                    ++count;
                }
    return count <= cap ? count : -1;
}

// Body intercept, image point, stencil cell and Neumann coefficients for each
// ghost (IBM/GCM_SET_BOUNDARY.F90:124-304, :307-494).  coeff is (8, nGhost)
// column-major like coeffGCMN; bi (3, nGhost) and ip (3, nGhost) are optional.
// Returns 0, or -(n+1) for the first ghost whose stencil search failed.
int fsi_geom_gcm_coeffs(int nx, int ny, int nz, const double *x, const double *y, const double *z,
                        int nv, const double *verts, int nt, const int32_t *tris,
                        double probeLengthNormalized, int nGhost,
                        const int32_t *iG, const int32_t *jG, const int32_t *kG,
                        int32_t *iCI, int32_t *jCI, int32_t *kCI, double *coeff,
                        double *probeLength, double *bi, double *ip, double *coeffD)
{
    static const int incI[8] = {0, 0, 1, 1, 0, 0, 1, 1};
    static const int incJ[8] = {0, 1, 1, 0, 0, 1, 1, 0};
    static const int incK[8] = {0, 0, 0, 0, 1, 1, 1, 1};
    std::vector<double> xc(nx + 2), yc(ny + 2), zc(nz + 2), dxv(nx + 1), dyv(ny + 1), dzv(nz + 1);
    for (int i = 0; i <= nx; ++i) { xc[i] = 0.5 * (x[i] + x[i + 1]); dxv[i] = x[i + 1] - x[i]; }
    for (int j = 0; j <= ny; ++j) { yc[j] = 0.5 * (y[j] + y[j + 1]); dyv[j] = y[j + 1] - y[j]; }
    for (int k = 0; k <= nz; ++k) { zc[k] = 0.5 * (z[k] + z[k + 1]); dzv[k] = z[k + 1] - z[k]; }
    xc[nx + 1] = x[nx + 1]; yc[ny + 1] = y[ny + 1]; zc[nz + 1] = z[nz + 1];
    const Surface surf = make_surface(nv, verts, nt, tris);
    for (int n = 0; n < nGhost; ++n) {
        int g_i = iG[n], g_j = jG[n], g_k = kG[n];
        V3 gc{xc[g_i], yc[g_j], zc[g_k]};
        V3 bip;
        int celem;
        body_intercept(surf, gc, bip, celem);
        double ds = std::sqrt(dot(bip - gc, bip - gc));
        V3 slope{(bip.x - gc.x) / ds, (bip.y - gc.y) / ds, (bip.z - gc.z) / ds};
        double pl = ds * probeLengthNormalized;
        V3 ipt = gc + pl * slope;
        probeLength[n] = pl;
        if (bi) { bi[3 * n] = bip.x; bi[3 * n + 1] = bip.y; bi[3 * n + 2] = bip.z; }
        if (ip) { ip[3 * n] = ipt.x; ip[3 * n + 1] = ipt.y; ip[3 * n + 2] = ipt.z; }
        auto nint = [](double v) { return (int)std::lround(v); };
        int iRange = nint(pl / dxv[g_i]) + 1, jRange = nint(pl / dyv[g_j]) + 1, kRange = nint(pl / dzv[g_k]) + 1;
        int ci = -1, cj = -1, ck = -1;
        for (int i = std::max(g_i - iRange, 0); i <= std::min(g_i + iRange, nx); ++i)
            if (xc[i] <= ipt.x && xc[i + 1] > ipt.x) ci = i;
        for (int j = std::max(g_j - jRange, 0); j <= std::min(g_j + jRange, ny); ++j)
            if (yc[j] <= ipt.y && yc[j + 1] > ipt.y) cj = j;
        for (int k = std::max(g_k - kRange, 0); k <= std::min(g_k + kRange, nz); ++k)
            if (zc[k] <= ipt.z && zc[k + 1] > ipt.z) ck = k;
        if (ci < 0 || cj < 0 || ck < 0) return -(n + 1);
        iCI[n] = ci; jCI[n] = cj; kCI[n] = ck;
        V3 bn = surf.nrm[celem];   // inward, as the reference's (the sign only scales the Neumann row)
        // The reference builds the Vandermonde matrix in absolute coordinates
        // (IBM/GCM_SET_BOUNDARY.F90:392-440), which loses about log10(1/h^3)
        // digits on fine cells, so the weights of a constant no longer sum to 1
        // and the all-Neumann operator stops being singular.  The same trilinear
        // interpolant is evaluated here in coordinates local to the stencil,
        // scaled by its cell sizes: identical weights, no cancellation.
        const double ox = xc[ci], oy = yc[cj], oz = zc[ck];
        const double sx = xc[ci + 1] - xc[ci], sy = yc[cj + 1] - yc[cj], sz = zc[ck + 1] - zc[ck];
        auto lx = [&](double v) { return (v - ox) / sx; };
        auto ly = [&](double v) { return (v - oy) / sy; };
        auto lz = [&](double v) { return (v - oz) / sz; };
        double V[64], VD[64];
        for (int r = 0; r < 8; ++r) {
            int i = ci + incI[r], j = cj + incJ[r], k = ck + incK[r];
            double x1 = lx(xc[i]), x2 = ly(yc[j]), x3 = lz(zc[k]);
            // Dirichlet matrix (GCM_Calc_VanMatrixDN, vanMatrixD): the ghost's
            // own row is the trilinear basis at the body intercept
            const bool self = (i == g_i && j == g_j && k == g_k);
            const double d1 = self ? lx(bip.x) : x1, d2 = self ? ly(bip.y) : x2, d3 = self ? lz(bip.z) : x3;
            VD[r + 8 * 0] = d1 * d2 * d3;
            VD[r + 8 * 1] = d1 * d2;
            VD[r + 8 * 2] = d1 * d3;
            VD[r + 8 * 3] = d2 * d3;
            VD[r + 8 * 4] = d1;
            VD[r + 8 * 5] = d2;
            VD[r + 8 * 6] = d3;
            VD[r + 8 * 7] = 1.0;
            if (self) {
                // Neumann row: n . grad in local coordinates (d/dx = (1/sx) d/dx'); its
                // right-hand side is uNormal = 0, so the row scale does not matter.
                double a1 = lx(bip.x), a2 = ly(bip.y), a3 = lz(bip.z);
                const V3 bn_l{bn.x / sx, bn.y / sy, bn.z / sz};
                V[r + 8 * 0] = bn_l.x * a2 * a3 + bn_l.y * a1 * a3 + bn_l.z * a1 * a2;
                V[r + 8 * 1] = bn_l.x * a2 + bn_l.y * a1;
                V[r + 8 * 2] = bn_l.x * a3 + bn_l.z * a1;
                V[r + 8 * 3] = bn_l.y * a3 + bn_l.z * a2;
                V[r + 8 * 4] = bn_l.x;
                V[r + 8 * 5] = bn_l.y;
                V[r + 8 * 6] = bn_l.z;
                V[r + 8 * 7] = 0.0;
            } else {
                V[r + 8 * 0] = x1 * x2 * x3;
                V[r + 8 * 1] = x1 * x2;
                V[r + 8 * 2] = x1 * x3;
                V[r + 8 * 3] = x2 * x3;
                V[r + 8 * 4] = x1;
                V[r + 8 * 5] = x2;
                V[r + 8 * 6] = x3;
                V[r + 8 * 7] = 1.0;
            }
        }
        if (!inv8(V)) return -(n + 1);
        const double px = lx(ipt.x), py = ly(ipt.y), pz = lz(ipt.z);
        double phi[8] = {px * py * pz, px * py, px * pz, py * pz, px, py, pz, 1.0};
        for (int r = 0; r < 8; ++r) {
            double s = 0.0;
            for (int m = 0; m < 8; ++m) s += V[m + 8 * r] * phi[m];
            coeff[8 * (size_t)n + r] = s;
        }
        if (coeffD) {
            if (!inv8(VD)) return -(n + 1);
            for (int r = 0; r < 8; ++r) {
                double s = 0.0;
                for (int m = 0; m < 8; ++m) s += VD[m + 8 * r] * phi[m];
                coeffD[8 * (size_t)n + r] = s;
            }
        }
    }
    return 0;
}

} // extern "C"
