// Host-side immersed-boundary geometry: the input producer for the pressure
// solve.  In the reference this layer (set_boundary, IBM/BOUNDARY_SET.F90:8-51)
// stays on the host and feeds the solver iblank, the ghost-cell list and the
// image-point interpolation coefficients.  This file restates it in C++ for
// closed triangulated surfaces (UNSTRUCTURED_SURFACE bodies):
//   - icosphere surface generation (stands in for unstruc_surface_in.dat,
//     IBM/BOUNDARY_MARKER_INIT.F90:209-247),
//   - iblank by the reference's band and dot-normal classification and fill
//     (IBM/BOUNDARY_IBLANK_FAST.F90:2-1024; the band cells spread over the host
//     threads), then its clean-up passes for a solid body
//     (IBM/BOUNDARY_SET.F90:267-410),
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
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <thread>
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
    std::vector<V3> cen;                  // centroids
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
    s.cen.resize(nt);
    s.vtri.assign(nv, {});
    for (int t = 0; t < nt; ++t) {
        V3 p1 = s.p(s.node(t, 0)), p2 = s.p(s.node(t, 1)), p3 = s.p(s.node(t, 2));
        V3 a = p2 - p1, b = p3 - p2;
        V3 n{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
        double mag = std::sqrt(n.x * n.x + n.y * n.y + n.z * n.z);
        s.nrm[t] = V3{n.x / mag, n.y / mag, n.z / mag};
        s.cen[t] = V3{(p1.x + p2.x + p3.x) / 3.0, (p1.y + p2.y + p3.y) / 3.0, (p1.z + p2.z + p3.z) / 3.0};
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

// The k markers nearest p in (squared distance, index) order: the order of
// repeated MINLOC with each found marker set aside.
void nearest_markers(const Surface &s, V3 p, int k, int *out)
{
    double bd[8];
    for (int r = 0; r < k; ++r) { bd[r] = 1e300; out[r] = -1; }
    for (int m = 0; m < s.nv; ++m) {
        V3 q = s.p(m);
        double dx = q.x - p.x, dy = q.y - p.y, dz = q.z - p.z;
        double d = dx * dx + dy * dy + dz * dz;
        for (int r = 0; r < k; ++r)
            if (d < bd[r]) {
                for (int u = k - 1; u > r; --u) { bd[u] = bd[u - 1]; out[u] = out[u - 1]; }
                bd[r] = d; out[r] = m;
                break;
            }
    }
}

// Signed distance of p from the plane (n, ref) as get_distance_face takes it
// (IBM/BOUNDARY_IBLANK_FAST.F90:3535-3555): |p - ref| cos(angle(n, p - ref)).
double plane_distance(V3 n, V3 ref, V3 p)
{
    if (p.x == ref.x && p.y == ref.y && p.z == ref.z) return 0.0;
    V3 v = p - ref;
    double len = 0.0;
    len = len + v.x * v.x; len = len + v.y * v.y; len = len + v.z * v.z;
    return std::sqrt(len) * std::cos(vec_angle(n, v));
}

// Whether the segment from p1 to p2 passes through element e: the segment's
// crossing of the element's plane (get_inter, :3513-3533, an end within 1e-10
// of the plane taken as is) lies inside the triangle by pointInTriangle's
// test (:3862-3910): the three (edge x (point - vertex)) vectors, each scaled
// by the first one's length, agree in direction within pi/10.
bool segment_crosses(const Surface &s, int e, V3 p1, V3 p2)
{
    const V3 n = s.nrm[e], ref = s.cen[e];
    double l1 = n.x * (p1.x - ref.x) + n.y * (p1.y - ref.y) + n.z * (p1.z - ref.z);
    double l2 = n.x * (p2.x - ref.x) + n.y * (p2.y - ref.y) + n.z * (p2.z - ref.z);
    V3 q;
    if (std::fabs(l1) < 1e-10) q = p1;
    else if (std::fabs(l2) < 1e-10) q = p2;
    else {
        double t = l1 / (l1 - l2);
        q = V3{p1.x + t * (p2.x - p1.x), p1.y + t * (p2.y - p1.y), p1.z + t * (p2.z - p1.z)};
    }
    const V3 a = s.p(s.node(e, 0)), b = s.p(s.node(e, 1)), c = s.p(s.node(e, 2));
    V3 c1 = cross(b - a, q - a), c2 = cross(c - b, q - b), c3 = cross(a - c, q - c);
    auto len = [](V3 v) { double t = 0.0; t = t + v.x * v.x; t = t + v.y * v.y; t = t + v.z * v.z; return std::sqrt(t); };
    double m1 = len(c1), m2 = len(c2), m3 = len(c3);
    if (m1 < 1e-20 || m2 < 1e-20 || m3 < 1e-20) return false;
    c1 = V3{c1.x / m1, c1.y / m1, c1.z / m1};
    c2 = V3{c2.x / m1, c2.y / m1, c2.z / m1};
    c3 = V3{c3.x / m1, c3.y / m1, c3.z / m1};
    const double lim = 4.0 * std::atan(1.0) / 10.0;
    return vec_angle(c1, c2) < lim && vec_angle(c2, c3) < lim;
}

// search_vertex_dotNorm (IBM/BOUNDARY_IBLANK_FAST.F90:504-1024) for the cell
// centre p: true when p is solid (dot product >= 0 with the inward normal of
// the chosen element).  The reference marker is the first of the seven
// nearest markers whose segment to p crosses none of the elements around the
// seven that do not contain it; a marker whose elements' normals are at least
// pi/2 apart (check_if_edge_marker, :3580-3703) makes p fluid; otherwise the
// element is, among the marker's elements, the nearest plane whose normal
// projection passes the area test, or before the first such element the
// smallest angle between (p - marker) and the outward normal (last of equals).
// Returns -1 when no reference marker exists (the reference stops there).
int dot_normal_solid(const Surface &s, V3 p, std::vector<int> &around)
{
    int near[7];
    nearest_markers(s, p, 7, near);
    around.clear();
    for (int q = 0; q < 7; ++q)
        if (near[q] >= 0) around.insert(around.end(), s.vtri[near[q]].begin(), s.vtri[near[q]].end());
    std::sort(around.begin(), around.end());
    around.erase(std::unique(around.begin(), around.end()), around.end());
    int ref = -1;
    for (int q = 0; q < 7 && ref < 0; ++q) {
        if (near[q] < 0) break;
        const int mk = near[q];
        const V3 pm = s.p(mk);
        bool blocked = false;
        for (int e : around) {
            if (s.node(e, 0) == mk || s.node(e, 1) == mk || s.node(e, 2) == mk) continue;
            double dc = plane_distance(s.nrm[e], s.cen[e], p), dm = plane_distance(s.nrm[e], s.cen[e], pm);
            if (dc * dm > 0.0) continue;
            if (segment_crosses(s, e, p, pm)) { blocked = true; break; }
        }
        if (!blocked) ref = mk;
    }
    if (ref < 0) return -1;
    const std::vector<int> &own = s.vtri[ref];
    if (own.size() < 2) return -1;
    const double half_pi = 4.0 * std::atan(1.0) / 2.0;
    for (size_t a = 0; a + 1 < own.size(); ++a)
        for (size_t b = a + 1; b < own.size(); ++b)
            if (vec_angle(-1.0 * s.nrm[own[a]], -1.0 * s.nrm[own[b]]) >= half_pi) return 0;
    double distIn = 1.0e16, angMin = 1.0e16;
    bool inside = false;
    int ce = -1;
    for (int e : own) {
        V3 bi;
        const V3 n = s.nrm[e];
        if (project_inside(s, e, p, bi)) {
            inside = true;
            const V3 p1 = s.p(s.node(e, 0));
            double plane = -n.x * p1.x - n.y * p1.y - n.z * p1.z;
            double d = std::fabs(-(n.x * p.x + n.y * p.y + n.z * p.z + plane));
            if (d <= distIn) { distIn = d; ce = e; }
        } else if (!inside) {
            double ang = vec_angle(p - s.p(ref), -1.0 * n);
            if (ang <= angMin) { angMin = ang; ce = e; }
        }
    }
    if (ce < 0) return -1;
    const V3 c = s.cen[ce], n = s.nrm[ce];
    double dn = (p.x - c.x) * n.x + (p.y - c.y) * n.y + (p.z - c.z) * n.z;
    return dn >= 0.0 ? 1 : 0;
}

// Body intercept of the point p (GCM_calc_bodyIntercept_Unstruc,
// IBM/GCM_INTERCEPT_KERNELS_UNSTRUC.F90:26-398).  For each of the three
// closest markers: the first of its elements (ascending) whose normal
// projection passes the inside test gives the intercept; failing that, the
// element whose outward normal makes the smallest angle with (p - marker)
// (last of equals) is taken and the intercept is the nearer foot on its two
// edges that leave the marker, clamped to the marker.  Of the three
// candidates the nearest (first of equals) wins.  False when the surface has
// fewer than three markers or one of the three belongs to no element.
bool body_intercept(const Surface &s, V3 p, V3 &bi, int &elem)
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
        if (mk < 0) return false;   // fewer than three markers
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
        if (ce < 0) return false;
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
    return true;
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
static int icosphere_impl(int nsub, double radius, double cx, double cy, double cz,
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

// iblank(i,j,k) = 1 for solid cells, i,j,k in 1..n?-1 (ghost layers stay 0), by
// the reference's set_iblank_canonical_body_fast (IBM/BOUNDARY_IBLANK_FAST.F90:
// 2-501): the cells whose centres bracket an element's bounding box form a band
// classified one by one by the dot-normal test; every other cell takes the value
// of the nearest band cell before it along k (or the first one after it when
// none precedes; a line without band cells is fluid) -- the reference's i and j
// fills are overwritten by its k fill.  Returns the number of solid cells, or -1
// when the dot-normal test finds no reference marker for a band cell.
static long iblank_impl(int nx, int ny, int nz, const double *x, const double *y, const double *z,
                        int nv, const double *verts, int nt, const int32_t *tris, int8_t *iblank)
{
    std::vector<double> xc(nx + 2), yc(ny + 2), zc(nz + 2);
    for (int i = 0; i <= nx; ++i) xc[i] = 0.5 * (x[i] + x[i + 1]);
    for (int j = 0; j <= ny; ++j) yc[j] = 0.5 * (y[j] + y[j + 1]);
    for (int k = 0; k <= nz; ++k) zc[k] = 0.5 * (z[k] + z[k + 1]);
    const size_t nf = (size_t)(nx + 2) * (size_t)(ny + 2) * (size_t)(nz + 2);
    std::memset(iblank, 0, nf);
    std::vector<int8_t> band(nf, 0);
    const Surface surf = make_surface(nv, verts, nt, tris);
    const int n_[3] = {nx, ny, nz};
    const double *lo_node[3] = {x, y, z};
    const std::vector<double> *cc[3] = {&xc, &yc, &zc};
    for (int t = 0; t < nt; ++t) {
        const V3 v[3] = {surf.p(surf.node(t, 0)), surf.p(surf.node(t, 1)), surf.p(surf.node(t, 2))};
        auto comp = [](V3 a, int d) { return d == 0 ? a.x : d == 1 ? a.y : a.z; };
        bool outside = false;
        int lo[3], hi[3];
        for (int d = 0; d < 3 && !outside; ++d) {
            const double a = comp(v[0], d), b = comp(v[1], d), c = comp(v[2], d);
            const double first = lo_node[d][1], last = lo_node[d][n_[d]];
            if ((a <= first && b <= first && c <= first) || (a >= last && b >= last && c >= last)) outside = true;
            const double bmin = std::min({a, b, c}), bmax = std::max({a, b, c});
            int cmin = 0, cmax = 0;
            const std::vector<double> &w = *cc[d];
            for (int i = 0; i < n_[d]; ++i) {
                if ((w[i] - bmin) * (w[i + 1] - bmin) <= 0.0) cmin = i;
                if ((w[i] - bmax) * (w[i + 1] - bmax) <= 0.0) cmax = i + 1;
            }
            lo[d] = cmin == 0 ? 1 : cmin;
            hi[d] = (cmax == 0 || cmax == n_[d]) ? n_[d] - 1 : cmax;
        }
        if (outside) continue;
        for (int k = lo[2]; k <= hi[2]; ++k)
            for (int j = lo[1]; j <= hi[1]; ++j)
                for (int i = lo[0]; i <= hi[0]; ++i) band[fidx(nx, ny, i, j, k)] = 1;
    }
    // the band cells are independent: split them over the host threads
    std::vector<size_t> cells;
    for (int k = 1; k <= nz - 1; ++k)
        for (int j = 1; j <= ny - 1; ++j)
            for (int i = 1; i <= nx - 1; ++i)
                if (band[fidx(nx, ny, i, j, k)]) cells.push_back(fidx(nx, ny, i, j, k));
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const size_t nthreads = std::min<size_t>(std::min(hw, 64u), std::max<size_t>(1, cells.size() / 2048));
    const size_t chunk = 256;
    std::atomic<size_t> next(0);
    std::atomic<bool> failed(false);
    auto work = [&]() {   // chunks taken from a shared counter: any number of workers covers every cell
        std::vector<int> around;
        around.reserve(64);
        for (size_t q0 = next.fetch_add(chunk); q0 < cells.size() && !failed.load(); q0 = next.fetch_add(chunk))
            for (size_t q = q0; q < std::min(q0 + chunk, cells.size()); ++q) {
                const size_t o = cells[q];
                const int i = (int)(o % (size_t)(nx + 2)), j = (int)((o / (size_t)(nx + 2)) % (size_t)(ny + 2));
                const int k = (int)(o / ((size_t)(nx + 2) * (size_t)(ny + 2)));
                int solid = dot_normal_solid(surf, V3{xc[i], yc[j], zc[k]}, around);
                if (solid < 0) failed = true;
                else iblank[o] = (int8_t)solid;
            }
    };
    std::vector<std::thread> pool;
    for (size_t t = 1; t < nthreads; ++t) {
        try { pool.emplace_back(work); } catch (...) { break; }   // fewer workers if a thread cannot start
    }
    work();
    for (auto &th : pool) th.join();
    if (failed) return -1;
    // the k fill: seed from the first band cell of the line, carry upward
    for (int j = 1; j <= ny - 1; ++j)
        for (int i = 1; i <= nx - 1; ++i) {
            int8_t carry = 0;
            for (int k = 1; k <= nz; ++k)
                if (band[fidx(nx, ny, i, j, k)]) { carry = iblank[fidx(nx, ny, i, j, k)]; break; }
            for (int k = 1; k <= nz - 1; ++k) {
                const size_t o = fidx(nx, ny, i, j, k);
                if (band[o]) carry = iblank[o];
                else iblank[o] = carry;
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
    long nsolid = 0;
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
static int gcm_coeffs_impl(int nx, int ny, int nz, const double *x, const double *y, const double *z,
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
        if (!body_intercept(surf, gc, bip, celem)) return -(n + 1);
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

// The exported entry points: no C++ exception crosses the C boundary (an
// allocation failure returns -2; the first two keep their documented codes
// otherwise).
int fsi_geom_icosphere(int nsub, double radius, double cx, double cy, double cz,
                       double *verts, int cap_verts, int32_t *tris, int cap_tris,
                       int *nv_out, int *nt_out)
{
    try { return icosphere_impl(nsub, radius, cx, cy, cz, verts, cap_verts, tris, cap_tris, nv_out, nt_out); }
    catch (...) { return -2; }
}

long fsi_geom_iblank(int nx, int ny, int nz, const double *x, const double *y, const double *z,
                     int nv, const double *verts, int nt, const int32_t *tris, int8_t *iblank)
{
    try { return iblank_impl(nx, ny, nz, x, y, z, nv, verts, nt, tris, iblank); }
    catch (...) { return -2; }
}

int fsi_geom_gcm_coeffs(int nx, int ny, int nz, const double *x, const double *y, const double *z,
                        int nv, const double *verts, int nt, const int32_t *tris,
                        double probeLengthNormalized, int nGhost,
                        const int32_t *iG, const int32_t *jG, const int32_t *kG,
                        int32_t *iCI, int32_t *jCI, int32_t *kCI, double *coeff,
                        double *probeLength, double *bi, double *ip, double *coeffD)
{
    try {
        return gcm_coeffs_impl(nx, ny, nz, x, y, z, nv, verts, nt, tris, probeLengthNormalized, nGhost, iG, jG, kG,
                               iCI, jCI, kCI, coeff, probeLength, bi, ip, coeffD);
    } catch (...) { return -(nGhost + 2); }
}

} // extern "C"
