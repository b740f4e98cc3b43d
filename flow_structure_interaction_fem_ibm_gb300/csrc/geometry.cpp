// Host-side immersed-boundary geometry: the input producer for the pressure
// solve.  In the reference this layer (set_boundary, IBM/BOUNDARY_SET.F90:8-51)
// stays on the host and feeds the solver iblank, the ghost-cell list and the
// image-point interpolation coefficients.  This file restates it in C++ for
// closed triangulated surfaces (UNSTRUCTURED_SURFACE bodies):
//   - icosphere surface generation (stands in for unstruc_surface_in.dat,
//     IBM/BOUNDARY_MARKER_INIT.F90:209-247),
//   - iblank by directional (scan-line) fill of cell centres enclosed by the
//     surface (the fill step of IBM/BOUNDARY_IBLANK_FAST.F90:2-501),
//   - ghost marks and the ordered ghost list (IBM/GCM_SET_BOUNDARY.F90:49-118),
//   - body intercept = closest surface point among the elements that share the
//     three closest markers (IBM/GCM_INTERCEPT_KERNELS_UNSTRUC.F90:26-398),
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

// Closest point on triangle abc to p (Ericson, Real-Time Collision Detection, 5.1.5).
V3 closest_on_tri(V3 p, V3 a, V3 b, V3 c)
{
    V3 ab = b - a, ac = c - a, ap = p - a;
    double d1 = dot(ab, ap), d2 = dot(ac, ap);
    if (d1 <= 0 && d2 <= 0) return a;
    V3 bp = p - b;
    double d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= 0 && d4 <= d3) return b;
    double vc = d1 * d4 - d3 * d2;
    if (vc <= 0 && d1 >= 0 && d3 <= 0) { double v = d1 / (d1 - d3); return a + v * ab; }
    V3 cp = p - c;
    double d5 = dot(ab, cp), d6 = dot(ac, cp);
    if (d6 >= 0 && d5 <= d6) return c;
    double vb = d5 * d2 - d1 * d6;
    if (vb <= 0 && d2 >= 0 && d6 <= 0) { double w = d2 / (d2 - d6); return a + w * ac; }
    double va = d3 * d6 - d5 * d4;
    if (va <= 0 && (d4 - d3) >= 0 && (d5 - d6) >= 0) {
        double w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        return b + w * (c - b);
    }
    double denom = 1.0 / (va + vb + vc);
    double v = vb * denom, w = vc * denom;
    return a + v * ab + w * ac;
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
                if (left & 1) { iblank[fidx(nx, ny, i, j, k)] = 1; ++nsolid; }
            }
        }
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
    // vertex -> elements adjacency and element normals
    std::vector<std::vector<int>> vtri(nv);
    std::vector<V3> nrm(nt);
    for (int t = 0; t < nt; ++t) {
        for (int q = 0; q < 3; ++q) vtri[tris[3 * t + q]].push_back(t);
        const double *a = verts + 3 * tris[3 * t], *b = verts + 3 * tris[3 * t + 1], *c = verts + 3 * tris[3 * t + 2];
        V3 n = cross(V3{b[0] - a[0], b[1] - a[1], b[2] - a[2]}, V3{c[0] - a[0], c[1] - a[1], c[2] - a[2]});
        double s = 1.0 / std::sqrt(dot(n, n));
        nrm[t] = s * n;
    }
    for (int n = 0; n < nGhost; ++n) {
        int g_i = iG[n], g_j = jG[n], g_k = kG[n];
        V3 gc{xc[g_i], yc[g_j], zc[g_k]};
        // three closest markers
        int best[3] = {-1, -1, -1};
        double bd[3] = {1e300, 1e300, 1e300};
        for (int m = 0; m < nv; ++m) {
            V3 pm{verts[3 * m], verts[3 * m + 1], verts[3 * m + 2]};
            double d = dot(pm - gc, pm - gc);
            for (int q = 0; q < 3; ++q)
                if (d < bd[q]) {
                    for (int r = 2; r > q; --r) { bd[r] = bd[r - 1]; best[r] = best[r - 1]; }
                    bd[q] = d; best[q] = m;
                    break;
                }
        }
        double dmin = 1e300;
        int celem = -1;
        V3 bip{0, 0, 0};
        for (int q = 0; q < 3; ++q) {
            if (best[q] < 0) continue;
            for (int t : vtri[best[q]]) {
                const double *a = verts + 3 * tris[3 * t], *b = verts + 3 * tris[3 * t + 1],
                             *c = verts + 3 * tris[3 * t + 2];
                V3 cp = closest_on_tri(gc, V3{a[0], a[1], a[2]}, V3{b[0], b[1], b[2]}, V3{c[0], c[1], c[2]});
                double d = dot(cp - gc, cp - gc);
                if (d < dmin) { dmin = d; celem = t; bip = cp; }
            }
        }
        double ds = std::sqrt(dot(bip - gc, bip - gc));
        V3 slope = (1.0 / ds) * (bip - gc);
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
        V3 bn = nrm[celem];
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
