/*
 * Oracle (TEST INFRASTRUCTURE ONLY): plain-C restatement, in the reference's
 * loop order and with its selection rules, of the host geometry that feeds the
 * pressure solve for one solid unstructured body in 3D:
 *
 *   og_orient_inward   determine_norm_dir_unstruc
 *                      (IBM/BOUNDARY_SET_ARCLENGTH_NORM.F90:200-320): the
 *                      reference's normals point INTO the body; every
 *                      triangle's nodes 2 and 3 are swapped when the element
 *                      at the marker nearest an outside point faces out.
 *   og_iblank          set_iblank_canonical_body_fast
 *                      (IBM/BOUNDARY_IBLANK_FAST.F90:2-501): a band of cells
 *                      around every element's bounding box is classified by
 *                      search_vertex_dotNorm (:504-1024), the other cells are
 *                      filled along i, then j, then k from the first decided
 *                      cell of each line; then the clean-up passes of
 *                      set_internal_boundary for a solid body
 *                      (IBM/BOUNDARY_SET.F90:267-410).
 *   og_ghost_list      GCM_set_internal_boundary (IBM/GCM_SET_BOUNDARY.F90:
 *                      22-118): ghost marks and their (k, j, i) order.
 *   og_gcm             the rest of GCM_set_internal_boundary (:119-304):
 *                      body intercept by GCM_calc_bodyIntercept_Unstruc
 *                      (IBM/GCM_INTERCEPT_KERNELS_UNSTRUC.F90:26-398), image
 *                      point, stencil search, GCM_Calc_VanMatrixDN
 *                      (IBM/GCM_SET_BOUNDARY.F90:307-494) in global
 *                      coordinates.  The reference inverts the two 8 x 8
 *                      matrices with LAPACK DGETRF/DGETRI; here LU with
 *                      partial pivoting and one solve per unit vector (the
 *                      same inverse up to rounding).
 *
 * Element normals and centroids follow calculate_arclength_norm_ds
 * (IBM/BOUNDARY_SET_ARCLENGTH_NORM.F90:69-165); vector_angle and mo follow
 * the reference's operation module (IBM/AMODULES.F90:905-988).
 *
 * Conventions: markers and elements are 0-based (the reference counts from
 * 1); MINLOC ties resolve to the lowest index as in Fortran.  Fields are
 * Fortran column-major (0:nx+1, 0:ny+1, 0:nz+1); nx, ny, nz are node counts
 * and cells run 1..n-1.  Built with -ffp-contract=off.
 *
 * Only the tests use this library, as the checker of the product geometry
 * (flow_structure_interaction_fem_ibm_gb300/csrc/geometry.cpp).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define OG_NSAVE 7      /* closest markers kept by search_vertex_dotNorm */
#define OG_NCHECK 3     /* closest markers tried by GCM_calc_bodyIntercept_Unstruc */

typedef struct {
    int nv, nt;
    const double *v;        /* (3, nv) marker coordinates */
    const int32_t *t;       /* (3, nt) element nodes */
    double *nrm;            /* (3, nt) unit normals (into the body) */
    double *cen;            /* (3, nt) centroids */
    double *area;           /* nt */
} surf_t;

static double og_pi(void) { return 4.0 * atan(1.0); }

static void cross3(const double *a, const double *b, double *c)
{
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

static double dot3(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

/* mo(a,3): running sum of squares from zero, then the square root */
static double mo3(const double *a)
{
    double s = 0.0;
    for (int i = 0; i < 3; ++i) s = s + a[i] * a[i];
    return sqrt(s);
}

/* vector_angle (IBM/AMODULES.F90:968-988): acos of the cosine, 0 or pi when
 * the cosine leaves (-1, 1).  The reference's second branch tests the sine
 * magnitude for a negative value, which a magnitude never has. */
static double vector_angle(const double *a, const double *b)
{
    double c = dot3(a, b) / (mo3(a) * mo3(b));
    if (c < 1.0 && c > -1.0) return acos(c);
    if (c > 0.0) return 0.0;
    if (c < 0.0) return og_pi();
    return NAN;
}

static const double *vtx(const surf_t *s, int m) { return s->v + 3 * (size_t)m; }
static int node(const surf_t *s, int e, int q) { return s->t[3 * (size_t)e + q]; }

/* calculate_arclength_norm_ds: n = (p2 - p1) x (p3 - p2) / |.|, centroid = (p1 + p2 + p3) / 3 */
static void surf_metrics(surf_t *s)
{
    for (int m = 0; m < s->nt; ++m) {
        const double *p1 = vtx(s, node(s, m, 0)), *p2 = vtx(s, node(s, m, 1)), *p3 = vtx(s, node(s, m, 2));
        double a[3] = {p2[0] - p1[0], p2[1] - p1[1], p2[2] - p1[2]};
        double b[3] = {p3[0] - p2[0], p3[1] - p2[1], p3[2] - p2[2]};
        double n[3];
        n[0] = a[1] * b[2] - a[2] * b[1];
        n[1] = a[2] * b[0] - a[0] * b[2];
        n[2] = a[0] * b[1] - a[1] * b[0];
        double mag = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        s->area[m] = 0.5 * mag;
        for (int q = 0; q < 3; ++q) {
            s->nrm[3 * (size_t)m + q] = n[q] / mag;
            s->cen[3 * (size_t)m + q] = (p1[q] + p2[q] + p3[q]) / 3.0;
        }
    }
}

static int surf_open(surf_t *s, int nv, const double *verts, int nt, const int32_t *tris)
{
    s->nv = nv; s->nt = nt; s->v = verts; s->t = tris;
    s->nrm = malloc(sizeof(double) * 3 * (size_t)nt);
    s->cen = malloc(sizeof(double) * 3 * (size_t)nt);
    s->area = malloc(sizeof(double) * (size_t)nt);
    if (!s->nrm || !s->cen || !s->area) return -1;
    surf_metrics(s);
    return 0;
}

static void surf_close(surf_t *s) { free(s->nrm); free(s->cen); free(s->area); }

/* the k closest markers by repeated MINLOC over squared distances, each found
 * marker then set to 1e20 */
static void closest_markers(const surf_t *s, const double *p, int k, int *out, double *scratch)
{
    for (int m = 0; m < s->nv; ++m) {
        const double *q = vtx(s, m);
        double dx = q[0] - p[0], dy = q[1] - p[1], dz = q[2] - p[2];
        scratch[m] = dx * dx + dy * dy + dz * dz;
    }
    for (int c = 0; c < k; ++c) {
        int best = 0;
        for (int m = 1; m < s->nv; ++m)
            if (scratch[m] < scratch[best]) best = m;
        out[c] = best;
        scratch[best] = 1.0e20;
    }
}

static int touches(const surf_t *s, int e, const int *mk, int nmk)
{
    for (int q = 0; q < 3; ++q)
        for (int c = 0; c < nmk; ++c)
            if (node(s, e, q) == mk[c]) return 1;
    return 0;
}

/* check_BIInsideTriangle (IBM/BOUNDARY_IBLANK_FAST.F90:1028-1159): normal
 * projection onto the element's plane and Heron's area test */
static void bi_inside(const surf_t *s, int e, const double *p, double *bi, double *area123,
                      double *areaDiff, double *distInside)
{
    const double *n = s->nrm + 3 * (size_t)e;
    const double *p1 = vtx(s, node(s, e, 0)), *p2 = vtx(s, node(s, e, 1)), *p3 = vtx(s, node(s, e, 2));
    double planeConst = -n[0] * p1[0] - n[1] * p1[1] - n[2] * p1[2];
    double d = -(n[0] * p[0] + n[1] * p[1] + n[2] * p[2] + planeConst);
    *distInside = fabs(d);
    for (int q = 0; q < 3; ++q) bi[q] = p[q] + n[q] * d;
#define OG_LEN(a, b) sqrt(((a)[0] - (b)[0]) * ((a)[0] - (b)[0]) + ((a)[1] - (b)[1]) * ((a)[1] - (b)[1]) + \
                          ((a)[2] - (b)[2]) * ((a)[2] - (b)[2]))
    double s12 = OG_LEN(p2, p1), s23 = OG_LEN(p3, p2), s31 = OG_LEN(p1, p3);
    double s14 = OG_LEN(bi, p1), s24 = OG_LEN(bi, p2), s34 = OG_LEN(bi, p3);
#undef OG_LEN
    double h123 = 0.5 * (s12 + s23 + s31), h124 = 0.5 * (s12 + s24 + s14);
    double h234 = 0.5 * (s23 + s24 + s34), h314 = 0.5 * (s31 + s34 + s14);
    double a123 = sqrt(h123 * (h123 - s12) * (h123 - s23) * (h123 - s31));
    double a124 = sqrt(h124 * (h124 - s12) * (h124 - s24) * (h124 - s14));
    double a234 = sqrt(h234 * (h234 - s23) * (h234 - s24) * (h234 - s34));
    double a314 = sqrt(h314 * (h314 - s31) * (h314 - s34) * (h314 - s14));
    *area123 = a123;
    *areaDiff = a124 + a234 + a314 - a123;
}

/* calc_BIOutsideTriangle (:1163-1435): the angle between (point - closest
 * marker) and the element's outward normal */
static double bi_outside(const surf_t *s, int e, const double *p, int cmarker)
{
    const double *c = vtx(s, cmarker);
    double vm[3] = {p[0] - c[0], p[1] - c[1], p[2] - c[2]};
    const double *n = s->nrm + 3 * (size_t)e;
    double out[3] = {-n[0], -n[1], -n[2]};
    return vector_angle(vm, out);
}

/* get_distance_face (:3535-3555): |p - ref| cos(angle(n, p - ref)) */
static double distance_face(const double *n, const double *ref, const double *p)
{
    if (p[0] == ref[0] && p[1] == ref[1] && p[2] == ref[2]) return 0.0;
    double v[3] = {p[0] - ref[0], p[1] - ref[1], p[2] - ref[2]};
    return mo3(v) * cos(vector_angle(n, v));
}

/* get_inter (:3513-3533): where the segment p1-p2 meets the plane (n, ref);
 * an end within 1e-10 of the plane is returned as is.  The reference expands
 * the parametric intersection into one rational expression per component; the
 * parametric form is used here. */
static void plane_inter(const double *n, const double *ref, const double *p1, const double *p2, double *out)
{
    double l1 = n[0] * (p1[0] - ref[0]) + n[1] * (p1[1] - ref[1]) + n[2] * (p1[2] - ref[2]);
    double l2 = n[0] * (p2[0] - ref[0]) + n[1] * (p2[1] - ref[1]) + n[2] * (p2[2] - ref[2]);
    if (fabs(l1) < 1e-10) { memcpy(out, p1, 3 * sizeof(double)); return; }
    if (fabs(l2) < 1e-10) { memcpy(out, p2, 3 * sizeof(double)); return; }
    double t = l1 / (l1 - l2);
    for (int q = 0; q < 3; ++q) out[q] = p1[q] + t * (p2[q] - p1[q]);
}

/* pointInTriangle (:3862-3910): the three edge x (point - vertex) vectors
 * (each scaled by the first one's length, as the reference does) agree in
 * direction to within pi/10 */
static int point_in_triangle(const double *n1, const double *n2, const double *n3, const double *p)
{
    double e1[3] = {n2[0] - n1[0], n2[1] - n1[1], n2[2] - n1[2]};
    double e2[3] = {n3[0] - n2[0], n3[1] - n2[1], n3[2] - n2[2]};
    double e3[3] = {n1[0] - n3[0], n1[1] - n3[1], n1[2] - n3[2]};
    double r1[3] = {p[0] - n1[0], p[1] - n1[1], p[2] - n1[2]};
    double r2[3] = {p[0] - n2[0], p[1] - n2[1], p[2] - n2[2]};
    double r3[3] = {p[0] - n3[0], p[1] - n3[1], p[2] - n3[2]};
    double c1[3], c2[3], c3[3];
    cross3(e1, r1, c1); cross3(e2, r2, c2); cross3(e3, r3, c3);
    double m1 = mo3(c1), m2 = mo3(c2), m3 = mo3(c3);
    if (m1 < 1e-20 || m2 < 1e-20 || m3 < 1e-20) return 0;
    for (int q = 0; q < 3; ++q) { c1[q] /= m1; c2[q] /= m1; c3[q] /= m1; }
    double lim = og_pi() / 10.0;
    return vector_angle(c1, c2) < lim && vector_angle(c2, c3) < lim;
}

/* check_if_edge_marker (:3580-3703): some pair of the marker's elements has
 * normals at least pi/2 apart.  Returns -1 when the marker has fewer than two
 * elements (the reference leaves its flag unset then). */
static int edge_marker(const surf_t *s, int mk, int *elems, int cap)
{
    int ne = 0;
    for (int m = 0; m < s->nt; ++m)
        if (node(s, m, 0) == mk || node(s, m, 1) == mk || node(s, m, 2) == mk) {
            if (ne < cap) elems[ne] = m;
            ++ne;
        }
    if (ne > cap || ne < 2) return -1;
    double half_pi = og_pi() / 2.0;
    for (int a = 0; a < ne - 1; ++a)
        for (int b = a + 1; b < ne; ++b) {
            const double *na = s->nrm + 3 * (size_t)elems[a], *nb = s->nrm + 3 * (size_t)elems[b];
            double ra[3] = {-na[0], -na[1], -na[2]}, rb[3] = {-nb[0], -nb[1], -nb[2]};
            if (vector_angle(ra, rb) >= half_pi) return 1;
        }
    return 0;
}

#define OG_NSIZE 1000   /* neighbour-element capacity of the reference */

/* search_vertex_dotNorm (:504-1024) for one cell centre p: returns 0 and the
 * dot product of (p - centroid) with the chosen element's inward normal, or -1
 * when no reference marker is found (the reference stops) or a list
 * overflows. */
static int search_vertex_dotnorm(const surf_t *s, const double *p, double *scratch, int *nbr, double *dotNorm,
                                 int *elemOut)
{
    int cv[OG_NSAVE];
    closest_markers(s, p, OG_NSAVE, cv, scratch);
    int nn = 0;
    for (int m = 0; m < s->nt; ++m)
        if (touches(s, m, cv, OG_NSAVE)) {
            if (nn >= OG_NSIZE) return -1;
            nbr[nn++] = m;
        }
    /* the reference marker: the first of the closest markers whose segment to
     * the cell crosses none of the neighbour elements that do not contain it */
    int choice = -1;
    for (int i = 0; i < OG_NSAVE && choice < 0; ++i) {
        const double *pm = vtx(s, cv[i]);
        int crossed = 0;
        for (int q = 0; q < nn && !crossed; ++q) {
            int e = nbr[q];
            int a = node(s, e, 0), b = node(s, e, 1), c = node(s, e, 2);
            if (a == cv[i] || b == cv[i] || c == cv[i]) continue;
            const double *en = s->nrm + 3 * (size_t)e, *er = s->cen + 3 * (size_t)e;
            double dc = distance_face(en, er, p), dm = distance_face(en, er, pm);
            if (dc * dm > 0.0) continue;
            double po[3];
            plane_inter(en, er, p, pm, po);
            if (point_in_triangle(vtx(s, a), vtx(s, b), vtx(s, c), po)) crossed = 1;
        }
        if (!crossed) choice = i;
    }
    if (choice < 0) return -1;
    const int ref = cv[choice];
    int em = edge_marker(s, ref, nbr, OG_NSIZE);
    if (em < 0) return -1;
    if (em == 1) { *dotNorm = -1.0; *elemOut = -1; return 0; }
    nn = 0;
    for (int m = 0; m < s->nt; ++m)
        if (node(s, m, 0) == ref || node(s, m, 1) == ref || node(s, m, 2) == ref) {
            if (nn >= OG_NSIZE) return -1;
            nbr[nn++] = m;
        }
    /* the element: among those whose normal projection falls inside, the
     * nearest plane (last of equals); before the first such element, the
     * smallest outside angle (last of equals) */
    double distIn = 1.0e16, angMin = 1.0e16;
    int inside = 0, ce = -1;
    for (int q = 0; q < nn; ++q) {
        int e = nbr[q];
        double bi[3], a123, adiff, din;
        bi_inside(s, e, p, bi, &a123, &adiff, &din);
        if (fabs(adiff) < 1.0e-4 * a123) {
            inside = 1;
            if (din <= distIn) { distIn = din; ce = e; }
        } else if (!inside) {
            double ang = bi_outside(s, e, p, ref);
            if (ang <= angMin) { angMin = ang; ce = e; }
        }
    }
    if (ce < 0) return -1;
    const double *cn = s->nrm + 3 * (size_t)ce, *cc = s->cen + 3 * (size_t)ce;
    *dotNorm = (p[0] - cc[0]) * cn[0] + (p[1] - cc[1]) * cn[1] + (p[2] - cc[2]) * cn[2];
    *elemOut = ce;
    return 0;
}

static void centres(int n, const double *x, double *xc, double *dx)
{
    for (int i = 0; i <= n; ++i) { xc[i] = 0.5 * (x[i + 1] + x[i]); dx[i] = x[i + 1] - x[i]; }
    xc[n + 1] = x[n + 1];
}

static size_t fi(int nx, int ny, int i, int j, int k)
{
    return (size_t)i + (size_t)(nx + 2) * ((size_t)j + (size_t)(ny + 2) * (size_t)k);
}

int og_orient_inward(int nv, const double *verts, int nt, int32_t *tris, double ox, double oy, double oz)
{
    /* marker nearest the outside point (last of equals: the reference tests <=) */
    int cnode = -1;
    double dmin = 1.0e8;
    for (int m = 0; m < nv; ++m) {
        const double *q = verts + 3 * (size_t)m;
        double d = sqrt((q[0] - ox) * (q[0] - ox) + (q[1] - oy) * (q[1] - oy) + (q[2] - oz) * (q[2] - oz));
        if (d <= dmin) { dmin = d; cnode = m; }
    }
    if (cnode < 0) return -1;
    int ce = -1;   /* last element containing it */
    for (int m = 0; m < nt; ++m)
        if (tris[3 * m] == cnode || tris[3 * m + 1] == cnode || tris[3 * m + 2] == cnode) ce = m;
    if (ce < 0) return -1;
    const double *p1 = verts + 3 * (size_t)tris[3 * ce], *p2 = verts + 3 * (size_t)tris[3 * ce + 1],
                 *p3 = verts + 3 * (size_t)tris[3 * ce + 2];
    double a[3] = {p2[0] - p1[0], p2[1] - p1[1], p2[2] - p1[2]};
    double b[3] = {p3[0] - p2[0], p3[1] - p2[1], p3[2] - p2[2]};
    double n[3];
    cross3(a, b, n);
    double c[3] = {(p1[0] + p2[0] + p3[0]) / 3.0, (p1[1] + p2[1] + p3[1]) / 3.0, (p1[2] + p2[2] + p3[2]) / 3.0};
    double vp = (c[0] - ox) * n[0] + (c[1] - oy) * n[1] + (c[2] - oz) * n[2];
    if (vp < 0.0) {
        for (int m = 0; m < nt; ++m) {
            int32_t t2 = tris[3 * m + 1];
            tris[3 * m + 1] = tris[3 * m + 2];
            tris[3 * m + 2] = t2;
        }
        return 1;
    }
    return 0;
}

/* set_iblank_canonical_body_fast for one solid body in 3D.  band (optional,
 * same shape as iblank) receives 1 for the cells classified by the dot-normal
 * test.  Returns the number of solid cells, or -1. */
long og_iblank(int nx, int ny, int nz, const double *x, const double *y, const double *z, int nv,
               const double *verts, int nt, const int32_t *tris, int8_t *iblank, int8_t *band)
{
    const int nxc = nx - 1, nyc = ny - 1, nzc = nz - 1;
    double *xc = malloc(sizeof(double) * (size_t)(nx + 2)), *dxv = malloc(sizeof(double) * (size_t)(nx + 2));
    double *yc = malloc(sizeof(double) * (size_t)(ny + 2)), *dyv = malloc(sizeof(double) * (size_t)(ny + 2));
    double *zc = malloc(sizeof(double) * (size_t)(nz + 2)), *dzv = malloc(sizeof(double) * (size_t)(nz + 2));
    const size_t nf = (size_t)(nx + 2) * (size_t)(ny + 2) * (size_t)(nz + 2);
    int8_t *und = calloc(nf, 1), *tmp = calloc(nf, 1);
    double *scratch = malloc(sizeof(double) * (size_t)(nv > 0 ? nv : 1));
    int *nbr = malloc(sizeof(int) * OG_NSIZE);
    surf_t s;
    long result = -1;
    if (!xc || !dxv || !yc || !dyv || !zc || !dzv || !und || !tmp || !scratch || !nbr) goto done;
    if (surf_open(&s, nv, verts, nt, tris) != 0) { surf_close(&s); goto done; }
    centres(nx, x, xc, dxv); centres(ny, y, yc, dyv); centres(nz, z, zc, dzv);

    /* undecided value 1 over (0:nx, 0:ny, 0:nz) */
    for (int k = 0; k <= nz; ++k)
        for (int j = 0; j <= ny; ++j)
            for (int i = 0; i <= nx; ++i) und[fi(nx, ny, i, j, k)] = 1;
    /* the band: cells whose centres bracket each element's bounding box */
    for (int m = 0; m < nt; ++m) {
        const double *v1 = verts + 3 * (size_t)tris[3 * m], *v2 = verts + 3 * (size_t)tris[3 * m + 1],
                     *v3 = verts + 3 * (size_t)tris[3 * m + 2];
        if ((v1[0] <= x[1] && v2[0] <= x[1] && v3[0] <= x[1]) || (v1[0] >= x[nx] && v2[0] >= x[nx] && v3[0] >= x[nx]) ||
            (v1[1] <= y[1] && v2[1] <= y[1] && v3[1] <= y[1]) || (v1[1] >= y[ny] && v2[1] >= y[ny] && v3[1] >= y[ny]) ||
            (v1[2] <= z[1] && v2[2] <= z[1] && v3[2] <= z[1]) || (v1[2] >= z[nz] && v2[2] >= z[nz] && v3[2] >= z[nz]))
            continue;
        int lo[3], hi[3];
        const int nn[3] = {nx, ny, nz}, nc[3] = {nxc, nyc, nzc};
        const double *cc[3] = {xc, yc, zc};
        for (int d = 0; d < 3; ++d) {
            double bmin = fmin(fmin(v1[d], v2[d]), v3[d]), bmax = fmax(fmax(v1[d], v2[d]), v3[d]);
            int cmin = 0, cmax = 0;
            for (int i = 0; i <= nn[d] - 1; ++i) {
                if ((cc[d][i] - bmin) * (cc[d][i + 1] - bmin) <= 0.0) cmin = i;
                if ((cc[d][i] - bmax) * (cc[d][i + 1] - bmax) <= 0.0) cmax = i + 1;
            }
            if (cmin == 0) cmin = 1;
            if (cmax == 0 || cmax == nn[d]) cmax = nc[d];
            lo[d] = cmin; hi[d] = cmax;
        }
        for (int k = lo[2]; k <= hi[2]; ++k)
            for (int j = lo[1]; j <= hi[1]; ++j)
                for (int i = lo[0]; i <= hi[0]; ++i) und[fi(nx, ny, i, j, k)] = -1;
    }
    /* the dot-normal test on the band */
    for (int k = 1; k <= nzc; ++k)
        for (int j = 1; j <= nyc; ++j)
            for (int i = 1; i <= nxc; ++i) {
                size_t o = fi(nx, ny, i, j, k);
                if (und[o] != -1) continue;
                double p[3] = {xc[i], yc[j], zc[k]}, dn;
                int e;
                if (search_vertex_dotnorm(&s, p, scratch, nbr, &dn, &e) != 0) { surf_close(&s); goto done; }
                tmp[o] = dn >= 0.0 ? 1 : 0;
            }
    /* fill along i: seed (0, j, k) from the first decided cell of the line */
    for (int k = 1; k <= nzc; ++k)
        for (int j = 1; j <= nyc; ++j)
            for (int ii = 1; ii <= nx; ++ii)
                if (und[fi(nx, ny, ii, j, k)] != 1) { tmp[fi(nx, ny, 0, j, k)] = tmp[fi(nx, ny, ii, j, k)]; break; }
    for (int i = 1; i <= nx; ++i)
        for (int k = 1; k <= nzc; ++k)
            for (int j = 1; j <= nyc; ++j)
                if (und[fi(nx, ny, i, j, k)] == 1) tmp[fi(nx, ny, i, j, k)] = tmp[fi(nx, ny, i - 1, j, k)];
    /* along j */
    for (int k = 1; k <= nzc; ++k)
        for (int i = 1; i <= nxc; ++i)
            for (int jj = 1; jj <= ny; ++jj)
                if (und[fi(nx, ny, i, jj, k)] != 1) { tmp[fi(nx, ny, i, 0, k)] = tmp[fi(nx, ny, i, jj, k)]; break; }
    for (int j = 1; j <= ny; ++j)
        for (int k = 1; k <= nzc; ++k)
            for (int i = 1; i <= nxc; ++i)
                if (und[fi(nx, ny, i, j, k)] == 1) tmp[fi(nx, ny, i, j, k)] = tmp[fi(nx, ny, i, j - 1, k)];
    /* along k (kk and k run to nzc + 1 = nz) */
    for (int j = 1; j <= nyc; ++j)
        for (int i = 1; i <= nxc; ++i)
            for (int kk = 1; kk <= nz; ++kk)
                if (und[fi(nx, ny, i, j, kk)] != 1) { tmp[fi(nx, ny, i, j, 0)] = tmp[fi(nx, ny, i, j, kk)]; break; }
    for (int k = 1; k <= nz; ++k)
        for (int j = 1; j <= nyc; ++j)
            for (int i = 1; i <= nxc; ++i)
                if (und[fi(nx, ny, i, j, k)] == 1) tmp[fi(nx, ny, i, j, k)] = tmp[fi(nx, ny, i, j, k - 1)];
    memset(iblank, 0, nf);
    if (band) memset(band, 0, nf);
    for (int k = 1; k <= nzc; ++k)
        for (int j = 1; j <= nyc; ++j)
            for (int i = 1; i <= nxc; ++i) {
                size_t o = fi(nx, ny, i, j, k);
                iblank[o] = tmp[o];
                if (band && und[o] == -1) band[o] = 1;
            }
    /* set_internal_boundary (IBM/BOUNDARY_SET.F90:267-410) then runs, for
     * solid bodies, find_isolatedIblank(1) (:440-499), find_iblankHoles(1)
     * (:502-602, which acts under SSM only) and fill_cell
     * (IBM/SSM_SET_BC.F90:1425-1511) */
    for (int k = 1; k <= nzc; ++k)
        for (int j = 1; j <= nyc; ++j)
            for (int i = 1; i <= nxc; ++i) {
                if (iblank[fi(nx, ny, i, j, k)] != 1) continue;
                int sum = 0;
                for (int kk = (k - 1 > 1 ? k - 1 : 1); kk <= (k + 1 < nzc ? k + 1 : nzc); ++kk)
                    for (int jj = (j - 1 > 1 ? j - 1 : 1); jj <= (j + 1 < nyc ? j + 1 : nyc); ++jj)
                        for (int ii = (i - 1 > 1 ? i - 1 : 1); ii <= (i + 1 < nxc ? i + 1 : nxc); ++ii)
                            sum += iblank[fi(nx, ny, ii, jj, kk)];
                if (sum <= 1) iblank[fi(nx, ny, i, j, k)] = 0;
            }
    /* fill_cell: a fluid cell between a solid neighbour and a flagged face
     * turns solid; under GCM the level-1 face flags are those of
     * set_outer_iup (IBM/BOUNDARY_SET.F90:54-130), set on the first and last
     * cell of every line */
    for (int pass = 0; pass < 3; ++pass)
        for (int k = 1; k <= nzc; ++k)
            for (int j = 1; j <= nyc; ++j)
                for (int i = 1; i <= nxc; ++i) {
                    size_t o = fi(nx, ny, i, j, k);
                    if (iblank[o] != 0) continue;
                    int c = pass == 0 ? i : pass == 1 ? j : k, last = pass == 0 ? nxc : pass == 1 ? nyc : nzc;
                    size_t om = pass == 0 ? fi(nx, ny, i - 1, j, k) : pass == 1 ? fi(nx, ny, i, j - 1, k) : fi(nx, ny, i, j, k - 1);
                    size_t op = pass == 0 ? fi(nx, ny, i + 1, j, k) : pass == 1 ? fi(nx, ny, i, j + 1, k) : fi(nx, ny, i, j, k + 1);
                    int up = c == last, um = c == 1;
                    if ((iblank[om] == 1 && up) || (iblank[op] == 1 && um)) iblank[o] = 1;
                }
    result = 0;
    for (size_t o = 0; o < nf; ++o) result += iblank[o];
    surf_close(&s);
done:
    free(xc); free(dxv); free(yc); free(dyv); free(zc); free(dzv);
    free(und); free(tmp); free(scratch); free(nbr);
    return result;
}

/* ghost marks and list (IBM/GCM_SET_BOUNDARY.F90:22-118); returns nGhost or
 * -1 when cap is too small */
int og_ghost_list(int nx, int ny, int nz, const int8_t *iblank, int8_t *ghost, int cap, int32_t *iG,
                  int32_t *jG, int32_t *kG)
{
    const size_t nf = (size_t)(nx + 2) * (size_t)(ny + 2) * (size_t)(nz + 2);
    memset(ghost, 0, nf);
    for (int k = 1; k <= nz - 1; ++k)
        for (int j = 1; j <= ny - 1; ++j)
            for (int i = 1; i <= nx - 1; ++i) {
                int iM = i - 1 > 1 ? i - 1 : 1, iP = i + 1 < nx - 1 ? i + 1 : nx - 1;
                int jM = j - 1 > 1 ? j - 1 : 1, jP = j + 1 < ny - 1 ? j + 1 : ny - 1;
                int kM = k - 1 > 1 ? k - 1 : 1, kP = k + 1 < nz - 1 ? k + 1 : nz - 1;
                int b = iblank[fi(nx, ny, i, j, k)];
                if (b * iblank[fi(nx, ny, iM, j, k)] == 0 || b * iblank[fi(nx, ny, iP, j, k)] == 0 ||
                    b * iblank[fi(nx, ny, i, jM, k)] == 0 || b * iblank[fi(nx, ny, i, jP, k)] == 0 ||
                    b * iblank[fi(nx, ny, i, j, kM)] == 0 || b * iblank[fi(nx, ny, i, j, kP)] == 0)
                    if (b == 1) ghost[fi(nx, ny, i, j, k)] = 1;
            }
    int n = 0;
    for (int k = 1; k <= nz - 1; ++k)
        for (int j = 1; j <= ny - 1; ++j)
            for (int i = 1; i <= nx - 1; ++i)
                if (ghost[fi(nx, ny, i, j, k)] == 1) {
                    if (n < cap) { iG[n] = i; jG[n] = j; kG[n] = k; }
                    ++n;
                }
    return n <= cap ? n : -1;
}

/* GCM_calc_bodyIntercept_Unstruc for the point p: body intercept bi and its
 * element; -1 on a list overflow */
static int body_intercept(const surf_t *s, const double *p, double *scratch, int *nbr, double *bi, int *elem)
{
    int cn[OG_NCHECK];
    closest_markers(s, p, OG_NCHECK, cn, scratch);
    double bit[OG_NCHECK][3];
    int cel[OG_NCHECK];
    for (int c = 0; c < OG_NCHECK; ++c) {
        int nn = 0;
        for (int m = 0; m < s->nt; ++m)
            if (node(s, m, 0) == cn[c] || node(s, m, 1) == cn[c] || node(s, m, 2) == cn[c]) {
                if (nn >= OG_NSIZE) return -1;
                nbr[nn++] = m;
            }
        int ce = -1, found = 0;
        double angMin = 1.0e16, b[3] = {0.0, 0.0, 0.0};
        for (int q = 0; q < nn && !found; ++q) {
            int e = nbr[q];
            double t[3], a123, adiff, din;
            bi_inside(s, e, p, t, &a123, &adiff, &din);
            if (fabs(adiff) < 1.0e-4 * a123) {
                memcpy(b, t, sizeof b);
                ce = e;
                found = 1;       /* the first element whose projection falls inside */
            } else {
                double ang = bi_outside(s, e, p, cn[c]);
                if (ang <= angMin) { angMin = ang; ce = e; memcpy(b, t, sizeof b); }
            }
        }
        if (ce < 0) return -1;
        if (!found) {
            /* projection onto the two edges of the chosen element that leave
             * the closest marker, clamped to the marker itself */
            int a = node(s, ce, 0), bb = node(s, ce, 1), cc = node(s, ce, 2), na, nb;
            if (a == cn[c]) { na = bb; nb = cc; }
            else if (bb == cn[c]) { na = cc; nb = a; }
            else { na = a; nb = bb; }
            const double *cv = vtx(s, cn[c]);
            double v01[3] = {p[0] - cv[0], p[1] - cv[1], p[2] - cv[2]};
            double dmin = 1.0e16, ei[3] = {cv[0], cv[1], cv[2]};
            for (int edge = 0; edge < 2; ++edge) {
                const double *pe = vtx(s, edge == 0 ? na : nb);
                double v12[3] = {pe[0] - cv[0], pe[1] - cv[1], pe[2] - cv[2]};
                double mag = sqrt(v12[0] * v12[0] + v12[1] * v12[1] + v12[2] * v12[2]);
                double inv = 1.0 / mag;
                for (int q = 0; q < 3; ++q) v12[q] = v12[q] * inv;
                double pl = v01[0] * v12[0] + v01[1] * v12[1] + v01[2] * v12[2];
                double t[3];
                if (pl < 0.0 || pl > mag) memcpy(t, cv, sizeof t);
                else for (int q = 0; q < 3; ++q) t[q] = cv[q] + pl * v12[q];
                double d = (t[0] - p[0]) * (t[0] - p[0]) + (t[1] - p[1]) * (t[1] - p[1]) + (t[2] - p[2]) * (t[2] - p[2]);
                if (d < dmin) { dmin = d; memcpy(ei, t, sizeof ei); }
            }
            memcpy(b, ei, sizeof b);
        }
        memcpy(bit[c], b, sizeof b);
        cel[c] = ce;
    }
    int best = 0;
    double dbest = 0.0;
    for (int c = 0; c < OG_NCHECK; ++c) {
        double d = (bit[c][0] - p[0]) * (bit[c][0] - p[0]) + (bit[c][1] - p[1]) * (bit[c][1] - p[1]) +
                   (bit[c][2] - p[2]) * (bit[c][2] - p[2]);
        if (c == 0 || d < dbest) { dbest = d; best = c; }
    }
    memcpy(bi, bit[best], 3 * sizeof(double));
    *elem = cel[best];
    return 0;
}

/* inverse of an 8 x 8 column-major matrix: LU with partial pivoting, then one
 * forward/back solve per unit vector; 0, or -1 for a zero pivot */
static int inverse8(const double *A, double *Ainv)
{
    double LU[64];
    int piv[8];
    memcpy(LU, A, sizeof LU);
    for (int k = 0; k < 8; ++k) {
        int p = k;
        for (int i = k + 1; i < 8; ++i)
            if (fabs(LU[i + 8 * k]) > fabs(LU[p + 8 * k])) p = i;
        piv[k] = p;
        if (LU[p + 8 * k] == 0.0) return -1;
        if (p != k)
            for (int j = 0; j < 8; ++j) { double t = LU[k + 8 * j]; LU[k + 8 * j] = LU[p + 8 * j]; LU[p + 8 * j] = t; }
        for (int i = k + 1; i < 8; ++i) {
            LU[i + 8 * k] /= LU[k + 8 * k];
            for (int j = k + 1; j < 8; ++j) LU[i + 8 * j] -= LU[i + 8 * k] * LU[k + 8 * j];
        }
    }
    for (int col = 0; col < 8; ++col) {
        double b[8] = {0};
        b[col] = 1.0;
        for (int k = 0; k < 8; ++k) { double t = b[k]; b[k] = b[piv[k]]; b[piv[k]] = t; }
        for (int i = 1; i < 8; ++i)
            for (int j = 0; j < i; ++j) b[i] -= LU[i + 8 * j] * b[j];
        for (int i = 7; i >= 0; --i) {
            for (int j = i + 1; j < 8; ++j) b[i] -= LU[i + 8 * j] * b[j];
            b[i] /= LU[i + 8 * i];
        }
        for (int i = 0; i < 8; ++i) Ainv[i + 8 * col] = b[i];
    }
    return 0;
}

static const int incI[8] = {0, 0, 1, 1, 0, 0, 1, 1};
static const int incJ[8] = {0, 1, 1, 0, 0, 1, 1, 0};
static const int incK[8] = {0, 0, 0, 0, 1, 1, 1, 1};

/* GCM_set_internal_boundary after the ghost list: per ghost the body
 * intercept bi (3, nGhost), its element, the probe length, the image point ip
 * (3, nGhost), the stencil cell and coeffGCMN / coeffGCMD (8, nGhost).
 * Returns 0, or -(n+1) for the first ghost whose stencil search or inverse
 * failed, or -(nGhost+1) on a list overflow. */
int og_gcm(int nx, int ny, int nz, const double *x, const double *y, const double *z, int nv,
           const double *verts, int nt, const int32_t *tris, double probeLengthNormalized, int nGhost,
           const int32_t *iG, const int32_t *jG, const int32_t *kG, int32_t *iCI, int32_t *jCI, int32_t *kCI,
           double *coeffN, double *coeffD, double *probe, double *bi, double *ip, int32_t *elem)
{
    double *xc = malloc(sizeof(double) * (size_t)(nx + 2)), *dxv = malloc(sizeof(double) * (size_t)(nx + 2));
    double *yc = malloc(sizeof(double) * (size_t)(ny + 2)), *dyv = malloc(sizeof(double) * (size_t)(ny + 2));
    double *zc = malloc(sizeof(double) * (size_t)(nz + 2)), *dzv = malloc(sizeof(double) * (size_t)(nz + 2));
    double *scratch = malloc(sizeof(double) * (size_t)(nv > 0 ? nv : 1));
    int *nbr = malloc(sizeof(int) * OG_NSIZE);
    surf_t s;
    int rc = -(nGhost + 1);
    if (!xc || !dxv || !yc || !dyv || !zc || !dzv || !scratch || !nbr) goto done;
    if (surf_open(&s, nv, verts, nt, tris) != 0) { surf_close(&s); goto done; }
    centres(nx, x, xc, dxv); centres(ny, y, yc, dyv); centres(nz, z, zc, dzv);
    rc = 0;
    for (int n = 0; n < nGhost && rc == 0; ++n) {
        const int gi = iG[n], gj = jG[n], gk = kG[n];
        double gc[3] = {xc[gi], yc[gj], zc[gk]}, b[3];
        int e;
        if (body_intercept(&s, gc, scratch, nbr, b, &e) != 0) { rc = -(nGhost + 1); break; }
        double ds = sqrt((gc[0] - b[0]) * (gc[0] - b[0]) + (gc[1] - b[1]) * (gc[1] - b[1]) + (gc[2] - b[2]) * (gc[2] - b[2]));
        double sl[3] = {(b[0] - gc[0]) / ds, (b[1] - gc[1]) / ds, (b[2] - gc[2]) / ds};
        double pl = ds * probeLengthNormalized;
        double xi = gc[0] + sl[0] * pl, yi = gc[1] + sl[1] * pl, zi = gc[2] + sl[2] * pl;
        probe[n] = pl;
        elem[n] = e;
        for (int q = 0; q < 3; ++q) bi[3 * (size_t)n + q] = b[q];
        ip[3 * (size_t)n] = xi; ip[3 * (size_t)n + 1] = yi; ip[3 * (size_t)n + 2] = zi;
        int iR = (int)lround(pl / dxv[gi]) + 1, jR = (int)lround(pl / dyv[gj]) + 1, kR = (int)lround(pl / dzv[gk]) + 1;
        int ci = -1, cj = -1, ck = -1;
        for (int i = gi - iR > 0 ? gi - iR : 0; i <= (gi + iR < nx ? gi + iR : nx); ++i)
            if (xc[i] <= xi && xc[i + 1] > xi) ci = i;
        for (int j = gj - jR > 0 ? gj - jR : 0; j <= (gj + jR < ny ? gj + jR : ny); ++j)
            if (yc[j] <= yi && yc[j + 1] > yi) cj = j;
        for (int k = gk - kR > 0 ? gk - kR : 0; k <= (gk + kR < nz ? gk + kR : nz); ++k)
            if (zc[k] <= zi && zc[k + 1] > zi) ck = k;
        iCI[n] = ci; jCI[n] = cj; kCI[n] = ck;
        if (ci < 0 || cj < 0 || ck < 0) { rc = -(n + 1); break; }
        const double *bn = s.nrm + 3 * (size_t)e;
        double VD[64], VN[64], ID[64], IN[64];
        for (int r = 0; r < 8; ++r) {
            int i = ci + incI[r], j = cj + incJ[r], k = ck + incK[r];
            double c1 = xc[i], c2 = yc[j], c3 = zc[k];
            double rowD[8] = {c1 * c2 * c3, c1 * c2, c1 * c3, c2 * c3, c1, c2, c3, 1.0};
            double rowN[8];
            memcpy(rowN, rowD, sizeof rowN);
            if (i == gi && j == gj && k == gk) {
                c1 = b[0]; c2 = b[1]; c3 = b[2];
                double n1 = bn[0], n2 = bn[1], n3 = bn[2];
                double d[8] = {c1 * c2 * c3, c1 * c2, c1 * c3, c2 * c3, c1, c2, c3, 1.0};
                memcpy(rowD, d, sizeof d);
                rowN[0] = n1 * c2 * c3 + n2 * c1 * c3 + n3 * c1 * c2;
                rowN[1] = n1 * c2 + n2 * c1;
                rowN[2] = n1 * c3 + n3 * c1;
                rowN[3] = n2 * c3 + n3 * c2;
                rowN[4] = n1; rowN[5] = n2; rowN[6] = n3; rowN[7] = 0.0;
            }
            for (int m = 0; m < 8; ++m) { VD[r + 8 * m] = rowD[m]; VN[r + 8 * m] = rowN[m]; }
        }
        if (inverse8(VD, ID) != 0 || inverse8(VN, IN) != 0) { rc = -(n + 1); break; }
        for (int r = 0; r < 8; ++r) {
            const double *d = ID + 8 * r, *m = IN + 8 * r;   /* column r of each inverse */
            coeffD[8 * (size_t)n + r] = d[0] * xi * yi * zi + d[1] * xi * yi + d[2] * xi * zi + d[3] * yi * zi +
                                        d[4] * xi + d[5] * yi + d[6] * zi + d[7];
            coeffN[8 * (size_t)n + r] = m[0] * xi * yi * zi + m[1] * xi * yi + m[2] * xi * zi + m[3] * yi * zi +
                                        m[4] * xi + m[5] * yi + m[6] * zi + m[7];
        }
    }
    surf_close(&s);
done:
    free(xc); free(dxv); free(yc); free(dyv); free(zc); free(dzv); free(scratch); free(nbr);
    return rc;
}
