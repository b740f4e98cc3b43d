/*
 * Plain-C host of the fsi_mg C ABI, laid out the way the reference's Fortran
 * module arrays are: column-major, lower bound 0, REAL(8) fields over
 * (0:nx+1,0:ny+1,0:nz+1), INTEGER(1) flags, INTEGER(4) ghost lists.  It plays
 * the role of the reference's time loop around solve_poisson
 * (IBM/CORE_POISSON.F90:493): MG_initial -> the hand-over after set_boundary
 * -> solve_poisson -> deallocate_memory.
 *
 * Test infrastructure: tests/test_abi.py builds it and the GPU tests run it on
 * an input file written by the test (all arrays in the order read below) and
 * compare its output with the Python binding's solve of the same input.
 *
 * usage: fsi_mg_driver <input> <output>
 * output: int32 status, int32 iters, float64 maxres, int32 loc[3], the
 *         solved pPrime, and the fluid-volume mean of pPrime computed here
 *         with Fortran index arithmetic.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include "fsi_mg.h"

/* (i,j,k) of a (0:nx+1,0:ny+1,0:nz+1) Fortran array */
#define F3(a, i, j, k) (a)[(size_t)(i) + (size_t)(nx + 2) * ((size_t)(j) + (size_t)(ny + 2) * (size_t)(k))]

static void *read_n(FILE *f, size_t bytes)
{
    void *p = malloc(bytes ? bytes : 1);
    if (!p || fread(p, 1, bytes, f) != bytes) {
        fprintf(stderr, "short input\n");
        exit(3);
    }
    return p;
}

int main(int argc, char **argv)
{
    if (argc != 3) {
        fprintf(stderr, "usage: %s <input> <output>\n", argv[0]);
        return 2;
    }
    FILE *in = fopen(argv[1], "rb");
    if (!in) { perror("input"); return 2; }
    fsi_mg_params *prm = (fsi_mg_params *)read_n(in, sizeof(fsi_mg_params));
    const int nx = prm->nx, ny = prm->ny, nz = prm->nz;
    const size_t nf = (size_t)(nx + 2) * (size_t)(ny + 2) * (size_t)(nz + 2);
    double *x = (double *)read_n(in, sizeof(double) * (size_t)(nx + 2));
    double *y = (double *)read_n(in, sizeof(double) * (size_t)(ny + 2));
    double *z = (double *)read_n(in, sizeof(double) * (size_t)(nz + 2));
    int8_t *iblank = (int8_t *)read_n(in, nf), *ghost = (int8_t *)read_n(in, nf);
    int8_t *fl[6];
    for (int q = 0; q < 6; ++q) fl[q] = (int8_t *)read_n(in, nf);
    int32_t *ng = (int32_t *)read_n(in, sizeof(int32_t));
    const int nGhost = *ng;
    int32_t *gl[6];
    for (int q = 0; q < 6; ++q) gl[q] = (int32_t *)read_n(in, sizeof(int32_t) * (size_t)nGhost);
    double *coeff = (double *)read_n(in, sizeof(double) * 8 * (size_t)nGhost);
    double *probe = (double *)read_n(in, sizeof(double) * (size_t)nGhost);
    const size_t npg = 2 * (size_t)(ny + 2) * (nz + 2) + 2 * (size_t)(nx + 2) * (nz + 2) + 2 * (size_t)(nx + 2) * (ny + 2);
    double *pgrad = (double *)read_n(in, sizeof(double) * npg);
    double *nlu0 = (double *)read_n(in, sizeof(double) * nf);
    fclose(in);

    double *pPrime = (double *)calloc(nf, sizeof(double));
    void *h = NULL;
    int rc = fsi_mg_create(prm, x, y, z, &h);                                   /* MG_initial */
    if (rc < 0) { fprintf(stderr, "fsi_mg_create: %s\n", fsi_mg_last_error()); return 1; }
    rc = fsi_mg_set_geometry(h, iblank, ghost, fl[0], fl[1], fl[2], fl[3], fl[4], fl[5], nGhost,
                             gl[0], gl[1], gl[2], gl[3], gl[4], gl[5], coeff, probe, pgrad);
    if (rc < 0) { fprintf(stderr, "fsi_mg_set_geometry: %s\n", fsi_mg_last_error()); return 1; }
    int iters = 0, loc[3] = {0, 0, 0};
    double maxres = 0.0, t = 0.0;
    const int st = fsi_mg_solve(h, pPrime, nlu0, NULL, &iters, &maxres, loc, &t);   /* solve_poisson */
    if (st < 0) { fprintf(stderr, "fsi_mg_solve: %s\n", fsi_mg_last_error()); return 1; }
    fsi_mg_destroy(h);                                                           /* deallocate_memory */

    /* fluid-volume mean over the interior cells, Fortran index arithmetic */
    double sp = 0.0, sv = 0.0;
    for (int k = 1; k <= nz - 1; ++k)
        for (int j = 1; j <= ny - 1; ++j)
            for (int i = 1; i <= nx - 1; ++i)
                if (F3(iblank, i, j, k) == 0) {
                    const double vol = (x[i + 1] - x[i]) * (y[j + 1] - y[j]) * (z[k + 1] - z[k]);
                    sp += F3(pPrime, i, j, k) * vol;
                    sv += vol;
                }
    const double mean = sp / sv;

    FILE *out = fopen(argv[2], "wb");
    if (!out) { perror("output"); return 2; }
    const int32_t hdr[2] = {st, iters};
    const int32_t l3[3] = {loc[0], loc[1], loc[2]};
    fwrite(hdr, sizeof(int32_t), 2, out);
    fwrite(&maxres, sizeof(double), 1, out);
    fwrite(l3, sizeof(int32_t), 3, out);
    fwrite(pPrime, sizeof(double), nf, out);
    fwrite(&mean, sizeof(double), 1, out);
    fclose(out);
    printf("status %d iters %d maxres %.3e\n", st, iters, maxres);
    return 0;
}
