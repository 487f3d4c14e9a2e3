/*
 * ORACLE -- test infrastructure, not the product.  Convection with diffusion folded in, one
 * column at a time, dense, in the reference's evaluation order: pydyn kernels.py:350-396
 * (convection_matrix), :399-420 (fastminv, the Crout inverse without pivoting), :423-457 (convec),
 * zoom/physics.py:33-52 (convec_region on the owned columns).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    double *p;
    int64_t n[4];
    int64_t s[4];
} ov;

#define A3(v, i, j, l) ((v)->p[(int64_t)(i) * (v)->s[0] + (int64_t)(j) * (v)->s[1] + (int64_t)(l) * (v)->s[2]])
#define A4(v, i, j, l, t) \
    ((v)->p[(int64_t)(i) * (v)->s[0] + (int64_t)(j) * (v)->s[1] + (int64_t)(l) * (v)->s[2] + (int64_t)(t) * (v)->s[3]])

/* np.maximum(0.0, x) */
static double max0(double x) { return isnan(x) ? x : (0.0 > x ? 0.0 : x); }

/* conv1 (n x n, row-major) of one column: m, entu, detu, entd, detd, dkg are the column's first n
 * levels (stride-1 copies), top / lfs its 1-based cloud top and level of free sinking. */
static void matrix(const double *m, const double *entu, const double *detu, const double *entd, const double *detd,
                   const double *dkg, int top, int lfs, double dt, int n, double *conv1, double *work) {
    double *fu = work, *fd = fu + (n + 1) * n, *amu = fd + (n + 1) * n, *amd = amu + n + 1;
    memset(work, 0, sizeof(double) * ((size_t)2 * (n + 1) * n + 2 * (n + 1)));
#define FU(k, l) fu[(k) * n + (l)]
#define FD(k, l) fd[(k) * n + (l)]
    for (int k = 1; k <= n; k++) { /* the updraft */
        int act = top >= k;
        double a = amu[k - 1] + entu[k - 1] - detu[k - 1];
        int up = a > 0.0;
        double zxi = up ? max0(1.0 - detu[k - 1] / (amu[k - 1] + entu[k - 1])) : 0.0;
        amu[k] = (act && up) ? a : 0.0;
        for (int l = 0; l < k - 1; l++) FU(k, l) = act ? FU(k - 1, l) * zxi : 0.0;
        FU(k, k - 1) = act ? entu[k - 1] / m[k - 1] * zxi : 0.0;
    }
    for (int k = n; k >= 2; k--) { /* the downdraft */
        int act = lfs >= k;
        double a = amd[k] - entd[k - 1] + detd[k - 1];
        int dn = a < 0.0;
        double zxi = dn ? max0(1.0 + detd[k - 1] / (amd[k] - entd[k - 1])) : 0.0;
        amd[k - 1] = (act && dn) ? a : 0.0;
        for (int l = k; l < n; l++) FD(k - 1, l) = act ? FD(k, l) * zxi : FD(k - 1, l);
        FD(k - 1, k - 1) = act ? -entd[k - 1] / m[k - 1] * zxi : FD(k - 1, k - 1);
    }
    for (int k = 1; k < n; k++) { /* combined, compensating subsidence, diffusion */
        for (int l = 0; l < n; l++) FD(k, l) = FU(k, l) + FD(k, l);
        FD(k, k) = FD(k, k) - amu[k] / m[k];
        FD(k, k - 1) = FD(k, k - 1) - amd[k] / m[k - 1];
        FD(k, k - 1) = FD(k, k - 1) + dkg[k - 1] / m[k - 1];
        FD(k, k) = FD(k, k) - dkg[k - 1] / m[k];
    }
    for (int k = 1; k <= n; k++) {
        for (int l = 0; l < n; l++) conv1[(k - 1) * n + l] = -dt * (FD(k - 1, l) - FD(k, l));
        conv1[(k - 1) * n + k - 1] = conv1[(k - 1) * n + k - 1] + 1.0;
    }
#undef FU
#undef FD
}

/* fastminv: Crout LU without pivoting, then the inverse by forward and back substitution of the
 * identity, in convection.F90's loop order.  a (n x n) is overwritten by the LU factors. */
static void crout_inverse(double *a, int n, double *inv, double *y) {
#define LU(i, j) a[(i) * n + (j)]
    for (int j = 0; j < n; j++) {
        for (int k = 0; k < j; k++)
            for (int i = k + 1; i < n; i++) LU(i, j) = LU(i, j) - LU(i, k) * LU(k, j);
        for (int i = j + 1; i < n; i++) LU(i, j) = LU(i, j) / LU(j, j);
    }
    for (int i = 0; i < n; i++)
        for (int c = 0; c < n; c++) y[i * n + c] = (i == c) ? 1.0 : 0.0;
    for (int i = 0; i < n; i++)
        for (int j = 0; j < i; j++)
            for (int c = 0; c < n; c++) y[i * n + c] = y[i * n + c] - LU(i, j) * y[j * n + c];
    for (int i = n - 1; i >= 0; i--) {
        for (int c = 0; c < n; c++) inv[i * n + c] = y[i * n + c];
        for (int j = i + 1; j < n; j++)
            for (int c = 0; c < n; c++) inv[i * n + c] = inv[i * n + c] - LU(i, j) * inv[j * n + c];
        for (int c = 0; c < n; c++) inv[i * n + c] = inv[i * n + c] / LU(i, i);
    }
#undef LU
}

/* convec on the listed columns (i, j) = (cols[2c], cols[2c+1]) of a region's interior views:
 * m, tracers (im, jm, lm[, nt]), entu.. (im, jm, >= lmax), dkg (im, jm, >= lmax), cloud_top /
 * cloud_lfs (im, jm) int32 with element strides ts0, ts1. */
void or_convec(const ov *m, const ov *rm, const ov *rxm, const ov *rym, const ov *rzm, const ov *entu, const ov *detu,
               const ov *entd, const ov *detd, const ov *dkg, const int32_t *top, const int32_t *lfs, int64_t ts0,
               int64_t ts1, const int32_t *cols, int ncol, double dt, int lmax) {
    const int n = lmax, nt = (int)rm->n[3];
    if (n <= 0) return;
#pragma omp parallel
    {  /* columns are independent: each thread its own work arrays */
    double *col = malloc(sizeof(double) * 6 * n);
    double *conv1 = malloc(sizeof(double) * n * n), *inv = malloc(sizeof(double) * n * n);
    double *y = malloc(sizeof(double) * n * n);
    double *work = malloc(sizeof(double) * (2 * (n + 1) * n + 2 * (n + 1)));
    double *srm = malloc(sizeof(double) * n), *zrm = malloc(sizeof(double) * n);
#pragma omp for schedule(dynamic, 8)
    for (int c = 0; c < ncol; c++) {
        const int i = cols[2 * c], j = cols[2 * c + 1];
        double *cm = col, *ce = col + n, *cd = col + 2 * n, *ced = col + 3 * n, *cdd = col + 4 * n, *ck = col + 5 * n;
        for (int l = 0; l < n; l++) {
            cm[l] = A3(m, i, j, l);
            ce[l] = A3(entu, i, j, l);
            cd[l] = A3(detu, i, j, l);
            ced[l] = A3(entd, i, j, l);
            cdd[l] = A3(detd, i, j, l);
            ck[l] = A3(dkg, i, j, l);
        }
        matrix(cm, ce, cd, ced, cdd, ck, top[i * ts0 + j * ts1], lfs[i * ts0 + j * ts1], dt, n, conv1, work);
        crout_inverse(conv1, n, inv, y);
        const ov *slopes[3] = {rxm, rym, rzm};
        for (int w = 0; w < 3; w++)
            for (int l = 0; l < n; l++)
                for (int t = 0; t < nt; t++) A4(slopes[w], i, j, l, t) = inv[l * n + l] * A4(slopes[w], i, j, l, t);
        for (int t = 0; t < nt; t++) {
            for (int l = 0; l < n; l++) {
                srm[l] = A4(rm, i, j, l, t);
                zrm[l] = 0.0;
            }
            for (int k = 0; k < n; k++)
                for (int l = 0; l < n; l++) zrm[l] = zrm[l] + inv[l * n + k] * srm[k];
            for (int l = 0; l < n; l++) A4(rm, i, j, l, t) = zrm[l];
        }
    }
    free(col);
    free(conv1);
    free(inv);
    free(y);
    free(work);
    free(srm);
    free(zrm);
    }
}
