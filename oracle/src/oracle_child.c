/*
 * ORACLE -- test infrastructure, not the product.  A child region's held-end x rows and y
 * columns, scalar C in the reference's evaluation order (pydyn zoom/advect.py:278-412,
 * zoom/check_cfl.py:113-193).  A held line has n cells whose two ends are held (the parent's)
 * and n-1 faces, face k between cells k and k+1.
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

static double clipc(double s, double r) {
    double hi = fabs(r), lo = -hi;
    double t = isnan(s) ? s : (s > lo ? s : lo);
    return isnan(t) ? t : (t < hi ? t : hi);
}

static void flux4c(double flux, double c, double rmu, double su, double tu, double wu, double *f, double *pf,
                   double *ft, double *fw) {
    double v = flux >= 0.0 ? c * (rmu + (1.0 - c) * su) : c * (rmu - (1.0 + c) * su);
    *f = v;
    *pf = flux * (c * c * su - 3.0 * v);
    *ft = c * tu;
    *fw = c * wu;
}

/* kernels.py:169-199 subcycle_rows with periodic=False for one row: nloop trial sub-steps of the
 * row's mass with its end cells held.  Faces rescaled in place per retry.  0 past nmax. */
static int held_search(const double *m, double *a, int n, int nmax) {
    double *mx = malloc(sizeof(double) * n);
    int nloop = 1;
    for (;;) {
        int ok = 1;
        memcpy(mx, m, sizeof(double) * n);
        for (int s = 0; s < nloop && ok; s++) {
            for (int k = 0; k < n - 1; k++) {
                double mu = a[k] >= 0.0 ? mx[k] : mx[k + 1];
                if (!(fabs(a[k] / mu) < 1.0)) ok = 0;
            }
            if (!ok) break;
            double prev = a[0];
            for (int i = 1; i < n - 1; i++) {
                mx[i] = (mx[i] + prev) - a[i];
                prev = a[i];
            }
        }
        if (ok) break;
        nloop++;
        for (int k = 0; k < n - 1; k++) a[k] = a[k] * (double)(nloop - 1) / (double)nloop;
        if (nloop > nmax) {
            free(mx);
            return 0;
        }
    }
    free(mx);
    return nloop;
}

/* _dynamu_child's rows (zoom/advect.py:278-345) or _dynamum_child's (check_cfl.py:113-137):
 * m (n, nj, nl) cells is-1..ie+1, tracers alike, am (n-1, nj, nl).  Returns 0 or 1 (cap). */
int or_advect_x_held(const ov *m, const ov *rm, const ov *rxm, const ov *rym, const ov *rzm, const ov *am,
                     int limits, int max_nloop, int mass_only) {
    const int n = (int)m->n[0], nj = (int)m->n[1], nl = (int)m->n[2];
    const int nt = mass_only ? 0 : (int)rm->n[3];
    const ov *qv[4] = {rm, rxm, rym, rzm};
    double *mr = malloc(sizeof(double) * n), *a = malloc(sizeof(double) * n);
    double *q = malloc(sizeof(double) * n * (4 * nt + 1));
    double *f = malloc(sizeof(double) * n * 4), *mi = malloc(sizeof(double) * n);
    int failed = 0;
    for (int j = 0; j < nj; j++)
        for (int l = 0; l < nl; l++) {
            for (int i = 0; i < n; i++) {
                mr[i] = A3(m, i, j, l);
                for (int w = 0; w < 4; w++)
                    for (int t = 0; t < nt; t++) q[(w * nt + t) * n + i] = A4(qv[w], i, j, l, t);
            }
            for (int k = 0; k < n - 1; k++) a[k] = A3(am, k, j, l);
            if (!mass_only && limits) /* the limiter on every cell of the row, the ends included */
                for (int t = 0; t < nt; t++)
                    for (int i = 0; i < n; i++) q[(1 * nt + t) * n + i] = clipc(q[(1 * nt + t) * n + i], q[(0 * nt + t) * n + i]);
            int nloop = held_search(mr, a, n, max_nloop - 1);
            if (!nloop) {
                failed = 1;
                continue;
            }
            for (int s = 0; s < nloop; s++) {
                if (mass_only) {
                    double prev = a[0];
                    for (int i = 1; i < n - 1; i++) {
                        mr[i] = (mr[i] + prev) - a[i];
                        prev = a[i];
                    }
                    continue;
                }
                for (int i = 0; i < n; i++) mi[i] = 1.0 / mr[i];
                for (int t = 0; t < nt; t++) {
                    double *rq = q + (0 * nt + t) * n, *xq = q + (1 * nt + t) * n;
                    double *yq = q + (2 * nt + t) * n, *zq = q + (3 * nt + t) * n;
                    double *ff = f, *pf = f + n, *fy = f + 2 * n, *fz = f + 3 * n;
                    for (int k = 0; k < n - 1; k++) {
                        int up = a[k] >= 0.0 ? k : k + 1;
                        flux4c(a[k], a[k] * mi[up], rq[up], xq[up], yq[up], zq[up], &ff[k], &pf[k], &fy[k], &fz[k]);
                    }
                    for (int i = 1; i < n - 1; i++) {
                        double mo = mr[i], lo = a[i - 1], hi = a[i];
                        double mn = (mo + lo) - hi;
                        double rmn = rq[i] - (ff[i] - ff[i - 1]);
                        double xn = xq[i] + (pf[i - 1] - pf[i] - (lo - hi) * xq[i] +
                                             3.0 * ((lo + hi) * rmn - (ff[i - 1] + ff[i]) * mo)) / mn;
                        if (limits) xn = clipc(xn, rmn);
                        rq[i] = rmn;
                        xq[i] = xn;
                        yq[i] = yq[i] - (fy[i] - fy[i - 1]);
                        zq[i] = zq[i] - (fz[i] - fz[i - 1]);
                    }
                }
                for (int i = 1; i < n - 1; i++) mr[i] = (mr[i] + a[i - 1]) - a[i];
            }
            for (int k = 0; k < n - 1; k++) A3(am, k, j, l) = a[k] * (double)nloop;
            for (int i = 0; i < n; i++) {
                A3(m, i, j, l) = mr[i];
                for (int w = 0; w < 4; w++)
                    for (int t = 0; t < nt; t++) A4(qv[w], i, j, l, t) = q[(w * nt + t) * n + i];
            }
        }
    free(mr);
    free(a);
    free(q);
    free(f);
    free(mi);
    return failed;
}

/* _dynamv_child (zoom/advect.py:348-412) or _dynamvm_child (check_cfl.py:162-193), the columns of
 * one scope: m (ni, n, nl) cells js-1..je+1, tracers alike, bm (ni, n-1, nl) the scope's faces
 * js..je+1, full the whole halo'd bm and full_l0 the level of it that is bm's level 0.  The
 * tracer search rescales the whole layer of `full` per retry; the mass-only search rescales the
 * scope's faces; both restore the whole layer times nloop.  Returns 0 or 1 (cap). */
int or_advect_y_held(const ov *m, const ov *rm, const ov *rxm, const ov *rym, const ov *rzm, const ov *bm,
                     const ov *full, int full_l0, int limits, int max_nloop, int mass_only) {
    const int ni = (int)m->n[0], n = (int)m->n[1], nl = (int)m->n[2];
    const int nt = mass_only ? 0 : (int)rm->n[3];
    const int nmax = mass_only ? max_nloop : max_nloop - 1;
    double *mx = malloc(sizeof(double) * n), *f = malloc(sizeof(double) * n * 4);
    int failed = 0;
    if (!mass_only && limits)
        for (int i = 0; i < ni; i++)
            for (int j = 0; j < n; j++)
                for (int l = 0; l < nl; l++)
                    for (int t = 0; t < nt; t++) A4(rym, i, j, l, t) = clipc(A4(rym, i, j, l, t), A4(rm, i, j, l, t));
    for (int l = 0; l < nl && !failed; l++) {
        const int lf = l + full_l0;
        int nloop = 1;
        for (;;) {
            int ok = 1;
            for (int i = 0; i < ni && ok; i++) {
                for (int j = 0; j < n; j++) mx[j] = A3(m, i, j, l);
                for (int s = 0; s < nloop && ok; s++) {
                    for (int k = 0; k < n - 1; k++) {
                        double b = A3(bm, i, k, l);
                        double mu = b >= 0.0 ? mx[k] : mx[k + 1];
                        if (!(fabs(b / mu) < 1.0)) {
                            ok = 0;
                            break;
                        }
                    }
                    if (!ok) break;
                    for (int j = 1; j < n - 1; j++) mx[j] = (mx[j] + A3(bm, i, j - 1, l)) - A3(bm, i, j, l);
                }
            }
            if (ok) break;
            if (mass_only) { /* the scope's faces */
                for (int i = 0; i < ni; i++)
                    for (int k = 0; k < n - 1; k++)
                        A3(bm, i, k, l) = A3(bm, i, k, l) * (double)nloop / (double)(nloop + 1);
            } else { /* the whole layer, halos included */
                for (int64_t fi = 0; fi < full->n[0]; fi++)
                    for (int64_t fj = 0; fj < full->n[1]; fj++)
                        A3(full, fi, fj, lf) = A3(full, fi, fj, lf) * (double)nloop / (double)(nloop + 1);
            }
            nloop++;
            if (nloop > nmax) {
                failed = 1;
                break;
            }
        }
        if (failed) break;
        for (int i = 0; i < ni; i++) {
            for (int s = 0; s < nloop; s++) {
                if (mass_only) {
                    for (int j = 1; j < n - 1; j++)
                        A3(m, i, j, l) = (A3(m, i, j, l) + A3(bm, i, j - 1, l)) - A3(bm, i, j, l);
                    continue;
                }
                for (int t = 0; t < nt; t++) {
                    double *ff = f, *pf = f + n, *fx = f + 2 * n, *fz = f + 3 * n;
                    for (int k = 0; k < n - 1; k++) {
                        double b = A3(bm, i, k, l);
                        int up = b >= 0.0 ? k : k + 1;
                        double beta = b / A3(m, i, up, l);
                        flux4c(b, beta, A4(rm, i, up, l, t), A4(rym, i, up, l, t), A4(rxm, i, up, l, t),
                               A4(rzm, i, up, l, t), &ff[k], &pf[k], &fx[k], &fz[k]);
                    }
                    for (int j = 1; j < n - 1; j++) {
                        double lo = A3(bm, i, j - 1, l), hi = A3(bm, i, j, l);
                        double mo = A3(m, i, j, l);
                        double mn = (mo + lo) - hi;
                        double inv = 1.0 / mn;
                        double rmn = A4(rm, i, j, l, t) + (ff[j - 1] - ff[j]);
                        double ry = A4(rym, i, j, l, t);
                        double ryn = ry + ((pf[j - 1] - pf[j]) - (lo - hi) * ry + 3.0 * (lo + hi) * rmn -
                                           3.0 * mo * (ff[j - 1] + ff[j])) * inv;
                        if (limits) ryn = clipc(ryn, rmn);
                        A4(rm, i, j, l, t) = rmn;
                        A4(rym, i, j, l, t) = ryn;
                        A4(rxm, i, j, l, t) = A4(rxm, i, j, l, t) + (fx[j - 1] - fx[j]);
                        A4(rzm, i, j, l, t) = A4(rzm, i, j, l, t) + (fz[j - 1] - fz[j]);
                    }
                }
                for (int j = 1; j < n - 1; j++) A3(m, i, j, l) = (A3(m, i, j, l) + A3(bm, i, j - 1, l)) - A3(bm, i, j, l);
            }
        }
        for (int64_t fi = 0; fi < full->n[0]; fi++) /* restore the whole layer: times nloop */
            for (int64_t fj = 0; fj < full->n[1]; fj++) A3(full, fi, fj, lf) = A3(full, fi, fj, lf) * (double)nloop;
    }
    free(mx);
    free(f);
    return failed;
}
