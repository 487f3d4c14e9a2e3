/*
 * ORACLE -- test infrastructure, not the product.  A scalar, single-threaded C restatement of
 * pydyn's slopes advection, Check_CFL mass kernels, dynam0 and m2phlb, one line at a time in
 * the reference's evaluation order.  Only tests, the smoke check and bench.py's CPU-baseline leg
 * use it; nothing in the pydyn_gb300 package links or calls it.
 *
 * Arrays are strided views (pointer, extents, element strides) of C-contiguous float64 arrays in
 * the pydyn layout (pydyn kernels.py:7-16): m (im, jm, lm), tracers (im, jm, lm, nt),
 * am (im+1, jm, lm), bm (im, jm+1, lm), cm (im, jm, lm+1).
 *
 * Evaluation rules of NumPy the reference relies on, restated per element:
 *   np.clip(s, -|r|, |r|):  t = isnan(s) ? s : (s > lo ? s : lo); isnan(t) ? t : (t < hi ? t : hi)
 *   x - np.diff(f)[i]     = x - (f[i+1] - f[i])
 *   ops.advance(m, f)[i]  = (m[i] + f[i]) - f[i+1]
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

/* kernels.py:65-67 _limit, NumPy's clip */
static double limit(double s, double r) {
    double hi = fabs(r), lo = -hi;
    double t = isnan(s) ? s : (s > lo ? s : lo);
    return isnan(t) ? t : (t < hi ? t : hi);
}

/* kernels.py:75-84 _slopes_fluxes */
static void flux4(double flux, double c, double rmu, double su, double tu, double wu, double *f, double *pf,
                  double *ft, double *fw) {
    double v = flux >= 0.0 ? c * (rmu + (1.0 - c) * su) : c * (rmu - (1.0 + c) * su);
    *f = v;
    *pf = flux * (c * c * su - 3.0 * v);
    *ft = c * tu;
    *fw = c * wu;
}

/* kernels.py:87-92 _along_slope_update for one cell */
static double slope_update(double s, double pflo, double pfhi, double lo, double hi, double rmnew, double flo,
                           double fhi, double mold, double mnew) {
    return s + (pflo - pfhi - (lo - hi) * s + 3.0 * ((lo + hi) * rmnew - (flo + fhi) * mold)) / mnew;
}

/* ops.py:304-307 progressive, applied for n = 2 .. nloop */
static double rescaled(double f, int nloop) {
    for (int n = 2; n <= nloop; n++) f = f * (double)(n - 1) / (double)n;
    return f;
}

/* ------------------------------------------------------------------ x (dynamu)
 * One periodic row of n cells (kernels.py:144-220): limiter, the row's own CFL search
 * (kernels.py:169-199: trial sub-steps in the division form ops.py:267-270, faces rescaled by
 * progressive per retry), the sub-steps in the reciprocal form.  q[w * nt + t]: cell 0 of tracer
 * t of array w (rm, rxm, rym, rzm), unit cell stride.  Returns nloop, or 0 past the cap nmax. */
static int x_row(double *m, double **q, int nt, double *a, int n, int mass_only, int limits, int nmax,
                 double *amax_out) {
    double *mx = malloc(sizeof(double) * (n + 1));
    int nloop = 1;
    double amax = 0.0;
    if (!mass_only && limits)
        for (int t = 0; t < nt; t++)
            for (int i = 0; i < n; i++) q[1 * nt + t][i] = limit(q[1 * nt + t][i], q[0 * nt + t][i]);
    for (;;) {
        int ok = 1;
        amax = 0.0;
        for (int i = 0; i < n; i++) mx[i] = m[i];
        for (int s = 0; s < nloop; s++) {
            double cmax = 0.0;
            for (int k = 0; k <= n; k++) {
                int up = a[k] >= 0.0 ? (k == 0 ? n - 1 : k - 1) : (k == n ? 0 : k);
                double c = fabs(a[k] / mx[up]);
                if (!(c < 1.0)) ok = 0;
                if (c > cmax) cmax = c;
            }
            if (!ok) break;
            if (cmax > amax) amax = cmax;
            for (int i = 0; i < n; i++) mx[i] = (mx[i] + a[i]) - a[i + 1];
        }
        if (ok) break;
        nloop++;
        for (int k = 0; k <= n; k++) a[k] = a[k] * (double)(nloop - 1) / (double)nloop;
        if (nloop > nmax) {
            free(mx);
            return 0;
        }
    }
    free(mx);
    if (amax_out) *amax_out = amax;
    if (mass_only) {
        for (int s = 0; s < nloop; s++)
            for (int i = 0; i < n; i++) m[i] = (m[i] + a[i]) - a[i + 1];
        return nloop;
    }
    double *f = malloc(sizeof(double) * 4 * (n + 1) * nt);
    double *mi = malloc(sizeof(double) * n);
    for (int s = 0; s < nloop; s++) {
        for (int i = 0; i < n; i++) mi[i] = 1.0 / m[i];
        for (int t = 0; t < nt; t++) {
            double *ff = f + (4 * t + 0) * (n + 1), *pf = f + (4 * t + 1) * (n + 1);
            double *fy = f + (4 * t + 2) * (n + 1), *fz = f + (4 * t + 3) * (n + 1);
            double *rm = q[0 * nt + t], *rxm = q[1 * nt + t], *rym = q[2 * nt + t], *rzm = q[3 * nt + t];
            for (int k = 0; k <= n; k++) {
                int up = a[k] >= 0.0 ? (k == 0 ? n - 1 : k - 1) : (k == n ? 0 : k);
                double alpha = a[k] * mi[up];
                flux4(a[k], alpha, rm[up], rxm[up], rym[up], rzm[up], &ff[k], &pf[k], &fy[k], &fz[k]);
            }
            ff[0] = ff[n]; /* the periodic seam */
            pf[0] = pf[n];
            fy[0] = fy[n];
            fz[0] = fz[n];
            for (int i = 0; i < n; i++) {
                double mo = m[i];
                double mn = (mo + a[i]) - a[i + 1];
                double rmn = rm[i] - (ff[i + 1] - ff[i]);
                double rxn = slope_update(rxm[i], pf[i], pf[i + 1], a[i], a[i + 1], rmn, ff[i], ff[i + 1], mo, mn);
                if (limits) rxn = limit(rxn, rmn);
                rm[i] = rmn;
                rxm[i] = rxn;
                rym[i] = rym[i] - (fy[i + 1] - fy[i]);
                rzm[i] = rzm[i] - (fz[i + 1] - fz[i]);
            }
        }
        for (int i = 0; i < n; i++) m[i] = (m[i] + a[i]) - a[i + 1];
    }
    free(f);
    free(mi);
    return nloop;
}

/* advect_x / advect_x_reduced / zoom _dynamu_region1 / cfl.dynamum on every (j, l) row
 * (kernels.py:129-166, redgrid.py:93-110, zoom/advect.py:237-275, cfl.py:140-167,
 * zoom/check_cfl.py:94-110).  clust[j] > 1 marks a reduced latitude.  halo: write the periodic
 * halos as the zoom region-1 body does.  Returns 0, or 1 when a row exceeded its cap. */
int or_advect_x(const ov *m, const ov *rm, const ov *rxm, const ov *rym, const ov *rzm, const ov *am,
                const int32_t *clust, int halo, int js, int je, int limits, int max_nloop, int mass_only,
                int32_t *nloop_out, double *amax_out) {
    const int im = (int)m->n[0], jm = (int)m->n[1], lm = (int)m->n[2];
    const int nt = mass_only ? 0 : (int)rm->n[3];
    const ov *qv[4] = {rm, rxm, rym, rzm};
    const int W = im + 2;
    double *mr = malloc(sizeof(double) * W);
    double *qr = malloc(sizeof(double) * W * (4 * nt + 1));
    double **qp = malloc(sizeof(double *) * (4 * nt + 1));
    double *a = malloc(sizeof(double) * W);
    int failed = 0;
    for (int w = 0; w < 4; w++)
        for (int t = 0; t < nt; t++) qp[w * nt + t] = qr + (size_t)(w * nt + t) * W;
    for (int j = 0; j < jm; j++) {
        const int c = clust ? clust[j] : 1;
        const int n = im / c;
        const int in_scope = (j + 1 >= js) && (j + 1 <= je);
        for (int l = 0; l < lm; l++) {
            /* uni2red (redgrid.py:56-67): seqsum of each cluster, in order */
            for (int k = 0; k < n; k++) {
                double acc = A3(m, k * c, j, l);
                for (int cc = 1; cc < c; cc++) acc = acc + A3(m, k * c + cc, j, l);
                mr[k] = acc;
                for (int w = 0; w < 4; w++)
                    for (int t = 0; t < nt; t++) {
                        double s = A4(qv[w], k * c, j, l, t);
                        for (int cc = 1; cc < c; cc++) s = s + A4(qv[w], k * c + cc, j, l, t);
                        qp[w * nt + t][k] = s;
                    }
            }
            /* uni2red_mf (redgrid.py:70-76) */
            for (int k = 1; k <= n; k++) a[k] = A3(am, k * c, j, l);
            a[0] = c > 1 ? a[n] : A3(am, 0, j, l);
            double amax = 0.0;
            int nl = x_row(mr, qp, nt, a, n, mass_only, limits, max_nloop - 1, &amax);
            if (nloop_out) nloop_out[j * lm + l] = nl;
            if (amax_out) amax_out[j * lm + l] = amax;
            if (nl == 0) {
                failed = 1;
                continue;
            }
            if (!clust) /* "restore old am": a * nloop (with a reduced grid am is kept whole) */
                for (int k = 0; k <= n; k++) A3(am, k, j, l) = a[k] * (double)nl;
            if (c == 1) {
                for (int i = 0; i < n; i++) {
                    A3(m, i, j, l) = mr[i];
                    for (int w = 0; w < 4; w++)
                        for (int t = 0; t < nt; t++) A4(qv[w], i, j, l, t) = qp[w * nt + t][i];
                }
                if (halo && in_scope) { /* q(0) = q(im), q(im+1) = q(1) */
                    A3(m, -1, j, l) = mr[n - 1];
                    A3(m, n, j, l) = mr[0];
                    for (int w = 0; w < 4; w++)
                        for (int t = 0; t < nt; t++) {
                            A4(qv[w], -1, j, l, t) = qp[w * nt + t][n - 1];
                            A4(qv[w], n, j, l, t) = qp[w * nt + t][0];
                        }
                }
            } else {
                /* red2uni (redgrid.py:79-90) with m_uni advanced by the untouched am */
                for (int i = 0; i < im; i++) {
                    int k = i / c;
                    double mun = (A3(m, i, j, l) + A3(am, i, j, l)) - A3(am, i + 1, j, l);
                    double sc = mun / mr[k];
                    for (int w = 0; w < 4; w++)
                        for (int t = 0; t < nt; t++) A4(qv[w], i, j, l, t) = sc * qp[w * nt + t][k];
                    A3(m, i, j, l) = mun;
                }
                /* zoom/advect.py:266-272: q(0) = q(im) on every reduced row (the CFL body only on
                 * its rows js..je, zoom/check_cfl.py:106-109) */
                if (halo && (!mass_only || in_scope)) {
                    A3(m, -1, j, l) = A3(m, im - 1, j, l);
                    for (int w = 0; w < 4; w++)
                        for (int t = 0; t < nt; t++) A4(qv[w], -1, j, l, t) = A4(qv[w], im - 1, j, l, t);
                }
            }
        }
    }
    free(mr);
    free(qr);
    free(qp);
    free(a);
    return failed;
}

/* ------------------------------------------------------------------ y (dynamv)
 * One layer (kernels.py:246-291): the layer's nloop from subcycles (ops.py:315-341) over all its
 * columns, the whole layer's faces rescaled in place, the sub-steps with the pole faces, and
 * b * nloop.  full: the halo'd bm whose layer faces outside (1:im, 1:jm+1) are rescaled alike
 * (zoom/advect.py:212-226).  mass_only: dynamvm (cfl.py:170-183).  Returns 0, 1 (cap), 2 (halo). */
int or_advect_y(const ov *m, const ov *rm, const ov *rxm, const ov *rym, const ov *rzm, const ov *bm, const ov *full,
                int full_l0, int limits, int max_nloop, int mass_only, int32_t *nloop_out) {
    const int im = (int)m->n[0], jm = (int)m->n[1], lm = (int)m->n[2];
    const int nt = mass_only ? 0 : (int)rm->n[3];
    const int nmax = mass_only ? max_nloop : max_nloop - 1;
    const ov *qv[4] = {rm, rxm, rym, rzm};
    if (!mass_only)
        for (int i = 0; i < im; i++)
            for (int l = 0; l < lm; l++)
                if (A3(bm, i, 0, l) != 0.0 || A3(bm, i, jm, l) != 0.0) return 2;
    double *mx = malloc(sizeof(double) * (size_t)im * jm);
    double *col = malloc(sizeof(double) * (jm + 1) * (3 + 8 * (nt > 0 ? nt : 1)));
    int status = 0;
    for (int l = 0; l < lm; l++) {
        if (!mass_only && limits)
            for (int i = 0; i < im; i++)
                for (int j = 0; j < jm; j++)
                    for (int t = 0; t < nt; t++) A4(rym, i, j, l, t) = limit(A4(rym, i, j, l, t), A4(rm, i, j, l, t));
        int nloop = 1;
        for (;;) {
            int ok = 1;
            for (int i = 0; i < im; i++)
                for (int j = 0; j < jm; j++) mx[i * jm + j] = A3(m, i, j, l);
            for (int s = 0; s < nloop && ok; s++) {
                for (int i = 0; i < im && ok; i++)
                    for (int k = 1; k < jm; k++) {
                        double b = A3(bm, i, k, l);
                        double mu = b >= 0.0 ? mx[i * jm + k - 1] : mx[i * jm + k];
                        if (!(fabs(b / mu) < 1.0)) {
                            ok = 0;
                            break;
                        }
                    }
                if (!ok) break;
                for (int i = 0; i < im; i++) {
                    double prev_lo = A3(bm, i, 0, l);
                    for (int j = 0; j < jm; j++) {
                        double hi = A3(bm, i, j + 1, l);
                        mx[i * jm + j] = (mx[i * jm + j] + prev_lo) - hi;
                        prev_lo = hi;
                    }
                }
            }
            if (ok) break;
            nloop++;
            for (int i = 0; i < im; i++) /* progressive: the whole layer, in place */
                for (int k = 0; k <= jm; k++) A3(bm, i, k, l) = A3(bm, i, k, l) * (double)(nloop - 1) / (double)nloop;
            if (nloop > nmax) break;
        }
        if (nloop_out) nloop_out[l] = nloop;
        if (nloop > nmax) {
            status = 1;
            break;
        }
        if (full && !mass_only && nloop > 1) {
            const int lf = l + full_l0;
            for (int64_t fi = 0; fi < full->n[0]; fi++)
                for (int64_t fj = 0; fj < full->n[1]; fj++) {
                    int inside = fi >= 1 && fi <= im && fj >= 1 && fj <= jm + 1;
                    if (inside) continue;
                    A3(full, fi, fj, lf) = rescaled(A3(full, fi, fj, lf), nloop) * (double)nloop;
                }
        }
        if (mass_only) { /* dynamvm: nloop = 1 advance, b * 1 */
            for (int i = 0; i < im; i++)
                for (int j = 0; j < jm; j++)
                    A3(m, i, j, l) = (A3(m, i, j, l) + A3(bm, i, j, l)) - A3(bm, i, j + 1, l);
            continue;
        }
        for (int i = 0; i < im; i++) {
            double *b = col;
            double *F = b + (jm + 1); /* [4][nt][jm+1]: f, pf, fx, fz */
            for (int k = 0; k <= jm; k++) b[k] = A3(bm, i, k, l);
            for (int s = 0; s < nloop; s++) {
                for (int w = 0; w < 4; w++)
                    for (int t = 0; t < nt; t++) F[(w * nt + t) * (jm + 1) + 0] = F[(w * nt + t) * (jm + 1) + jm] = 0.0;
                for (int k = 1; k < jm; k++) {
                    int up = b[k] >= 0.0 ? k - 1 : k;
                    double beta = b[k] / A3(m, i, up, l);
                    for (int t = 0; t < nt; t++) {
                        double f, pf, fx, fz;
                        flux4(b[k], beta, A4(rm, i, up, l, t), A4(rym, i, up, l, t), A4(rxm, i, up, l, t),
                              A4(rzm, i, up, l, t), &f, &pf, &fx, &fz);
                        if (k == 1 && b[k] >= 0.0) { /* out of the south pole cell: no slope */
                            f = beta * A4(rm, i, 0, l, t);
                            pf = (-3.0 * b[k]) * f;
                            fx = 0.0;
                            fz = beta * A4(rzm, i, 0, l, t);
                        }
                        if (k == jm - 1 && b[k] < 0.0) {
                            f = beta * A4(rm, i, jm - 1, l, t);
                            pf = (-3.0 * b[k]) * f;
                            fx = 0.0;
                            fz = beta * A4(rzm, i, jm - 1, l, t);
                        }
                        F[(0 * nt + t) * (jm + 1) + k] = f;
                        F[(1 * nt + t) * (jm + 1) + k] = pf;
                        F[(2 * nt + t) * (jm + 1) + k] = fx;
                        F[(3 * nt + t) * (jm + 1) + k] = fz;
                    }
                }
                for (int j = 0; j < jm; j++) {
                    double mo = A3(m, i, j, l);
                    double mn = (mo + b[j]) - b[j + 1];
                    double inv = 1.0 / mn;
                    double conv = b[j] - b[j + 1], mean = 3.0 * (b[j] + b[j + 1]), m3 = 3.0 * mo;
                    for (int t = 0; t < nt; t++) {
                        const double *f = F + (0 * nt + t) * (jm + 1), *pf = F + (1 * nt + t) * (jm + 1);
                        const double *fx = F + (2 * nt + t) * (jm + 1), *fz = F + (3 * nt + t) * (jm + 1);
                        double rmn = A4(rm, i, j, l, t) - (f[j + 1] - f[j]);
                        double ry = A4(rym, i, j, l, t);
                        double ryn = ry + ((pf[j] - pf[j + 1]) - conv * ry + mean * rmn - m3 * (f[j] + f[j + 1])) * inv;
                        if (limits) ryn = limit(ryn, rmn);
                        double rxn = A4(rxm, i, j, l, t) - (fx[j + 1] - fx[j]);
                        A4(rzm, i, j, l, t) = A4(rzm, i, j, l, t) - (fz[j + 1] - fz[j]);
                        A4(rm, i, j, l, t) = rmn;
                        if (j != 0 && j != jm - 1) {
                            A4(rym, i, j, l, t) = ryn;
                            A4(rxm, i, j, l, t) = rxn;
                        }
                    }
                    A3(m, i, j, l) = mn;
                }
            }
        }
        for (int i = 0; i < im; i++)
            for (int k = 0; k <= jm; k++) A3(bm, i, k, l) = A3(bm, i, k, l) * (double)nloop;
    }
    free(mx);
    free(col);
    (void)qv;
    return status;
}

/* ------------------------------------------------------------------ z (dynamw)
 * kernels.py:295-346: the region-wide n_advz from subcycles with `fresh` (cm / n), the trial mass
 * advanced on the scope only (zoom/advect.py:415-441 column_trial; the whole region for region
 * 1), then n_advz sub-steps on the scope with cm / n_advz; cm restored exactly.
 * mass_only: dynamwm (cfl.py:186-194, zoom/check_cfl.py:206-216).  Returns 0, 1 (cap), 2 (halo). */
int or_advect_z(const ov *m, const ov *rm, const ov *rxm, const ov *rym, const ov *rzm, const ov *cm, int si0,
                int si1, int sj0, int sj1, int limits, int iter_limit, int mass_only, int32_t *n_out) {
    const int im = (int)m->n[0], jm = (int)m->n[1], lm = (int)m->n[2];
    const int nt = mass_only ? 0 : (int)rm->n[3];
    if (!mass_only)
        for (int i = 0; i < im; i++)
            for (int j = 0; j < jm; j++)
                if (A3(cm, i, j, 0) != 0.0 || A3(cm, i, j, lm) != 0.0) return 2;
    if (!mass_only && limits)
        for (int i = si0; i < si1; i++)
            for (int j = sj0; j < sj1; j++)
                for (int l = 0; l < lm; l++)
                    for (int t = 0; t < nt; t++) A4(rzm, i, j, l, t) = limit(A4(rzm, i, j, l, t), A4(rm, i, j, l, t));
    double *mx = malloc(sizeof(double) * (size_t)im * jm * lm);
    int n = 1;
    for (;;) {
        int ok = 1;
        for (int i = 0; i < im; i++)
            for (int j = 0; j < jm; j++)
                for (int l = 0; l < lm; l++) mx[((size_t)i * jm + j) * lm + l] = A3(m, i, j, l);
        for (int s = 0; s < n && ok; s++) {
            for (int i = 0; i < im && ok; i++)
                for (int j = 0; j < jm && ok; j++)
                    for (int k = 1; k < lm; k++) {
                        double c = A3(cm, i, j, k) / (double)n;
                        double *col = mx + ((size_t)i * jm + j) * lm;
                        double mu = c >= 0.0 ? col[k - 1] : col[k];
                        if (!(fabs(c / mu) < 1.0)) {
                            ok = 0;
                            break;
                        }
                    }
            if (!ok) break;
            for (int i = si0; i < si1; i++)
                for (int j = sj0; j < sj1; j++) {
                    double *col = mx + ((size_t)i * jm + j) * lm;
                    for (int l = 0; l < lm; l++)
                        col[l] = (col[l] + A3(cm, i, j, l) / (double)n) - A3(cm, i, j, l + 1) / (double)n;
                }
        }
        if (ok) break;
        n++;
        if (n > iter_limit) {
            free(mx);
            if (n_out) *n_out = n;
            return 1;
        }
    }
    if (n_out) *n_out = n;
    if (mass_only) {
        for (int i = si0; i < si1; i++)
            for (int j = sj0; j < sj1; j++)
                for (int l = 0; l < lm; l++) A3(m, i, j, l) = mx[((size_t)i * jm + j) * lm + l];
        free(mx);
        return 0;
    }
    free(mx);
    double *c = malloc(sizeof(double) * (lm + 1) * (1 + 4 * (nt > 0 ? nt : 1)));
    double *F = c + (lm + 1);
    for (int i = si0; i < si1; i++)
        for (int j = sj0; j < sj1; j++) {
            for (int k = 0; k <= lm; k++) c[k] = A3(cm, i, j, k) / (double)n;
            for (int s = 0; s < n; s++) {
                for (int w = 0; w < 4; w++)
                    for (int t = 0; t < nt; t++) F[(w * nt + t) * (lm + 1) + 0] = F[(w * nt + t) * (lm + 1) + lm] = 0.0;
                for (int k = 1; k < lm; k++) {
                    int up = c[k] >= 0.0 ? k - 1 : k;
                    double gamma = c[k] / A3(m, i, j, up);
                    for (int t = 0; t < nt; t++) {
                        double f, pf, fx, fy;
                        flux4(c[k], gamma, A4(rm, i, j, up, t), A4(rzm, i, j, up, t), A4(rxm, i, j, up, t),
                              A4(rym, i, j, up, t), &f, &pf, &fx, &fy);
                        F[(0 * nt + t) * (lm + 1) + k] = f;
                        F[(1 * nt + t) * (lm + 1) + k] = pf;
                        F[(2 * nt + t) * (lm + 1) + k] = fx;
                        F[(3 * nt + t) * (lm + 1) + k] = fy;
                    }
                }
                for (int l = 0; l < lm; l++) {
                    double mo = A3(m, i, j, l);
                    double mn = (mo + c[l]) - c[l + 1];
                    for (int t = 0; t < nt; t++) {
                        const double *f = F + (0 * nt + t) * (lm + 1), *pf = F + (1 * nt + t) * (lm + 1);
                        const double *fx = F + (2 * nt + t) * (lm + 1), *fy = F + (3 * nt + t) * (lm + 1);
                        double rmn = (A4(rm, i, j, l, t) + f[l]) - f[l + 1];
                        double rzn = slope_update(A4(rzm, i, j, l, t), pf[l], pf[l + 1], c[l], c[l + 1], rmn, f[l],
                                                  f[l + 1], mo, mn);
                        if (limits) rzn = limit(rzn, rmn);
                        A4(rm, i, j, l, t) = rmn;
                        A4(rzm, i, j, l, t) = rzn;
                        A4(rxm, i, j, l, t) = (A4(rxm, i, j, l, t) + fx[l]) - fx[l + 1];
                        A4(rym, i, j, l, t) = (A4(rym, i, j, l, t) + fy[l]) - fy[l + 1];
                    }
                    A3(m, i, j, l) = mn;
                }
            }
        }
    free(c);
    return 0;
}

/* ------------------------------------------------------------------ dynam0, m2phlb
 * kernels.py:102-125 fluxes_from_meteo (convergence ops.py:273-274, pit a seqsum bottom-up). */
void or_fluxes_from_meteo(const ov *pu, const ov *pv, const double *bt, double dt, const ov *am, const ov *bm,
                          const ov *cm) {
    const int im = (int)pv->n[0], jm = (int)pu->n[1], lm = (int)pu->n[2];
    double *conv = malloc(sizeof(double) * lm);
    for (int i = 0; i <= im; i++)
        for (int j = 0; j < jm; j++)
            for (int l = 0; l < lm; l++) A3(am, i, j, l) = dt * A3(pu, i, j, l);
    for (int i = 0; i < im; i++)
        for (int j = 0; j <= jm; j++)
            for (int l = 0; l < lm; l++) A3(bm, i, j, l) = dt * A3(pv, i, j, l);
    for (int i = 0; i < im; i++)
        for (int j = 0; j < jm; j++) {
            for (int l = 0; l < lm; l++)
                conv[l] = A3(pu, i, j, l) - A3(pu, i + 1, j, l) + A3(pv, i, j, l) - A3(pv, i, j + 1, l);
            double pit = conv[0];
            for (int l = 1; l < lm; l++) pit = pit + conv[l];
            A3(cm, i, j, 0) = 0.0;
            A3(cm, i, j, lm) = 0.0;
            double sd = 0.0;
            for (int l = lm - 1; l >= 1; l--) {
                if (l == lm - 1)
                    sd = conv[l] - (bt[l] - bt[l + 1]) * pit;
                else
                    sd = sd + conv[l] - (bt[l] - bt[l + 1]) * pit;
                A3(cm, i, j, l) = -dt * sd;
            }
        }
    free(conv);
}

/* zoom/massflow.py:24-56 m2phlb1 / m2phlb: p = seqsum_l(m) g / dxyp; a child's ring rescaled to the
 * parent cell's area; sp(i, j) = p; phlb = at + bt p.  sp is (im, jm). */
void or_m2phlb(const ov *m, const ov *sp, const ov *phlb, const double *dxyp, const double *at, const double *bt,
               int xr, int yr, int jbeg, const double *dxyp_parent) {
    const double grav = 9.80665;
    const int im = (int)m->n[0], jm = (int)m->n[1], lm = (int)m->n[2];
    for (int i = 0; i < im; i++)
        for (int j = 0; j < jm; j++) {
            double s = A3(m, i, j, 0);
            for (int l = 1; l < lm; l++) s = s + A3(m, i, j, l);
            double p = s * grav / dxyp[j];
            if (xr > 0) {
                int fi = i + 1, fj = j + 1;
                int interior = xr < fi && fi < im - xr + 1 && yr < fj && fj < jm - yr + 1;
                if (!interior) p = p * dxyp[j] * (double)xr * (double)yr / dxyp_parent[jbeg + (fj - 1) / yr - 1];
            }
            sp->p[i * sp->s[0] + j * sp->s[1]] = p;
            for (int l = 0; l <= lm; l++) A3(phlb, i, j, l) = at[l] + bt[l] * p;
        }
}
