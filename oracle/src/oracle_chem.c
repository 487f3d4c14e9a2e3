/*
 * ORACLE -- test infrastructure, not the product.  The CH4 `c` operator's loss rates and decay
 * per cell, scalar C in the reference's evaluation order: pydyn chem.py:59-88 (rebin_many),
 * :91-98 (strat_edges), :101-104 (tropopause), :107-111 (_column), :114-150 (loss_rates),
 * :168-170 (decay).  exp / pow / cos are the package's gbmath (the functions pydyn is pointed at
 * through ops.use_libm when the golden fixtures are made).
 *
 * rebin_many sums, per output layer and in input order from +0.0, data * thickness over the
 * input layers first..last-1 whose overlap is positive; the other terms it adds are +0.0, which
 * leave a sum that cannot be -0.0 unchanged, so they are skipped here.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>

#include "../../pydyn_gb300/csrc/gbmath.h"

typedef struct {
    double *p;
    int64_t n[4];
    int64_t s[4];
} ov;

#define A1(v, i) ((v)->p[(int64_t)(i) * (v)->s[0]])
#define A2(v, i, j) ((v)->p[(int64_t)(i) * (v)->s[0] + (int64_t)(j) * (v)->s[1]])
#define A3(v, i, j, l) ((v)->p[(int64_t)(i) * (v)->s[0] + (int64_t)(j) * (v)->s[1] + (int64_t)(l) * (v)->s[2]])
#define A4(v, i, j, l, k) \
    ((v)->p[(int64_t)(i) * (v)->s[0] + (int64_t)(j) * (v)->s[1] + (int64_t)(l) * (v)->s[2] + (int64_t)(k) * (v)->s[3]])

static double npmax(double a, double b) { return isnan(a) ? a : (isnan(b) ? b : (a > b ? a : b)); }
static double npmin(double a, double b) { return isnan(a) ? a : (isnan(b) ? b : (a < b ? a : b)); }

/* The layer mean over [top, bot] of data given on the descending edges ip[0..nip]. */
static double rebin_layer(const double *ip, int nip, const double *data, int dstride, double bot, double top) {
    int first = 0, last = 0;
    for (int k = 0; k < nip; k++) {
        first += ip[k + 1] >= bot;
        last += ip[k] > top;
    }
    double overlap = 0.0;
    for (int k = first; k < last; k++) {
        double thickness = npmin(bot, ip[k]) - npmax(top, ip[k + 1]);
        if (thickness > 0.0) overlap = overlap + data[(int64_t)k * dstride] * thickness;
    }
    double width = bot - top;
    return width > 0.0 ? overlap / width : overlap;
}

static int descending(const double *x, int n) {
    for (int k = 0; k + 1 < n; k++)
        if (!(x[k + 1] - x[k] < 0.0)) return 0;
    return 1;
}

/* loss_rates + decay of every cell of a region: temper, oh_3d (im, jm, lm); phlb (im, jm, lm+1);
 * lat (jm); strat_press, strat_oh, strat_cl, strat_od (jm, ns); pl_trop, cl_trop (im, jm, ntrop)
 * or NULL; soil (im, jm) or NULL; oh_factor (im) or NULL, a per-longitude multiplier of oh_3d.
 * Outputs loss (im, jm, lm, 4) and decay (im, jm, lm), either may be NULL.  Returns 0, or 4
 * when a column's levels are not strictly descending (chem.py:47-49). */
int or_loss_rates(const ov *temper, const ov *phlb, const double *lat, const ov *strat_press, const ov *strat_oh,
                  const ov *strat_cl, const ov *strat_od, const ov *oh_3d, const ov *pl_trop, const ov *cl_trop,
                  const ov *soil, const double *oh_factor, double oh_scale, double cl_scale, double o1d_scale,
                  double soil_rate, double dt, const ov *loss, const ov *decay) {
    const int im = (int)temper->n[0], jm = (int)temper->n[1], lm = (int)temper->n[2];
    const int ns = (int)strat_press->n[1];
    const int ntrop = pl_trop ? (int)pl_trop->n[2] : 0;
    int rc = 0;
#pragma omp parallel
    {  /* latitudes are independent: each thread its own work arrays */
    double *edges = malloc(sizeof(double) * (ns + 1));
    double *tedges = malloc(sizeof(double) * (ntrop + 2));
    double *col = malloc(sizeof(double) * (lm + 1));
#pragma omp for schedule(dynamic, 1) reduction(| : rc)
    for (int j = 0; j < jm; j++) {
        /* strat_edges: midpoints, a half layer below the first, 0 above the last; hPa -> Pa */
        const double p0 = A2(strat_press, j, 0), p1 = ns > 1 ? A2(strat_press, j, 1) : 0.0;
        edges[0] = (p0 + 0.5 * (p0 - p1)) * 100.0;
        for (int k = 1; k < ns; k++) edges[k] = ((A2(strat_press, j, k - 1) + A2(strat_press, j, k)) / 2.0) * 100.0;
        edges[ns] = 0.0 * 100.0;
        if (!descending(edges, ns + 1)) {
            rc |= 4;
            continue;
        }
        const double c = gbm_cos(lat[j]);
        const double trop = 30000.0 - 21500.0 * (c * c);
        for (int i = 0; i < im && !rc; i++) {
            for (int l = 0; l <= lm; l++) col[l] = A3(phlb, i, j, l);
            if (!descending(col, lm + 1)) {
                rc |= 4;
                break;
            }
            if (ntrop) {
                for (int k = 0; k < ntrop; k++) tedges[k] = A3(pl_trop, i, j, k);
                tedges[ntrop] = 0.0;
                if (!descending(tedges, ntrop + 1)) {
                    rc |= 4;
                    break;
                }
            }
            for (int l = 0; l < lm; l++) {
                const double bot = col[l], top = col[l + 1];
                const int below = bot > edges[0];
                const double s_oh = below ? A2(strat_oh, j, 0)
                                          : rebin_layer(edges, ns, &A2(strat_oh, j, 0), (int)strat_oh->s[1], bot, top);
                const double s_cl = below ? A2(strat_cl, j, 0)
                                          : rebin_layer(edges, ns, &A2(strat_cl, j, 0), (int)strat_cl->s[1], bot, top);
                const double s_od = below ? A2(strat_od, j, 0)
                                          : rebin_layer(edges, ns, &A2(strat_od, j, 0), (int)strat_od->s[1], bot, top);
                const double T = A3(temper, i, j, l);
                double trop_cl = 0.0;
                if (ntrop) {
                    double v = bot > tedges[0] ? A3(cl_trop, i, j, 0)
                                               : rebin_layer(tedges, ntrop, &A3(cl_trop, i, j, 0), (int)cl_trop->s[2],
                                                             bot, top);
                    const double krate = (2.36e-12 * gbm_pow(T / 298.0, 1.37)) * gbm_exp(-939.0 / T);
                    trop_cl = (v * krate) * cl_scale;
                }
                double oh = A3(oh_3d, i, j, l);
                if (oh_factor) oh = oh * oh_factor[i];
                const double krate_oh = 2.45e-12 * gbm_exp(-1775.0 / T);
                const double spiv = (krate_oh * oh) * oh_scale;
                const int strat = bot < trop;
                const double L0 = strat ? s_oh : spiv;
                const double L1 = strat ? s_cl : s_cl + trop_cl;
                const double L2 = s_od * o1d_scale;
                const double L3 = (soil && l == 0) ? -(soil_rate * A2(soil, i, j)) : 0.0;
                if (loss) {
                    A4(loss, i, j, l, 0) = L0;
                    A4(loss, i, j, l, 1) = L1;
                    A4(loss, i, j, l, 2) = L2;
                    A4(loss, i, j, l, 3) = L3;
                }
                if (decay) A3(decay, i, j, l) = gbm_exp(-((((L0 + L1) + L2) + L3) * dt));
            }
        }
    }
    free(edges);
    free(tedges);
    free(col);
    }
    return rc;
}
