// dynam0 (k_fluxes_ambm elementwise, k_fluxes_cm the columns' serial sums) and m2phlb: the
// per-half-step mass fluxes from the meteo fluxes, and the surface
// pressure / half-level pressures from the column mass.
// Reference: pydyn kernels.py:102-125 (fluxes_from_meteo), ops.py:273-274 (convergence),
// zoom/massflow.py:24-56 (m2phlb1, m2phlb), balance.py:222-226.
#include "gb_common.cuh"

namespace {

constexpr double GRAV = 9.80665;  // Binas, balance.py

__device__ __forceinline__ double &AT(const DV &v, int64_t i, int64_t j, int64_t l) {
    return v.p[i * v.s0 + j * v.s1 + l * v.s2];
}

// The column loops read their inputs B levels at a time into registers before using them, so
// that a batch's loads are in flight together (a thread per column: few warps hide little latency).
constexpr int B = 8;

// the convergence of cell (i, j, l): pu(i-1) - pu(i) + pv(j) - pv(j+1), left to right
__device__ __forceinline__ double convergence(const DV &pu, const DV &pv, int i, int j, int l) {
    return ((AT(pu, i, j, l) - AT(pu, i + 1, j, l)) + AT(pv, i, j, l)) - AT(pv, i, j + 1, l);
}

// One thread per (i, j, l) of the face grid [0, im] x [0, jm] x lm: am = dt pu (j < jm) and
// bm = dt pv (i < im), element by element.
__global__ void k_fluxes_ambm(DV pu, DV pv, double dt, DV am, DV bm, int im, int jm, int lm) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)(im + 1) * (jm + 1) * lm) return;
    const int l = (int)(t % lm);
    const int64_t c = t / lm;
    const int i = (int)(c / (jm + 1)), j = (int)(c % (jm + 1));
    if (j < jm) AT(am, i, j, l) = dt * AT(pu, i, j, l);
    if (i < im) AT(bm, i, j, l) = dt * AT(pv, i, j, l);
}

// One thread per cell column (i, j) of [0, im) x [0, jm): cm from the convergence distributed by
// the hybrid b (the column's serial sums).
__global__ void k_fluxes_cm(DV pu, DV pv, const double *bt, double dt, DV cm, int im, int jm, int lm) {
    int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= (int64_t)im * jm) return;
    const int i = (int)(k / jm), j = (int)(k % jm);
    {
        // pit = the column sum of the convergence, bottom-up
        double pit = 0.0;
        for (int l0 = 0; l0 < lm; l0 += B) {
            double c[B];
#pragma unroll
            for (int u = 0; u < B; ++u)
                if (l0 + u < lm) c[u] = convergence(pu, pv, i, j, l0 + u);
#pragma unroll
            for (int u = 0; u < B; ++u)
                if (l0 + u < lm) pit = (l0 + u == 0) ? c[u] : pit + c[u];
        }
        // sd(l) from the top down; cm = -dt sd on the interior interfaces
        double sd = 0.0;
        AT(cm, i, j, lm) = 0.0;
        for (int l0 = lm - 1; l0 >= 1; l0 -= B) {
            double c[B];
#pragma unroll
            for (int u = 0; u < B; ++u)
                if (l0 - u >= 1) c[u] = convergence(pu, pv, i, j, l0 - u);
#pragma unroll
            for (int u = 0; u < B; ++u) {
                const int l = l0 - u;
                if (l < 1) break;
                if (l == lm - 1)
                    sd = c[u] - (bt[lm - 1] - bt[lm]) * pit;
                else
                    sd = (sd + c[u]) - (bt[l] - bt[l + 1]) * pit;
                AT(cm, i, j, l) = (-dt) * sd;
            }
        }
        AT(cm, i, j, 0) = 0.0;
    }
}

__global__ void k_m2phlb(DV m, DV sp, DV phlb, const double *dxyp, const double *at, const double *bt, int im,
                         int jm, int lm, int xr, int yr, int jbeg, const double *dxyp_parent) {
    int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= (int64_t)im * jm) return;
    const int i = (int)(k / jm), j = (int)(k % jm);
    double acc = AT(m, i, j, 0);
    for (int l = 1; l < lm; ++l) acc = acc + AT(m, i, j, l);
    double p = div_ip(acc * GRAV, dxyp[j]);
    if (xr > 0) {
        // the child's ring: rescaled to the parent cell's area (Fortran i, j from 1)
        const int fi = i + 1, fj = j + 1;
        const bool interior = (xr < fi && fi < im - xr + 1) && (yr < fj && fj < jm - yr + 1);
        if (!interior) {
            const int jpar = jbeg + (fj - 1) / yr;  // 1-based parent row
            p = div_ip(((p * dxyp[j]) * (double)xr) * (double)yr, dxyp_parent[jpar - 1]);
        }
    }
    sp.p[i * sp.s0 + j * sp.s1] = p;
    for (int l = 0; l <= lm; ++l) AT(phlb, i, j, l) = at[l] + bt[l] * p;
}

}  // namespace

extern "C" int gb_fluxes_from_meteo(gb_ctx *ctx, const gb_view *pu, const gb_view *pv, const double *bt, double dt,
                                    const gb_view *am, const gb_view *bm, const gb_view *cm) {
    if (!ctx || !pu || !pv || !bt || !am || !bm || !cm) return GB_EARG;
    const int im = (int)pv->n[0], jm = (int)pu->n[1], lm = (int)pu->n[2];
    if (pu->n[0] != im + 1 || pv->n[1] != jm + 1 || cm->n[2] != lm + 1) {
        gb_set_error("gb_fluxes_from_meteo: inconsistent shapes");
        return GB_EARG;
    }
    const int64_t faces = (int64_t)(im + 1) * (jm + 1) * lm, cols = (int64_t)im * jm;
    k_fluxes_ambm<<<(int)((faces + 255) / 256), 256, 0, ctx->stream>>>(dv(pu), dv(pv), dt, dv(am), dv(bm), im, jm, lm);
    if (int rc = gb_after_launch(ctx, "fluxes_ambm")) return rc;
    k_fluxes_cm<<<(int)((cols + 63) / 64), 64, 0, ctx->stream>>>(dv(pu), dv(pv), bt, dt, dv(cm), im, jm, lm);
    return gb_after_launch(ctx, "fluxes_cm");
}

extern "C" int gb_m2phlb(gb_ctx *ctx, const gb_view *m, const gb_view *sp, const gb_view *phlb, const double *dxyp,
                         const double *at, const double *bt, int ring_xr, int ring_yr, int jbeg,
                         const double *dxyp_parent) {
    if (!ctx || !m || !sp || !phlb || !dxyp || !at || !bt) return GB_EARG;
    const int im = (int)m->n[0], jm = (int)m->n[1], lm = (int)m->n[2];
    int64_t total = (int64_t)im * jm;
    k_m2phlb<<<(int)((total + 127) / 128), 128, 0, ctx->stream>>>(dv(m), dv(sp), dv(phlb), dxyp, at, bt, im, jm, lm,
                                                                  ring_xr, ring_yr, jbeg, dxyp_parent);
    return gb_after_launch(ctx, "m2phlb");
}

// ------------------------------------------------------------------ the device math, for tests
#include "gbmath.h"

namespace {
__global__ void k_math_eval(int op, const double *x, const double *y, double *out, int64_t n) {
    int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    double r;
    switch (op) {
        case 0: r = gbm_exp(x[k]); break;
        case 1: r = gbm_log(x[k]); break;
        case 2: r = gbm_pow(x[k], y[k]); break;
        case 3: r = gbm_cos(x[k]); break;
        case 4: r = gbm_sin(x[k]); break;
        case 5: r = div_by_recip(x[k], y[k], recip_for(y[k])); break;
        case 7: r = div_ip(x[k], y[k]); break;
        case 8: r = add_ip(x[k], y[k]); break;
        case 9: r = sub_ip(x[k], y[k]); break;
        case 10: r = sqrt_ip(x[k]); break;
        case 11: r = sqrt(x[k]); break;
        case 12: r = blend01(1.0, x[k], y[k]); break;  // 1 x + (1 - 1) y
        case 13: r = blend01(0.0, x[k], y[k]); break;  // 0 x + (1 - 0) y
        case 14: r = mul01(0.0, x[k]); break;          // 0 x
        case 15: r = jqif_ip(x[k], y[k]); break;
        default: r = x[k] / y[k]; break;
    }
    out[k] = r;
}
}  // namespace

extern "C" int gb_math_eval(gb_ctx *ctx, int op, const double *x, const double *y, double *out, int64_t n) {
    if (!ctx || !x || !y || !out || n < 0) return GB_EARG;
    if (n == 0) return GB_OK;
    k_math_eval<<<(int)((n + 127) / 128), 128, 0, ctx->stream>>>(op, x, y, out, n);
    return gb_after_launch(ctx, "math_eval");
}
