// dynamw: vertical slopes advection, one sub-cycle count n_advz for the whole region.
//
// The region-wide search is a short sequence of launches with no host round trip.  Round 0:
// every column finds its own smallest passing n (cm / n, the "fresh" division of
// ops.py:310-312) and the candidate is their maximum (order-free integer atomic).  Round
// r >= 1: every column checks the candidate; a column that fails it pushes the next
// candidate to its own next passing n.  The region's n_advz is the first candidate every
// column passes -- the smallest n all columns pass, as the reference's sequential search
// finds it, with no assumption that passing is monotone in n.  k_z_steps: one warp per
// column (lanes along l, contiguous in memory), all n_advz sub-steps on chip; cm is divided
// in registers, so it is left bitwise as it was (the exact restore of kernels.py:328-346).
// Reference: pydyn kernels.py:295-346 (advect_z, advect_z_substeps), ops.py:315-341,
// zoom/advect.py:415-472 (column_trial, _dynamw_child: the search over the region, the update
// on the scope), cfl.py:186-194 and zoom/check_cfl.py:206-216 (dynamwm).
#include "gb_common.cuh"

namespace {

constexpr int WARPS = 4;
constexpr int ROUNDS = 3;  // round 0 + two verification rounds

struct ZArgs {
    DV m, q[4], cm;
    int im, jm, lm, nt;
    int si0, si1, sj0, sj1;  // scope (0-based, half-open): the columns the trial mass advances on
    int limits, nmax;
    int ncell;               // lm + 2
    int tc;                  // tracers staged at once (launch_z)
    gb_ctl *ctl;
    int mass_only;
    int32_t *coln;           // work space (im * jm): the n each column's last trial passed at
};

__device__ __forceinline__ double &AT(const DV &v, int64_t i, int64_t j, int64_t l) {
    return v.p[i * v.s0 + j * v.s1 + l * v.s2];
}
__device__ __forceinline__ double &AT4(const DV &v, int64_t i, int64_t j, int64_t l, int64_t t) {
    return v.p[i * v.s0 + j * v.s1 + l * v.s2 + t * v.s3];
}

// n trial sub-steps of one column under cm / n (ops.py:330-341; zoom/advect.py:415-441).
__device__ bool z_trial(const ZArgs &A, int i, int j, int n, double *mx, double *cf, int lane) {
    const int lm = A.lm;
    const bool scope = i >= A.si0 && i < A.si1 && j >= A.sj0 && j < A.sj1;
    for (int k = lane; k <= lm; k += GB_WARP) cf[k] = AT(A.cm, i, j, k) / (double)n;
    for (int k = lane; k < lm; k += GB_WARP) mx[k] = AT(A.m, i, j, k);
    __syncwarp();
    for (int s = 0; s < n; ++s) {
        bool lok = true;
        for (int k = 1 + lane; k < lm; k += GB_WARP) {
            double c = cf[k];
            double mu = (c >= 0.0) ? mx[k - 1] : mx[k];
            lok = lok && cfl_pass(c, mu);
        }
        if (!__all_sync(FULL_MASK, lok)) return false;
        if (!scope) continue;  // outside the scope the trial mass is never advanced
        for (int k = lane; k < lm; k += GB_WARP) mx[k] = (mx[k] + cf[k]) - cf[k + 1];
        __syncwarp();
    }
    return true;
}

__global__ void __launch_bounds__(WARPS * 32) k_z_search(ZArgs A, int round) {
    extern __shared__ double smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t col = (int64_t)blockIdx.x * WARPS + warp;
    if (col >= (int64_t)A.im * A.jm) return;
    if (A.mass_only && __shfl_sync(FULL_MASK, *(volatile int *)&A.ctl->cfl_failed, 0)) return;
    if (round >= 2 && !A.ctl->zsearch_changed[round - 1]) return;  // settled already
    const int i = (int)(col / A.jm), j = (int)(col % A.jm);
    double *mx = smem + (size_t)warp * 2 * A.ncell;
    double *cf = mx + A.ncell;
    if (round == 0) {
        // the outer interfaces must carry nothing (kernels.py:301-302)
        if (!A.mass_only && lane == 0 && (AT(A.cm, i, j, 0) != 0.0 || AT(A.cm, i, j, A.lm) != 0.0))
            raise_status(A.ctl, GB_EHALO);
        int n = 1;
        while (n <= A.nmax && !z_trial(A, i, j, n, mx, cf, lane)) ++n;
        if (lane == 0) {
            A.coln[col] = n;
            atomicMax(&A.ctl->zsearch_n[1], n);
        }
        return;
    }
    const int cand = A.ctl->zsearch_n[round];
    if (cand > A.nmax) return;  // some column never passes: the steps raise the error
    if (A.coln[col] == cand) return;  // its own trial passed at the candidate already
    if (z_trial(A, i, j, cand, mx, cf, lane)) {
        if (lane == 0) A.coln[col] = cand;
        return;
    }
    int n = cand + 1;
    while (n <= A.nmax && !z_trial(A, i, j, n, mx, cf, lane)) ++n;
    if (lane == 0) {
        A.coln[col] = n;
        atomicMax(&A.ctl->zsearch_n[round + 1], n);
        atomicExch(&A.ctl->zsearch_changed[round], 1);
    }
}

// n_advz of the search, or a status: nmax + 1 when no n passes, -1 when it did not settle
__device__ int z_settled(const ZArgs &A) {
    for (int r = 1; r < ROUNDS; ++r)
        if (!A.ctl->zsearch_changed[r]) return A.ctl->zsearch_n[r];
    return -1;
}

__global__ void k_z_last(ZArgs A, int32_t *n_out) { *n_out = z_settled(A); }

template <bool MASS_ONLY>
__global__ void __launch_bounds__(WARPS * 32) k_z_steps(ZArgs A) {
    extern __shared__ double smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t col = (int64_t)blockIdx.x * WARPS + warp;
    if (MASS_ONLY && __shfl_sync(FULL_MASK, *(volatile int *)&A.ctl->cfl_failed, 0)) return;
    const int n = z_settled(A);
    if (n < 0 || n > A.nmax) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            if (MASS_ONLY)
                atomicExch(&A.ctl->cfl_failed, 1);
            else
                raise_status(A.ctl, n < 0 ? GB_ESEARCH : GB_ECFL);
        }
        return;
    }
    if (col >= (int64_t)(A.si1 - A.si0) * (A.sj1 - A.sj0)) return;
    const int ns = A.sj1 - A.sj0;
    const int i = A.si0 + (int)(col / ns), j = A.sj0 + (int)(col % ns);
    const int lm = A.lm, nt = MASS_ONLY ? 0 : A.nt, NC = A.ncell;
    const int tc = MASS_ONLY ? 0 : A.tc;  // tracers staged at once (a chunk)
    double *m_s = smem + (size_t)warp * NC * (3 + 8 * tc);
    double *c_s = m_s + NC;
    double *m0_s = c_s + NC;           // the staged mass, each chunk's start
    double *q_s = m0_s + NC;
    double *f_s = q_s + 4 * tc * NC;
    auto Q = [&](int w, int t) { return q_s + (size_t)(w * tc + t) * NC; };
    auto F = [&](int w, int t) { return f_s + (size_t)(w * tc + t) * NC; };

    for (int k = lane; k <= lm; k += GB_WARP) c_s[k] = AT(A.cm, i, j, k) / (double)n;
    for (int k = lane; k < lm; k += GB_WARP) {
        m_s[k] = AT(A.m, i, j, k);
        m0_s[k] = m_s[k];
    }
    __syncwarp();

    if (MASS_ONLY) {  // dynamwm: n_advz = 1 passed; the mass advanced once on the scope
        for (int k = lane; k < lm; k += GB_WARP) AT(A.m, i, j, k) = (m_s[k] + c_s[k]) - c_s[k + 1];
        return;
    }

    // the tracers, tc at a time: each chunk restarts from the staged mass and repeats the same
    // mass updates; tracers never mix, so the chunking changes no value
    for (int t0 = 0; t0 < nt; t0 += tc) {
        const int ntc = min(tc, nt - t0);
        for (int k = lane; k < lm; k += GB_WARP) {
            m_s[k] = m0_s[k];
            for (int w = 0; w < 4; ++w)
                for (int t = 0; t < ntc; ++t) Q(w, t)[k] = AT4(A.q[w], i, j, k, t0 + t);
            if (A.limits)
                for (int t = 0; t < ntc; ++t) Q(3, t)[k] = np_limit(Q(3, t)[k], Q(0, t)[k]);
        }
        if (lane == 0)
            for (int w = 0; w < 4; ++w)
                for (int t = 0; t < ntc; ++t) F(w, t)[0] = F(w, t)[lm] = 0.0;
        __syncwarp();

        for (int s = 0; s < n; ++s) {
            for (int k = 1 + lane; k < lm; k += GB_WARP) {
                const double ck = c_s[k];
                const int up = (ck >= 0.0) ? k - 1 : k;
                const double gamma = ck / m_s[up];
                for (int t = 0; t < ntc; ++t) {
                    double f, pf, fx, fy;
                    // the along slope is rzm, the cross slopes rxm, rym
                    slopes_flux(ck, gamma, Q(0, t)[up], Q(3, t)[up], Q(1, t)[up], Q(2, t)[up], f, pf, fx, fy);
                    F(0, t)[k] = f; F(1, t)[k] = pf; F(2, t)[k] = fx; F(3, t)[k] = fy;
                }
            }
            __syncwarp();
            for (int k = lane; k < lm; k += GB_WARP) {
                const double mo = m_s[k], clo = c_s[k], chi = c_s[k + 1];
                const double mn = (mo + clo) - chi;
                for (int t = 0; t < ntc; ++t) {
                    const double *f = F(0, t), *pf = F(1, t), *fx = F(2, t), *fy = F(3, t);
                    // advectz: rm + f(l-1) - f(l), no parentheses
                    const double rmn = (Q(0, t)[k] + f[k]) - f[k + 1];
                    double rzn = along_slope(Q(3, t)[k], pf[k], pf[k + 1], clo, chi, rmn, f[k], f[k + 1], mo, mn);
                    if (A.limits) rzn = np_limit(rzn, rmn);
                    Q(0, t)[k] = rmn;
                    Q(3, t)[k] = rzn;
                    Q(1, t)[k] = (Q(1, t)[k] + fx[k]) - fx[k + 1];
                    Q(2, t)[k] = (Q(2, t)[k] + fy[k]) - fy[k + 1];
                }
                m_s[k] = mn;
            }
            __syncwarp();
        }
        for (int k = lane; k < lm; k += GB_WARP)
            for (int w = 0; w < 4; ++w)
                for (int t = 0; t < ntc; ++t) AT4(A.q[w], i, j, k, t0 + t) = Q(w, t)[k];
        __syncwarp();  // the next chunk overwrites the staged tracers
    }
    for (int k = lane; k < lm; k += GB_WARP) AT(A.m, i, j, k) = m_s[k];
}

// tracers a warp stages at once: as many as fit in the block's shared memory (all when they do)
int tracer_chunk(int warps, int ncell, int fixed, int per_tracer, int nt) {
    const size_t cap = 227 * 1024;
    int tc = nt;
    while (tc > 1 && (size_t)warps * ncell * (fixed + per_tracer * tc) * sizeof(double) > cap) --tc;
    return tc;
}

int launch_z(gb_ctx *ctx, ZArgs &A) {
    A.ncell = A.lm + 2;
    GB_CHECK_CUDA(cudaMemsetAsync(A.ctl->zsearch_n, 0, sizeof(A.ctl->zsearch_n) + sizeof(A.ctl->zsearch_changed),
                                  ctx->stream));
    size_t smem_s = (size_t)WARPS * 2 * A.ncell * sizeof(double);
    int64_t cols = (int64_t)A.im * A.jm;
    int blocks = (int)((cols + WARPS - 1) / WARPS);
    if (blocks == 0) return GB_OK;
    A.coln = reinterpret_cast<int32_t *>(gb_work(ctx, (size_t)cols * sizeof(int32_t)));
    if (!A.coln) return GB_ECUDA;
    for (int r = 0; r < ROUNDS; ++r) {
        k_z_search<<<blocks, WARPS * 32, smem_s, ctx->stream>>>(A, r);
        int rc = gb_after_launch(ctx, "z_search");
        if (rc) return rc;
    }
    A.tc = A.mass_only ? 0 : tracer_chunk(WARPS, A.ncell, 3, 8, A.nt);
    size_t smem = (size_t)WARPS * A.ncell * (3 + 8 * A.tc) * sizeof(double);
    int64_t scols = (int64_t)(A.si1 - A.si0) * (A.sj1 - A.sj0);
    int sblocks = (int)((scols + WARPS - 1) / WARPS);
    if (sblocks < 1) sblocks = 1;
    if (A.mass_only) {
        GB_CHECK_CUDA(cudaFuncSetAttribute(k_z_steps<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_z_steps<true><<<sblocks, WARPS * 32, smem, ctx->stream>>>(A);
    } else {
        GB_CHECK_CUDA(cudaFuncSetAttribute(k_z_steps<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_z_steps<false><<<sblocks, WARPS * 32, smem, ctx->stream>>>(A);
    }
    return gb_after_launch(ctx, A.mass_only ? "cfl_z" : "z_steps");
}

}  // namespace

extern "C" int gb_advect_z_scope(gb_ctx *ctx, const gb_view *m, const gb_view *rm, const gb_view *rxm,
                                 const gb_view *rym, const gb_view *rzm, const gb_view *cm, int si0, int si1,
                                 int sj0, int sj1, int limits, int iter_limit) {
    if (!ctx || !m || !rm || !rxm || !rym || !rzm || !cm) return GB_EARG;
    ZArgs A{};
    A.m = dv(m);
    A.q[0] = dv(rm); A.q[1] = dv(rxm); A.q[2] = dv(rym); A.q[3] = dv(rzm);
    A.cm = dv(cm);
    A.im = (int)m->n[0]; A.jm = (int)m->n[1]; A.lm = (int)m->n[2]; A.nt = (int)rm->n[3];
    if (cm->n[2] != A.lm + 1) {
        gb_set_error("gb_advect_z: cm must have lm+1 interfaces");
        return GB_EARG;
    }
    A.si0 = si0; A.si1 = si1; A.sj0 = sj0; A.sj1 = sj1;
    A.limits = limits; A.nmax = iter_limit;
    A.ctl = ctx->ctl;
    A.mass_only = 0;
    return launch_z(ctx, A);
}

extern "C" int gb_advect_z(gb_ctx *ctx, const gb_view *m, const gb_view *rm, const gb_view *rxm,
                           const gb_view *rym, const gb_view *rzm, const gb_view *cm, int limits,
                           int iter_limit, int32_t *n_out) {
    (void)n_out;
    return gb_advect_z_scope(ctx, m, rm, rxm, rym, rzm, cm, 0, (int)m->n[0], 0, (int)m->n[1], limits, iter_limit);
}

extern "C" int gb_cfl_z(gb_ctx *ctx, const gb_view *m, const gb_view *cm, int si0, int si1, int sj0, int sj1,
                        int iter_limit) {
    if (!ctx || !m || !cm) return GB_EARG;
    ZArgs A{};
    A.m = dv(m);
    for (int w = 0; w < 4; ++w) A.q[w] = A.m;
    A.cm = dv(cm);
    A.im = (int)m->n[0]; A.jm = (int)m->n[1]; A.lm = (int)m->n[2]; A.nt = 0;
    A.si0 = si0; A.si1 = si1; A.sj0 = sj0; A.sj1 = sj1;
    A.limits = 0; A.nmax = iter_limit;
    A.ctl = ctx->ctl;
    A.mass_only = 1;
    return launch_z(ctx, A);
}

// n_advz of the context's last dynamw (or dynamwm) into a device int32, -1 if its search did not
// settle: what the adjoint of that call divides cm by
extern "C" int gb_advect_z_last(gb_ctx *ctx, int32_t *n_out) {
    if (!ctx || !n_out) return GB_EARG;
    ZArgs A{};
    A.ctl = ctx->ctl;
    k_z_last<<<1, 1, 0, ctx->stream>>>(A, n_out);
    return gb_after_launch(ctx, "advect_z_last");
}
