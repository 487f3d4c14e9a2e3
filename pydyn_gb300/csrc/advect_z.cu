// dynamw: vertical slopes advection, one sub-cycle count n_advz for the whole region.
//
// The region-wide search is a short sequence of launches with no host round trip.  Round 0:
// every column finds its own smallest passing n (cm / n, the "fresh" division of
// ops.py:310-312) and the candidate is their maximum (order-free integer atomic).  Round
// r >= 1: every column checks the candidate; a column that fails it pushes the next
// candidate to its own next passing n.  The region's n_advz is the first candidate every
// column passes -- the smallest n all columns pass, as the reference's sequential search
// finds it, with no assumption that passing is monotone in n.  k_z_steps: all n_advz
// sub-steps on chip; cm is divided in shared memory, so it is left bitwise as it was (the exact
// restore of kernels.py:328-346).
//
// Both kernels run a block over P whole columns, one thread per (column, level): P = 32 /
// gcd(lm, 32) (halved while the block exceeds 576 threads) makes the block a whole number of
// warps (16 columns of 34 levels are 17 warps),
// so every FP64 instruction issues with its lanes full, where a warp per column of 34 levels
// would issue each statement twice, the second time for two lanes.  A column's threads meet at
// block barriers; per-column decisions (a failed Courant test, the search's next n) go through
// shared memory.
// Reference: pydyn kernels.py:295-346 (advect_z, advect_z_substeps), ops.py:315-341,
// zoom/advect.py:415-472 (column_trial, _dynamw_child: the search over the region, the update
// on the scope), cfl.py:186-194 and zoom/check_cfl.py:206-216 (dynamwm).
#include "gb_common.cuh"

namespace {

constexpr int ROUNDS = 3;      // round 0 + two verification rounds
constexpr int MAX_COLS = 32;   // columns per block
constexpr int MAX_THREADS = 576;  // two blocks an SM at <= 56 registers a thread

struct ZArgs {
    DV m, q[4], cm;
    int im, jm, lm, nt;
    int si0, si1, sj0, sj1;  // scope (0-based, half-open): the columns the trial mass advances on
    int limits, nmax;
    int ncell;               // lm + 2
    int P;                   // columns per block
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

// columns per block for lm levels: whole warps where they fit in a block
int cols_per_block(int lm) {
    int g = 32, a = lm;
    while (a % 2 == 0 && g > 1) { a /= 2; g /= 2; }  // g = 32 / gcd(lm, 32)
    int P = g;
    while (P > 1 && P * lm > MAX_THREADS) P /= 2;
    return P;
}

// a column's search state in the block (shared memory)
struct ZCol {
    int n;       // the n being tried
    int state;   // 0 idle (nothing to try), 1 trying, 2 failed the trial in progress
    int moved;   // round >= 1: failed the candidate at least once
};

// One trial of every trying column of the block at its own n (ops.py:330-341;
// zoom/advect.py:415-441): n sub-steps of the mass under cm / n, each tested first; a failure
// ends that column's trial (state 2).  mx, cf: P * ncell doubles each.
__device__ void z_trials(const ZArgs &A, ZCol *zc, double *mx, double *cf, int p, int k, int64_t col0, int ncols,
                         bool scope) {
    const int lm = A.lm, P = A.P, NC = A.ncell;
    // cf = cm / n over every column's lm + 1 interfaces, spread over the block's threads.  At
    // n = 1 the quotient is cm itself (x / 1 = x exactly; a NaN fails the test either way), and
    // these trial values decide only pass or fail, so the division is left out there.
    for (int e = threadIdx.x; e < P * (lm + 1); e += blockDim.x) {
        const int q = e / (lm + 1), kk = e % (lm + 1);
        if (q < ncols && zc[q].state == 1) {
            const int64_t col = col0 + q;
            const int i = (int)(col / A.jm), j = (int)(col % A.jm);
            const double v = AT(A.cm, i, j, kk);
            cf[q * NC + kk] = zc[q].n == 1 ? v : div_ip(v, (double)zc[q].n);
        }
    }
    const bool mine = p < ncols && zc[p].state == 1;
    const int64_t col = col0 + p;
    const int i = mine ? (int)(col / A.jm) : 0, j = mine ? (int)(col % A.jm) : 0;
    if (mine) mx[p * NC + k] = AT(A.m, i, j, k);
    int nmax_s = 0;
    for (int q = 0; q < ncols; ++q)
        if (zc[q].state == 1 && zc[q].n > nmax_s) nmax_s = zc[q].n;
    __syncthreads();
    const double *c = cf + p * NC;
    double *x = mx + p * NC;
    for (int s = 0; s < nmax_s; ++s) {
        const bool run = mine && s < zc[p].n && zc[p].state == 1;
        if (run && k >= 1) {
            const double ck = c[k];
            const double mu = ge_zero(ck) ? x[k - 1] : x[k];
            if (!cfl_pass(ck, mu)) zc[p].state = 2;  // every failing thread writes the same value
        }
        __syncthreads();
        // outside the scope the trial mass is never advanced
        if (run && scope && zc[p].state == 1) x[k] = (x[k] + c[k]) - c[k + 1];
        __syncthreads();
    }
}

__global__ void __launch_bounds__(MAX_THREADS, 2) k_z_search(ZArgs A, int round) {
    extern __shared__ double smem[];
    __shared__ ZCol zc[MAX_COLS];
    __shared__ int s_skip;
    const int lm = A.lm, P = A.P;
    const int p = threadIdx.x / lm, k = threadIdx.x % lm;
    const int64_t total = (int64_t)A.im * A.jm, col0 = (int64_t)blockIdx.x * P;
    const int ncols = (int)min((int64_t)P, total - col0);
    if (threadIdx.x == 0) {
        // block-uniform exits: the rehearsal already failed, or the search settled a round ago
        s_skip = (A.mass_only && *(volatile int *)&A.ctl->cfl_failed) || (round >= 2 && !A.ctl->zsearch_changed[round - 1]);
    }
    __syncthreads();
    if (s_skip) return;
    const int cand = round == 0 ? 1 : A.ctl->zsearch_n[round];
    if (round >= 1 && cand > A.nmax) return;  // some column never passes: the steps raise the error
    double *mx = smem, *cf = smem + (size_t)P * A.ncell;
    const bool live = p < ncols;
    const int64_t col = col0 + p;
    const int i = live ? (int)(col / A.jm) : 0, j = live ? (int)(col % A.jm) : 0;
    const bool scope = live && i >= A.si0 && i < A.si1 && j >= A.sj0 && j < A.sj1;
    if (live && k == 0) {
        if (round == 0) {
            // the outer interfaces must carry nothing (kernels.py:301-302)
            if (!A.mass_only && (AT(A.cm, i, j, 0) != 0.0 || AT(A.cm, i, j, lm) != 0.0)) raise_status(A.ctl, GB_EHALO);
            zc[p] = ZCol{1, A.nmax >= 1 ? 1 : 0, 0};
            if (A.nmax < 1) {  // no n to try: the search ends at nmax + 1
                A.coln[col] = 1;
                atomicMax(&A.ctl->zsearch_n[1], 1);
            }
        } else {
            // its own trial passed at the candidate already: nothing to try
            zc[p] = ZCol{cand, A.coln[col] == cand ? 0 : 1, 0};
        }
    }
    __syncthreads();
    while (true) {
        if (!__syncthreads_or(live && k == 0 && zc[p].state == 1)) break;
        z_trials(A, zc, mx, cf, p, k, col0, ncols, scope);
        if (live && k == 0 && zc[p].state != 0) {
            if (zc[p].state == 1) {  // passed at n
                zc[p].state = 0;
                A.coln[col] = zc[p].n;
                if (round == 0 || zc[p].moved) {
                    atomicMax(&A.ctl->zsearch_n[round + 1], zc[p].n);
                    if (round >= 1) atomicExch(&A.ctl->zsearch_changed[round], 1);
                }
            } else if (zc[p].n + 1 > A.nmax) {  // no n up to the cap passes
                zc[p].state = 0;
                A.coln[col] = zc[p].n + 1;
                atomicMax(&A.ctl->zsearch_n[round + 1], zc[p].n + 1);
                if (round >= 1) atomicExch(&A.ctl->zsearch_changed[round], 1);
            } else {
                zc[p].n += 1;
                zc[p].state = 1;
                zc[p].moved = 1;
            }
        }
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
__global__ void __launch_bounds__(MAX_THREADS, 2) k_z_steps(ZArgs A) {
    extern __shared__ double smem[];
    __shared__ int s_n;
    const int lm = A.lm, P = A.P, NC = A.ncell;
    const int p = threadIdx.x / lm, k = threadIdx.x % lm;
    if (threadIdx.x == 0) {
        int n = z_settled(A);
        if (MASS_ONLY && *(volatile int *)&A.ctl->cfl_failed) n = 0;  // the rehearsal failed already
        s_n = n;
    }
    __syncthreads();
    const int n = s_n;
    if (MASS_ONLY && n == 0) return;
    if (n < 0 || n > A.nmax) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            if (MASS_ONLY)
                atomicExch(&A.ctl->cfl_failed, 1);
            else
                raise_status(A.ctl, n < 0 ? GB_ESEARCH : GB_ECFL);
        }
        return;
    }
    const int ns = A.sj1 - A.sj0;
    const int64_t total = (int64_t)(A.si1 - A.si0) * ns, col0 = (int64_t)blockIdx.x * P;
    const int ncols = (int)min((int64_t)P, total - col0);
    const bool live = p < ncols;
    const int64_t col = col0 + p;
    const int i = live ? A.si0 + (int)(col / ns) : 0, j = live ? A.sj0 + (int)(col % ns) : 0;
    const int nt = MASS_ONLY ? 0 : A.nt;
    const int tc = MASS_ONLY ? 0 : A.tc;  // tracers staged at once (a chunk)
    const size_t per = (size_t)NC * (3 + 8 * tc);
    // cm / n of every column's interfaces, spread over the block's threads
    for (int e = threadIdx.x; e < ncols * (lm + 1); e += blockDim.x) {
        const int q = e / (lm + 1), kk = e % (lm + 1);
        const int64_t cq = col0 + q;
        smem[q * per + NC + kk] = div_ip(AT(A.cm, A.si0 + (int)(cq / ns), A.sj0 + (int)(cq % ns), kk), (double)n);
    }
    double *m_s = smem + p * per;
    double *c_s = m_s + NC;
    double *m0_s = c_s + NC;           // the staged mass, each chunk's start
    double *q_s = m0_s + NC;
    double *f_s = q_s + 4 * tc * NC;
    auto Q = [&](int w, int t) { return q_s + (size_t)(w * tc + t) * NC; };
    auto F = [&](int w, int t) { return f_s + (size_t)(w * tc + t) * NC; };
    if (live) {
        m_s[k] = AT(A.m, i, j, k);
        m0_s[k] = m_s[k];
    }
    __syncthreads();

    if constexpr (MASS_ONLY) {  // dynamwm: n_advz = 1 passed; the mass advanced once on the scope
        if (live) AT(A.m, i, j, k) = (m_s[k] + c_s[k]) - c_s[k + 1];
    } else {
        // the tracers, tc at a time: each chunk restarts from the staged mass and repeats the same
        // mass updates; tracers never mix, so the chunking changes no value
        for (int t0 = 0; t0 < nt; t0 += tc) {
            const int ntc = min(tc, nt - t0);
            if (live) {
                m_s[k] = m0_s[k];
                for (int w = 0; w < 4; ++w)
                    for (int t = 0; t < ntc; ++t) Q(w, t)[k] = AT4(A.q[w], i, j, k, t0 + t);
                if (A.limits)
                    for (int t = 0; t < ntc; ++t) Q(3, t)[k] = np_limit(Q(3, t)[k], Q(0, t)[k]);
                if (k == 0)
                    for (int w = 0; w < 4; ++w)
                        for (int t = 0; t < ntc; ++t) F(w, t)[0] = F(w, t)[lm] = 0.0;
            }
            __syncthreads();

            for (int s = 0; s < n; ++s) {
                if (live && k >= 1) {
                    const double ck = c_s[k];
                    const int up = ge_zero(ck) ? k - 1 : k;
                    const double gamma = div_ip(ck, m_s[up]);
                    for (int t = 0; t < ntc; ++t) {
                        double f, pf, fx, fy;
                        // the along slope is rzm, the cross slopes rxm, rym
                        slopes_flux(ck, gamma, Q(0, t)[up], Q(3, t)[up], Q(1, t)[up], Q(2, t)[up], f, pf, fx, fy);
                        F(0, t)[k] = f; F(1, t)[k] = pf; F(2, t)[k] = fx; F(3, t)[k] = fy;
                    }
                }
                __syncthreads();
                if (live) {
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
                __syncthreads();
            }
            if (live)
                for (int w = 0; w < 4; ++w)
                    for (int t = 0; t < ntc; ++t) AT4(A.q[w], i, j, k, t0 + t) = Q(w, t)[k];
            __syncthreads();  // the next chunk overwrites the staged tracers
        }
        if (live) AT(A.m, i, j, k) = m_s[k];
    }
}

// tracers a block stages at once: as many as fit in its shared memory (all when they do)
int tracer_chunk(int cols, int ncell, int fixed, int per_tracer, int nt) {
    const size_t cap = 227 * 1024;
    int tc = nt;
    while (tc > 1 && (size_t)cols * ncell * (fixed + per_tracer * tc) * sizeof(double) > cap) --tc;
    return tc;
}

int launch_z(gb_ctx *ctx, ZArgs &A) {
    if (A.lm > MAX_THREADS) {
        gb_set_error("gb_advect_z: at most 576 levels");
        return GB_EARG;
    }
    A.ncell = A.lm + 2;
    A.P = cols_per_block(A.lm);
    const int threads = (A.P * A.lm + 31) / 32 * 32;
    GB_CHECK_CUDA(cudaMemsetAsync(A.ctl->zsearch_n, 0, sizeof(A.ctl->zsearch_n) + sizeof(A.ctl->zsearch_changed),
                                  ctx->stream));
    const size_t smem_s = (size_t)A.P * 2 * A.ncell * sizeof(double);
    const int64_t cols = (int64_t)A.im * A.jm;
    const int blocks = (int)((cols + A.P - 1) / A.P);
    if (blocks == 0) return GB_OK;
    A.coln = reinterpret_cast<int32_t *>(gb_work(ctx, (size_t)cols * sizeof(int32_t)));
    if (!A.coln) return GB_ECUDA;
    GB_CHECK_CUDA(cudaFuncSetAttribute(k_z_search, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_s));
    // with a cap of one (Check_CFL's rehearsal) round 0 decides: every column passes at n = 1 or
    // records 2, so round 1 has nothing to try and round 2 finds nothing changed
    const int rounds = A.nmax <= 1 ? 1 : ROUNDS;
    for (int r = 0; r < rounds; ++r) {
        k_z_search<<<blocks, threads, smem_s, ctx->stream>>>(A, r);
        int rc = gb_after_launch(ctx, "z_search");
        if (rc) return rc;
    }
    A.tc = A.mass_only ? 0 : tracer_chunk(A.P, A.ncell, 3, 8, A.nt);
    const size_t smem = (size_t)A.P * A.ncell * (3 + 8 * A.tc) * sizeof(double);
    if (smem > 227 * 1024) {
        gb_set_error("gb_advect_z: the columns of a block do not fit in shared memory");
        return GB_EARG;
    }
    const int64_t scols = (int64_t)(A.si1 - A.si0) * (A.sj1 - A.sj0);
    int sblocks = (int)((scols + A.P - 1) / A.P);
    if (sblocks < 1) sblocks = 1;
    if (A.mass_only) {
        GB_CHECK_CUDA(cudaFuncSetAttribute(k_z_steps<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_z_steps<true><<<sblocks, threads, smem, ctx->stream>>>(A);
    } else {
        GB_CHECK_CUDA(cudaFuncSetAttribute(k_z_steps<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_z_steps<false><<<sblocks, threads, smem, ctx->stream>>>(A);
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
