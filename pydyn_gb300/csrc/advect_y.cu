// dynamv: meridional slopes advection with polar caps, one sub-cycle count per layer.
//
// Two launches.  k_y_search: one CTA per layer runs the layer's CFL search exactly as the
// reference does -- every column of the layer tried at n = 1, 2, ... until all pass -- with
// the progressively rescaled faces recomputed from the untouched bm (the rescale is a fixed
// chain per face), and rescales the faces of the halo'd layer that the columns do not own.
// k_y_steps: one warp per (i, l) column stages the column in shared memory, runs the layer's
// sub-steps on chip and writes the column and its faces (rescaled, then times nloop) once.
// Reference: pydyn kernels.py:223-291 (advect_y, _advect_layer_y), ops.py:315-341
// (subcycles, _trial), zoom/advect.py:201-226 (_dynamv_region1, _rescale_layer_halo),
// cfl.py:170-183 (dynamvm) and zoom/advect.py:348-412 (_dynamv_child).
#include "gb_common.cuh"

namespace {

constexpr int SEARCH_THREADS = 256;
constexpr int STEP_WARPS = 4;

struct YArgs {
    DV m, q[4], bm, full;
    int im, jm, lm, nt;
    int full_l0;       // level of `full` that is bm's level 0
    int limits, nmax;  // nmax = max_nloop - 1
    int ncell;         // jm + 2
    int32_t *nloop;    // lm, written by the search
    int32_t *nloop_out;
    gb_ctl *ctl;
    int mass_only;     // the Check_CFL rehearsal (dynamvm): search capped, then one advance
};

__device__ __forceinline__ double &AT(const DV &v, int64_t i, int64_t j, int64_t l) {
    return v.p[i * v.s0 + j * v.s1 + l * v.s2];
}
__device__ __forceinline__ double &AT4(const DV &v, int64_t i, int64_t j, int64_t l, int64_t t) {
    return v.p[i * v.s0 + j * v.s1 + l * v.s2 + t * v.s3];
}

// One column's trial (ops.py:330-341, closed axis): n sub-steps of its mass with faces b
// (already rescaled), the Courant number of each interior face checked before each.
__device__ bool column_trial(const YArgs &A, int i, int l, int n, double *mx, double *bf, int lane) {
    const int jm = A.jm;
    for (int k = lane; k <= jm; k += GB_WARP) bf[k] = progressive_chain(AT(A.bm, i, k, l), n);
    for (int k = lane; k < jm; k += GB_WARP) mx[k] = AT(A.m, i, k, l);
    __syncwarp();
    for (int s = 0; s < n; ++s) {
        bool lok = true;
        for (int k = 1 + lane; k < jm; k += GB_WARP) {
            double f = bf[k];
            double mu = (f >= 0.0) ? mx[k - 1] : mx[k];
            lok = lok && (fabs(f / mu) < 1.0);
        }
        if (!__all_sync(FULL_MASK, lok)) return false;
        for (int k = lane; k < jm; k += GB_WARP) mx[k] = (mx[k] + bf[k]) - bf[k + 1];
        __syncwarp();
    }
    return true;
}

__global__ void __launch_bounds__(SEARCH_THREADS) k_y_search(YArgs A) {
    extern __shared__ double smem[];
    __shared__ int s_fail;
    __shared__ int s_halo;
    __shared__ int s_abort;
    const int l = blockIdx.x;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nwarps = SEARCH_THREADS / 32;
    double *mx = smem + (size_t)warp * 2 * A.ncell;
    double *bf = mx + A.ncell;

    // one read of the rehearsal flag for the whole CTA, so that every thread takes the same path
    if (threadIdx.x == 0) {
        s_abort = A.mass_only ? *(volatile int *)&A.ctl->cfl_failed : 0;
        s_halo = 0;
    }
    __syncthreads();
    if (s_abort) return;

    // the polar outer faces must carry nothing (kernels.py:233-234); dynamvm does not check
    if (!A.mass_only)
        for (int i = threadIdx.x; i < A.im; i += SEARCH_THREADS)
            if (AT(A.bm, i, 0, l) != 0.0 || AT(A.bm, i, A.jm, l) != 0.0) s_halo = 1;
    __syncthreads();
    if (s_halo) {
        if (threadIdx.x == 0) raise_status(A.ctl, GB_EHALO);
        return;
    }

    int nloop = 1;
    while (true) {
        if (threadIdx.x == 0) s_fail = 0;
        __syncthreads();
        for (int i = warp; i < A.im; i += nwarps) {
            if (!column_trial(A, i, l, nloop, mx, bf, lane)) {
                if (lane == 0) s_fail = 1;
            }
            __syncwarp();
        }
        __syncthreads();
        const int failed = s_fail;
        __syncthreads();
        if (!failed) break;
        nloop += 1;
        if (nloop > A.nmax) break;
    }
    if (threadIdx.x == 0) {
        A.nloop[l] = nloop;
        if (A.nloop_out) A.nloop_out[l] = nloop;
        if (nloop > A.nmax) {
            if (A.mass_only)
                atomicExch(&A.ctl->cfl_failed, 1);
            else
                raise_status(A.ctl, GB_ECFL);
        }
    }
    if (nloop > A.nmax || A.mass_only) return;

    // the faces of the halo'd layer outside the columns' own: rescaled and restored alike
    if (A.full.p && nloop > 1) {
        const int64_t ni = A.full.n0, nj = A.full.n1;
        const int lf = l + A.full_l0;
        for (int64_t k = threadIdx.x; k < ni * nj; k += SEARCH_THREADS) {
            int64_t fi = k / nj, fj = k % nj;
            bool inside = fi >= 1 && fi <= A.im && fj >= 1 && fj <= A.jm + 1;
            if (inside) continue;
            double &b = AT(A.full, fi, fj, lf);
            b = progressive_chain(b, nloop) * (double)nloop;
        }
    }
}

template <bool MASS_ONLY>
__global__ void __launch_bounds__(STEP_WARPS * 32) k_y_steps(YArgs A) {
    extern __shared__ double smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t col = (int64_t)blockIdx.x * STEP_WARPS + warp;
    if (col >= (int64_t)A.im * A.lm) return;
    if (MASS_ONLY && __shfl_sync(FULL_MASK, *(volatile int *)&A.ctl->cfl_failed, 0)) return;
    const int i = (int)(col / A.lm), l = (int)(col % A.lm);
    const int nloop = A.nloop[l];
    if (nloop > A.nmax) return;
    const int jm = A.jm, nt = MASS_ONLY ? 0 : A.nt, NC = A.ncell;
    double *m_s = smem + (size_t)warp * NC * (2 + 8 * nt);
    double *b_s = m_s + NC;
    double *q_s = b_s + NC;            // [4][nt]: rm, rxm, rym, rzm
    double *f_s = q_s + 4 * nt * NC;   // [4][nt]: f, pf, fx, fz
    auto Q = [&](int w, int t) { return q_s + (size_t)(w * nt + t) * NC; };
    auto F = [&](int w, int t) { return f_s + (size_t)(w * nt + t) * NC; };

    for (int k = lane; k <= jm; k += GB_WARP) b_s[k] = progressive_chain(AT(A.bm, i, k, l), nloop);
    for (int k = lane; k < jm; k += GB_WARP) {
        m_s[k] = AT(A.m, i, k, l);
        for (int w = 0; w < 4; ++w)
            for (int t = 0; t < nt; ++t) Q(w, t)[k] = AT4(A.q[w], i, k, l, t);
    }
    __syncwarp();

    if (MASS_ONLY) {  // dynamvm: nloop = 1 passed; one advance; b * 1
        for (int k = lane; k < jm; k += GB_WARP) AT(A.m, i, k, l) = (m_s[k] + b_s[k]) - b_s[k + 1];
        return;
    }

    if (A.limits)  // every row, the pole cells included
        for (int t = 0; t < nt; ++t)
            for (int k = lane; k < jm; k += GB_WARP) Q(2, t)[k] = np_limit(Q(2, t)[k], Q(0, t)[k]);
    // closed outer faces
    if (lane == 0)
        for (int w = 0; w < 4; ++w)
            for (int t = 0; t < nt; ++t) F(w, t)[0] = F(w, t)[jm] = 0.0;
    __syncwarp();

    for (int s = 0; s < nloop; ++s) {
        for (int k = 1 + lane; k < jm; k += GB_WARP) {
            const double bk = b_s[k];
            const int up = (bk >= 0.0) ? k - 1 : k;
            const double beta = bk / m_s[up];
            for (int t = 0; t < nt; ++t) {
                double f, pf, fx, fz;
                // the along slope is rym, the cross slopes rxm, rzm
                slopes_flux(bk, beta, Q(0, t)[up], Q(2, t)[up], Q(1, t)[up], Q(3, t)[up], f, pf, fx, fz);
                // flow out of a pole cell carries no slope (Fortran faces 2 and jmr)
                if (k == 1 && bk >= 0.0) {
                    f = beta * Q(0, t)[0];
                    pf = (-3.0 * bk) * f;
                    fx = 0.0;
                    fz = beta * Q(3, t)[0];
                }
                if (k == jm - 1 && bk < 0.0) {
                    f = beta * Q(0, t)[jm - 1];
                    pf = (-3.0 * bk) * f;
                    fx = 0.0;
                    fz = beta * Q(3, t)[jm - 1];
                }
                F(0, t)[k] = f; F(1, t)[k] = pf; F(2, t)[k] = fx; F(3, t)[k] = fz;
            }
        }
        __syncwarp();
        for (int j = lane; j < jm; j += GB_WARP) {
            const double mo = m_s[j], blo = b_s[j], bhi = b_s[j + 1];
            const double mn = (mo + blo) - bhi;
            const double inv = 1.0 / mn;  // production dynamv hoists the reciprocal
            const double fc = blo - bhi;
            const double fm = 3.0 * (blo + bhi);
            const double mx3 = 3.0 * mo;
            const bool pole = (j == 0) || (j == jm - 1);
            for (int t = 0; t < nt; ++t) {
                const double *f = F(0, t), *pf = F(1, t), *fx = F(2, t), *fz = F(3, t);
                const double rmn = Q(0, t)[j] - (f[j + 1] - f[j]);
                const double ry = Q(2, t)[j];
                double ryn = ry + ((((pf[j] - pf[j + 1]) - fc * ry) + fm * rmn) - mx3 * (f[j] + f[j + 1])) * inv;
                if (A.limits) ryn = np_limit(ryn, rmn);
                const double rx = Q(1, t)[j];
                const double rxn = rx - (fx[j + 1] - fx[j]);
                Q(3, t)[j] = Q(3, t)[j] - (fz[j + 1] - fz[j]);
                Q(0, t)[j] = rmn;
                if (!pole) {  // the poles keep rxm, rym (only rm, rzm are updated there)
                    Q(2, t)[j] = ryn;
                    Q(1, t)[j] = rxn;
                }
            }
            m_s[j] = mn;
        }
        __syncwarp();
    }

    for (int k = lane; k < jm; k += GB_WARP) {
        AT(A.m, i, k, l) = m_s[k];
        for (int w = 0; w < 4; ++w)
            for (int t = 0; t < nt; ++t) AT4(A.q[w], i, k, l, t) = Q(w, t)[k];
    }
    for (int k = lane; k <= jm; k += GB_WARP) AT(A.bm, i, k, l) = b_s[k] * (double)nloop;
}

int launch_y(gb_ctx *ctx, YArgs &A) {
    A.ncell = A.jm + 2;
    A.nloop = gb_scratch_i(ctx, A.lm);
    if (!A.nloop) {
        gb_set_error("gb_advect_y: too many levels for the scratch");
        return GB_EARG;
    }
    size_t smem_s = (size_t)(SEARCH_THREADS / 32) * 2 * A.ncell * sizeof(double);
    GB_CHECK_CUDA(cudaFuncSetAttribute(k_y_search, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_s));
    k_y_search<<<A.lm, SEARCH_THREADS, smem_s, ctx->stream>>>(A);
    int rc = gb_after_launch(ctx, "y_search");
    if (rc) return rc;
    const int nt = A.mass_only ? 0 : A.nt;
    size_t smem = (size_t)STEP_WARPS * A.ncell * (2 + 8 * nt) * sizeof(double);
    int64_t cols = (int64_t)A.im * A.lm;
    int blocks = (int)((cols + STEP_WARPS - 1) / STEP_WARPS);
    if (A.mass_only) {
        GB_CHECK_CUDA(cudaFuncSetAttribute(k_y_steps<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_y_steps<true><<<blocks, STEP_WARPS * 32, smem, ctx->stream>>>(A);
    } else {
        GB_CHECK_CUDA(cudaFuncSetAttribute(k_y_steps<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_y_steps<false><<<blocks, STEP_WARPS * 32, smem, ctx->stream>>>(A);
    }
    return gb_after_launch(ctx, A.mass_only ? "cfl_y" : "y_steps");
}

}  // namespace

extern "C" int gb_advect_y(gb_ctx *ctx, const gb_view *m, const gb_view *rm, const gb_view *rxm,
                           const gb_view *rym, const gb_view *rzm, const gb_view *bm,
                           const gb_view *bm_full, int bm_full_l0, int limits, int max_nloop,
                           int32_t *nloop_out) {
    if (!ctx || !m || !rm || !rxm || !rym || !rzm || !bm) return GB_EARG;
    YArgs A{};
    A.m = dv(m);
    A.q[0] = dv(rm); A.q[1] = dv(rxm); A.q[2] = dv(rym); A.q[3] = dv(rzm);
    A.bm = dv(bm);
    A.full = bm_full ? dv(bm_full) : DV{};
    A.full_l0 = bm_full_l0;
    A.im = (int)m->n[0]; A.jm = (int)m->n[1]; A.lm = (int)m->n[2]; A.nt = (int)rm->n[3];
    if (bm->n[1] != A.jm + 1) {
        gb_set_error("gb_advect_y: bm must have jm+1 faces");
        return GB_EARG;
    }
    A.limits = limits; A.nmax = max_nloop - 1;
    A.nloop_out = nloop_out;
    A.ctl = ctx->ctl;
    A.mass_only = 0;
    return launch_y(ctx, A);
}

extern "C" int gb_cfl_y(gb_ctx *ctx, const gb_view *m, const gb_view *bm, int max_nloop) {
    if (!ctx || !m || !bm) return GB_EARG;
    YArgs A{};
    A.m = dv(m);
    for (int w = 0; w < 4; ++w) A.q[w] = A.m;
    A.bm = dv(bm);
    A.full = DV{};
    A.im = (int)m->n[0]; A.jm = (int)m->n[1]; A.lm = (int)m->n[2]; A.nt = 0;
    A.limits = 0;
    A.nmax = max_nloop;  // dynamvm gives up once nloop would exceed max_nloop (cfl.py:175)
    A.ctl = ctx->ctl;
    A.mass_only = 1;
    return launch_y(ctx, A);
}
