// The adjoint of the tracer operators of a region-1 step with unlimited slopes: dynamv and
// dynamw (the transposes of their sub-steps, gb_adjoint.cuh), convection (the transpose of
// rm = C rm and the slopes times C's diagonal), and the surface-flux gradient of the emission.
// Chemistry at fixed OH multiplies every tracer moment by a per-cell decay, so it is its own
// transpose: the adjoint applies gb_chemistry itself to the adjoints.
//
// Each kernel reads the air mass and fluxes the forward operator saw (taped by the host when it
// recomputes a stretch of steps from a checkpoint) and overwrites the tracer adjoints (one
// tracer) with the adjoints before the operator.
// Reference: pydyn kernels.py:223-291 (dynamv), :295-346 (dynamw), :423-457 (convec),
// zoom/physics.py:33-78 (convec_region, sources_region, chemistry_region).
#include "gb_adjoint.cuh"
#include "gb_common.cuh"

namespace {

constexpr int WARPS = 4;

__device__ __forceinline__ double &AT(const DV &v, int64_t i, int64_t j, int64_t l) {
    return v.p[i * v.s0 + j * v.s1 + l * v.s2];
}

struct LineArgs {
    DV m, f, q[4];    // mass, faces, adjoints (rm, along slope, cross A, cross B) as (i, j, l)
    int ni, nj, nl;   // mass extents
    const int32_t *nloop;  // dynamv: per level; dynamw: one
    int ncell;
    gb_ctl *ctl;
};

// dynamv: one warp per (i, l) column of jm cells, faces 0..jm (the polar ones zero); the layer's
// nloop and its progressively rescaled faces, as k_y_steps rescales them
__global__ void __launch_bounds__(WARPS * 32) k_adj_y(LineArgs A) {
    extern __shared__ double smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t col = (int64_t)blockIdx.x * WARPS + warp;
    if (col >= (int64_t)A.ni * A.nl) return;
    const int i = (int)(col / A.nl), l = (int)(col % A.nl);
    const int n = A.nj, NC = A.ncell;
    const int nloop = A.nloop[l];
    if (nloop < 1) {
        if (lane == 0) raise_status(A.ctl, GB_EARG);
        return;
    }
    const AdjLine L = adj_line(smem + (size_t)warp * adj_doubles_per_line(NC), NC);
    for (int k = lane; k <= n; k += GB_WARP) L.a[k] = progressive_chain(AT(A.f, i, k, l), nloop);
    for (int k = lane; k < n; k += GB_WARP) {
        L.m0[k] = AT(A.m, i, k, l);
        for (int w = 0; w < 4; ++w) L.q[w][k] = AT(A.q[w], i, k, l);
    }
    __syncwarp();
    adj_line_substeps(L, n, nloop, LINE_POLAR, false, lane);
    for (int k = lane; k < n; k += GB_WARP)
        for (int w = 0; w < 4; ++w) AT(A.q[w], i, k, l) = L.q[w][k];
}

// dynamw: one warp per (i, j) column of lm cells, interfaces 0..lm (the outer ones zero), cm / n
__global__ void __launch_bounds__(WARPS * 32) k_adj_z(LineArgs A) {
    extern __shared__ double smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t col = (int64_t)blockIdx.x * WARPS + warp;
    if (col >= (int64_t)A.ni * A.nj) return;
    const int i = (int)(col / A.nj), j = (int)(col % A.nj);
    const int n = A.nl, NC = A.ncell;
    const int nz = A.nloop[0];
    if (nz < 1) {
        if (lane == 0) raise_status(A.ctl, GB_EARG);
        return;
    }
    const AdjLine L = adj_line(smem + (size_t)warp * adj_doubles_per_line(NC), NC);
    for (int k = lane; k <= n; k += GB_WARP) L.a[k] = AT(A.f, i, j, k) / (double)nz;
    for (int k = lane; k < n; k += GB_WARP) {
        L.m0[k] = AT(A.m, i, j, k);
        for (int w = 0; w < 4; ++w) L.q[w][k] = AT(A.q[w], i, j, k);
    }
    __syncwarp();
    adj_line_substeps(L, n, nz, LINE_CLOSED, false, lane);
    for (int k = lane; k < n; k += GB_WARP)
        for (int w = 0; w < 4; ++w) AT(A.q[w], i, j, k) = L.q[w][k];
}

// convection: thread per (column, level k) in blocks of whole columns.  rm_b(k) <- sum over l
// of C(l, k) rm_b(l) (in l order), the slopes' adjoints times C(k, k); levels >= n untouched.
struct VArgs {
    DV q[4];
    const double *inv;     // ncol * n * n, C(l, k) at l * n + k
    const int32_t *cols;   // (i, j) pairs
    int ncol, n, per;
};

__global__ void k_adj_convec(VArgs A) {
    const int n = A.n;
    const int cl = threadIdx.x / n, k = threadIdx.x % n;
    const int c = blockIdx.x * A.per + cl;
    const bool live = cl < A.per && c < A.ncol;
    const int i = live ? A.cols[2 * c] : 0, j = live ? A.cols[2 * c + 1] : 0;
    const double *X = live ? A.inv + (size_t)c * n * n : nullptr;
    double acc = 0.0;
    if (live) {
        for (int l = 0; l < n; ++l) acc = acc + X[(size_t)l * n + k] * AT(A.q[0], i, j, l);
        const double dg = X[(size_t)k * n + k];
        for (int w = 1; w < 4; ++w) AT(A.q[w], i, j, k) = dg * AT(A.q[w], i, j, k);
    }
    __syncthreads();  // every thread of the column has read rm_b
    if (live) AT(A.q[0], i, j, k) = acc;
}

int gcd(int a, int b) { return b == 0 ? a : gcd(b, a % b); }

// emission: d J / d flux(i, j) += area(j) scale (rm_b(i, j, level) - rzm_b(i, j, level)) on the
// owned columns (x = flux area scale is added to rm and taken from rzm)
__global__ void k_adj_sources(DV rm, DV rzm, DV grad, const double *area, double scale, int level,
                              const int32_t *cols, int ncol) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncol) return;
    const int i = cols[2 * c], j = cols[2 * c + 1];
    const double d = AT(rm, i, j, level) - AT(rzm, i, j, level);
    double &g = grad.p[(int64_t)i * grad.s0 + (int64_t)j * grad.s1];
    g = g + (area[j] * scale) * d;
}

LineArgs line_args(gb_ctx *ctx, const gb_view *m, const gb_view *f, const gb_view *const *q, const int32_t *nloop) {
    LineArgs A{};
    A.m = dv(m);
    A.f = dv(f);
    for (int w = 0; w < 4; ++w) A.q[w] = dv(q[w]);
    A.ni = (int)m->n[0]; A.nj = (int)m->n[1]; A.nl = (int)m->n[2];
    A.nloop = nloop;
    A.ctl = ctx->ctl;
    return A;
}

}  // namespace

extern "C" int gb_adjoint_y(gb_ctx *ctx, const gb_view *m, const gb_view *rm_b, const gb_view *rxm_b,
                            const gb_view *rym_b, const gb_view *rzm_b, const gb_view *bm, const int32_t *nloop) {
    if (!ctx || !m || !rm_b || !rxm_b || !rym_b || !rzm_b || !bm || !nloop) return GB_EARG;
    if (bm->n[0] != m->n[0] || bm->n[1] != m->n[1] + 1 || bm->n[2] != m->n[2]) {
        gb_set_error("gb_adjoint_y: bm must be (im, jm+1, lm) over m's (im, jm, lm)");
        return GB_EARG;
    }
    const gb_view *q[4] = {rm_b, rym_b, rxm_b, rzm_b};  // along slope rym, cross rxm (kept at the poles), rzm
    LineArgs A = line_args(ctx, m, bm, q, nloop);
    A.ncell = A.nj + 2;
    const size_t smem = (size_t)WARPS * 15 * A.ncell * sizeof(double);
    const int64_t cols = (int64_t)A.ni * A.nl;
    if (cols == 0) return GB_OK;
    GB_CHECK_CUDA(cudaFuncSetAttribute(k_adj_y, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_adj_y<<<(unsigned)((cols + WARPS - 1) / WARPS), WARPS * 32, smem, ctx->stream>>>(A);
    return gb_after_launch(ctx, "adjoint_y");
}

extern "C" int gb_adjoint_z(gb_ctx *ctx, const gb_view *m, const gb_view *rm_b, const gb_view *rxm_b,
                            const gb_view *rym_b, const gb_view *rzm_b, const gb_view *cm, const int32_t *n_advz) {
    if (!ctx || !m || !rm_b || !rxm_b || !rym_b || !rzm_b || !cm || !n_advz) return GB_EARG;
    if (cm->n[0] != m->n[0] || cm->n[1] != m->n[1] || cm->n[2] != m->n[2] + 1) {
        gb_set_error("gb_adjoint_z: cm must be (im, jm, lm+1) over m's (im, jm, lm)");
        return GB_EARG;
    }
    const gb_view *q[4] = {rm_b, rzm_b, rxm_b, rym_b};  // along slope rzm, cross rxm, rym
    LineArgs A = line_args(ctx, m, cm, q, n_advz);
    A.ncell = A.nl + 2;
    const size_t smem = (size_t)WARPS * 15 * A.ncell * sizeof(double);
    const int64_t cols = (int64_t)A.ni * A.nj;
    if (cols == 0) return GB_OK;
    GB_CHECK_CUDA(cudaFuncSetAttribute(k_adj_z, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_adj_z<<<(unsigned)((cols + WARPS - 1) / WARPS), WARPS * 32, smem, ctx->stream>>>(A);
    return gb_after_launch(ctx, "adjoint_z");
}

extern "C" int gb_adjoint_convec(gb_ctx *ctx, const gb_view *rm_b, const gb_view *rxm_b, const gb_view *rym_b,
                                 const gb_view *rzm_b, const double *inv, const int32_t *cols, int ncol, int lmax) {
    if (!ctx || !rm_b || !rxm_b || !rym_b || !rzm_b || !inv || (ncol > 0 && !cols)) return GB_EARG;
    if (lmax < 1 || lmax > rm_b->n[2] || lmax > 1024) {
        gb_set_error("gb_adjoint_convec: 1 <= lmax <= levels");
        return GB_EARG;
    }
    if (ncol <= 0) return GB_OK;
    VArgs A{};
    A.q[0] = dv(rm_b); A.q[1] = dv(rxm_b); A.q[2] = dv(rym_b); A.q[3] = dv(rzm_b);
    A.inv = inv; A.cols = cols; A.ncol = ncol; A.n = lmax;
    int per = 32 / gcd(lmax, 32);
    while (per > 1 && per * lmax > 1024) per /= 2;
    if (per * lmax < 128) per = (128 + lmax - 1) / lmax;
    while (per > 1 && ((per * lmax + 31) / 32) * 32 > 1024) --per;
    A.per = per;
    const int threads = ((per * lmax + 31) / 32) * 32;
    k_adj_convec<<<(ncol + per - 1) / per, threads, 0, ctx->stream>>>(A);
    return gb_after_launch(ctx, "adjoint_convec");
}

extern "C" int gb_adjoint_sources(gb_ctx *ctx, const gb_view *rm_b, const gb_view *rzm_b, const gb_view *grad,
                                  const double *area, double scale, int level, const int32_t *cols, int ncol) {
    if (!ctx || !rm_b || !rzm_b || !grad || !area || (ncol > 0 && !cols) || ncol < 0) return GB_EARG;
    if (level < 1 || level > rm_b->n[2]) {
        gb_set_error("gb_adjoint_sources: level (1-based) outside the arrays");
        return GB_EARG;
    }
    if (ncol == 0) return GB_OK;
    k_adj_sources<<<(ncol + 127) / 128, 128, 0, ctx->stream>>>(dv(rm_b), dv(rzm_b), dv(grad), area, scale, level - 1,
                                                                 cols, ncol);
    return gb_after_launch(ctx, "adjoint_sources");
}
