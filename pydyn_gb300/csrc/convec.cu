// convec: implicit convection with Kzz diffusion folded into one matrix per column, inverted
// by Crout LU without pivoting, applied to the tracer mass and (by its diagonal) the slopes.
//
// One warp per owned column; the column's matrix lives in shared memory with lanes across its
// columns (the element l of every row belongs to lane l % 32).  The reference's operation
// order is kept element by element; work is skipped only where a multiplier is exactly zero,
// which leaves every result bit unchanged: the skipped statement is x - w * y with w = +-0,
// which returns x unless x is a zero, and the accumulators of the substitutions are never
// -0 (they start at +0 or 1 and a subtraction yields -0 only from -0 - +0).  The structural
// zeros are many: above the cloud the matrix is tridiagonal (diffusion only), so most of the
// O(n^3) inverse becomes O(n^2).
//
// The inverse of a column is kept (with the air mass it was made from) and reused by the next
// call in the same convection epoch when that air mass is bitwise unchanged -- the two `v` of
// a step's half steps, between which only sources and chemistry (tracers) run.
//
// Reference: pydyn kernels.py:350-396 (convection_matrix), :399-420 (fastminv), :423-457
// (convec), zoom/physics.py:33-52 (convec_region).
#include "gb_common.cuh"

namespace {

constexpr int WARPS = 2;
constexpr int NMAX = 64;  // levels a lane pair can hold

struct CArgs {
    DV m, q[4];
    DV entu, detu, entd, detd, dkg;
    const int32_t *top, *lfs;
    int64_t ts0, ts1;
    const int32_t *cols;  // (i, j) pairs
    int ncol, n, nt;
    double dt;
    double *cache_inv;   // ncol * n * n, or null (no reuse)
    double *cache_m;     // ncol * n
    int32_t *cache_tag;  // ncol
    const int32_t *epoch;
};

__device__ __forceinline__ double &AT(const DV &v, int64_t i, int64_t j, int64_t l) {
    return v.p[i * v.s0 + j * v.s1 + l * v.s2];
}
__device__ __forceinline__ double &AT4(const DV &v, int64_t i, int64_t j, int64_t l, int64_t t) {
    return v.p[i * v.s0 + j * v.s1 + l * v.s2 + t * v.s3];
}
__device__ __forceinline__ double max0(double x) { return isnan(x) ? x : (0.0 > x ? 0.0 : x); }

// shared memory of one warp (doubles): A n*n (conv1, then LU), Y (n+1)*n (f, then L^-1, then
// the inverse), vectors m, amu, amd, zu, zd (n+1 each)
__host__ __device__ __forceinline__ size_t warp_doubles(int n) { return (size_t)n * n + (size_t)(n + 1) * n + 5 * (n + 1); }

__global__ void __launch_bounds__(WARPS * 32) k_convec(CArgs A) {
    extern __shared__ double smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int c = blockIdx.x * WARPS + warp;
    if (c >= A.ncol) return;
    const int n = A.n;
    double *S = smem + (size_t)warp * warp_doubles(n);
    double *LU = S;                    // n x n
    double *Y = LU + (size_t)n * n;    // (n+1) x n
    double *mc = Y + (size_t)(n + 1) * n;
    double *amu = mc + (n + 1), *amd = amu + (n + 1), *zu = amd + (n + 1), *zd = zu + (n + 1);
    const int i = A.cols[2 * c], j = A.cols[2 * c + 1];

    for (int l = lane; l < n; l += 32) mc[l] = AT(A.m, i, j, l);
    __syncwarp();

    // ---- the cached inverse, when this column's inputs are bitwise those it was made from
    bool reuse = false;
    double *cinv = nullptr;
    if (A.cache_inv) {
        cinv = A.cache_inv + (size_t)c * n * n;
        double *cm = A.cache_m + (size_t)c * n;
        bool same = A.cache_tag[c] == *A.epoch;
        for (int l = lane; l < n; l += 32)
            same = same && (__double_as_longlong(cm[l]) == __double_as_longlong(mc[l]));
        reuse = __all_sync(FULL_MASK, same);
    }

    if (reuse) {
        for (int k = lane; k < n * n; k += 32) Y[k] = cinv[k];
        __syncwarp();
    } else {
        const int top = A.top[i * A.ts0 + j * A.ts1], lfs = A.lfs[i * A.ts0 + j * A.ts1];
        // ---- the scalar chains of the updraft (upward) and downdraft (downward); every lane
        // computes them alike, lane 0 stores them
        {
            double mu = 0.0;
            if (lane == 0) amu[0] = 0.0;
            for (int k = 1; k <= n; ++k) {
                const double eu = AT(A.entu, i, j, k - 1), du = AT(A.detu, i, j, k - 1);
                const bool act = top >= k;
                const double a = mu + eu - du;
                const bool up = a > 0.0;
                const double z = up ? max0(1.0 - du / (mu + eu)) : 0.0;
                mu = (act && up) ? a : 0.0;
                if (lane == 0) {
                    amu[k] = mu;
                    zu[k] = act ? z : -1.0;  // -1 marks an inactive level
                }
            }
            double md = 0.0;
            if (lane == 0) {
                amd[n] = 0.0;
                amd[0] = 0.0;
                zd[0] = zd[1] = -1.0;
            }
            for (int k = n; k >= 2; --k) {
                const double ed = AT(A.entd, i, j, k - 1), dd = AT(A.detd, i, j, k - 1);
                const bool act = lfs >= k;
                const double a = md - ed + dd;
                const bool dn = a < 0.0;
                const double z = dn ? max0(1.0 + dd / (md - ed)) : 0.0;
                md = (act && dn) ? a : 0.0;
                if (lane == 0) {
                    amd[k - 1] = md;
                    zd[k] = act ? z : -1.0;
                }
            }
        }
        __syncwarp();
        // ---- f = fd (downward chains per column l), then + fu row by row, then the diagonals
        for (int l = lane; l < n; l += 32) {
            for (int k = 0; k <= n; ++k) Y[(size_t)k * n + l] = 0.0;
            double v = 0.0;  // fd(k-1, l) for k = l+1 down to 2
            for (int k = n; k >= 2; --k) {
                const double z = zd[k];
                const bool act = z >= 0.0;
                if (k - 1 == l)
                    v = act ? -AT(A.entd, i, j, k - 1) / mc[k - 1] * z : 0.0;
                else if (k - 1 < l)
                    v = act ? v * z : 0.0;
                else
                    continue;
                Y[(size_t)(k - 1) * n + l] = v;
            }
        }
        __syncwarp();
        for (int l = lane; l < n; l += 32) {
            double u = 0.0;  // fu(k, l) for k = 1..n
            for (int k = 1; k <= n; ++k) {
                const double z = zu[k];
                const bool act = z >= 0.0;
                if (l < k - 1)
                    u = act ? u * z : 0.0;
                else if (l == k - 1)
                    u = act ? AT(A.entu, i, j, k - 1) / mc[k - 1] * z : 0.0;
                else
                    u = 0.0;
                if (k <= n - 1) {
                    double f = u + Y[(size_t)k * n + l];
                    if (l == k) f = f - amu[k] / mc[k];
                    if (l == k - 1) {
                        f = f - amd[k] / mc[k - 1];
                        f = f + AT(A.dkg, i, j, k - 1) / mc[k - 1];
                    }
                    if (l == k) f = f - AT(A.dkg, i, j, k - 1) / mc[k];
                    Y[(size_t)k * n + l] = f;
                }
            }
        }
        __syncwarp();
        // ---- conv1 = I - dt (f(k-1) - f(k)) into LU
        const double mdt = -A.dt;
        for (int l = lane; l < n; l += 32)
            for (int k = 1; k <= n; ++k) {
                double v = mdt * (Y[(size_t)(k - 1) * n + l] - Y[(size_t)k * n + l]);
                if (l == k - 1) v = v + 1.0;
                LU[(size_t)(k - 1) * n + l] = v;
            }
        __syncwarp();
        // ---- Crout LU, column by column; lanes across rows
        for (int cj = 0; cj < n; ++cj) {
            double c0 = lane < n ? LU[(size_t)lane * n + cj] : 0.0;
            double c1 = lane + 32 < n ? LU[(size_t)(lane + 32) * n + cj] : 0.0;
            for (int k = 0; k < cj; ++k) {
                const double v = __shfl_sync(FULL_MASK, k < 32 ? c0 : c1, k & 31);  // LU(k, cj), final
                if (v == 0.0) continue;  // warp-uniform
                if (lane > k && lane < n) c0 = c0 - LU[(size_t)lane * n + k] * v;
                if (lane + 32 > k && lane + 32 < n) c1 = c1 - LU[(size_t)(lane + 32) * n + k] * v;
            }
            const double d = __shfl_sync(FULL_MASK, cj < 32 ? c0 : c1, cj & 31);
            if (lane > cj && lane < n) c0 = c0 / d;
            if (lane + 32 > cj && lane + 32 < n) c1 = c1 / d;
            if (lane < n) LU[(size_t)lane * n + cj] = c0;
            if (lane + 32 < n) LU[(size_t)(lane + 32) * n + cj] = c1;
            __syncwarp();
        }
        // ---- forward substitution of the identity: Y = L^-1 (lanes across columns)
        for (int r = 0; r < n; ++r) {
            double a0 = (lane == r) ? 1.0 : 0.0, a1 = (lane + 32 == r) ? 1.0 : 0.0;
            for (int k = 0; k < r; ++k) {
                const double w = LU[(size_t)r * n + k];
                if (w == 0.0) continue;
                if (lane <= k) a0 = a0 - w * Y[(size_t)k * n + lane];
                if (lane + 32 <= k) a1 = a1 - w * Y[(size_t)k * n + lane + 32];
            }
            if (lane < n) Y[(size_t)r * n + lane] = a0;
            if (lane + 32 < n) Y[(size_t)r * n + lane + 32] = a1;
            __syncwarp();
        }
        // ---- back substitution: the inverse, rows from the bottom, in place of Y
        for (int r = n - 1; r >= 0; --r) {
            double a0 = lane < n ? Y[(size_t)r * n + lane] : 0.0;
            double a1 = lane + 32 < n ? Y[(size_t)r * n + lane + 32] : 0.0;
            for (int k = r + 1; k < n; ++k) {
                const double w = LU[(size_t)r * n + k];
                if (w == 0.0) continue;
                if (lane < n) a0 = a0 - w * Y[(size_t)k * n + lane];
                if (lane + 32 < n) a1 = a1 - w * Y[(size_t)k * n + lane + 32];
            }
            const double d = LU[(size_t)r * n + r];
            if (lane < n) Y[(size_t)r * n + lane] = a0 / d;
            if (lane + 32 < n) Y[(size_t)r * n + lane + 32] = a1 / d;
            __syncwarp();
        }
        if (A.cache_inv) {
            for (int k = lane; k < n * n; k += 32) cinv[k] = Y[k];
            for (int l = lane; l < n; l += 32) A.cache_m[(size_t)c * n + l] = mc[l];
            if (lane == 0) A.cache_tag[c] = *A.epoch;
        }
    }

    // ---- apply: slopes times the diagonal, rm = C rm accumulated in k (lanes across rows)
    for (int l = lane; l < n; l += 32) {
        const double dg = Y[(size_t)l * n + l];
        for (int w = 1; w < 4; ++w)
            for (int t = 0; t < A.nt; ++t) AT4(A.q[w], i, j, l, t) = dg * AT4(A.q[w], i, j, l, t);
    }
    for (int t = 0; t < A.nt; ++t) {
        double zr0 = 0.0, zr1 = 0.0;
        for (int k = 0; k < n; ++k) {
            const double s = AT4(A.q[0], i, j, k, t);  // every lane reads the same rm(k)
            if (lane < n) zr0 = zr0 + Y[(size_t)lane * n + k] * s;
            if (lane + 32 < n) zr1 = zr1 + Y[(size_t)(lane + 32) * n + k] * s;
        }
        __syncwarp();
        if (lane < n) AT4(A.q[0], i, j, lane, t) = zr0;
        if (lane + 32 < n) AT4(A.q[0], i, j, lane + 32, t) = zr1;
        __syncwarp();
    }
}

}  // namespace

extern "C" int gb_convec(gb_ctx *ctx, const gb_view *m, const gb_view *rm, const gb_view *rxm, const gb_view *rym,
                         const gb_view *rzm, const gb_view *entu, const gb_view *detu, const gb_view *entd,
                         const gb_view *detd, const gb_view *dkg, const int32_t *top, const int32_t *lfs,
                         int64_t ts0, int64_t ts1, const int32_t *cols, int ncol, double dt, int lmax,
                         double *cache_inv, double *cache_m, int32_t *cache_tag, const int32_t *epoch) {
    if (!ctx || !m || !rm || !entu || !dkg || !top || !lfs || !cols) return GB_EARG;
    if (lmax <= 0 || ncol <= 0) return GB_OK;
    if (lmax > NMAX) {
        gb_set_error("gb_convec: at most 64 convection levels");
        return GB_EARG;
    }
    if (cache_inv && (!cache_m || !cache_tag || !epoch)) return GB_EARG;
    CArgs A{};
    A.m = dv(m);
    A.q[0] = dv(rm); A.q[1] = dv(rxm); A.q[2] = dv(rym); A.q[3] = dv(rzm);
    A.entu = dv(entu); A.detu = dv(detu); A.entd = dv(entd); A.detd = dv(detd); A.dkg = dv(dkg);
    A.top = top; A.lfs = lfs; A.ts0 = ts0; A.ts1 = ts1;
    A.cols = cols; A.ncol = ncol; A.n = lmax; A.nt = (int)rm->n[3];
    A.dt = dt;
    A.cache_inv = cache_inv; A.cache_m = cache_m; A.cache_tag = cache_tag; A.epoch = epoch;
    const size_t smem = (size_t)WARPS * warp_doubles(lmax) * sizeof(double);
    GB_CHECK_CUDA(cudaFuncSetAttribute(k_convec, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int blocks = (ncol + WARPS - 1) / WARPS;
    k_convec<<<blocks, WARPS * 32, smem, ctx->stream>>>(A);
    return gb_after_launch(ctx, "convec");
}
