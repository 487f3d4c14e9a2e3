// convec: implicit convection with Kzz diffusion folded into one matrix per column, inverted
// by Crout LU without pivoting, applied to the tracer mass and (by its diagonal) the slopes.
//
// Two launches, shaped so that the FP64 pipe -- this GPU's scarcest unit -- issues with its
// lanes full:
//   k_convec_lu     one warp per owned column, the matrix in shared memory: the updraft and
//                   downdraft chains, the per-level quotients (each division once, lanes across
//                   levels), f and conv1 = I - dt (f(k-1) - f(k)), Crout LU column by column
//                   with the rows a term updates packed onto the lanes, and L^-1 by forward
//                   substitution (row k's terms applied to every later row at once, the
//                   (row, column) elements packed onto the lanes).  U goes to a work space, L^-1
//                   to the inverse's place.
//   k_convec_apply  one thread per (column, column of the inverse): the back substitution
//                   U X = L^-1 of its column of the inverse; then, whole columns per block, one
//                   thread per (column, level): the slopes times the inverse's diagonal and
//                   rm = C rm accumulated in k.
// The reference's operation order is kept element by element -- every element receives its
// terms in the same k order as in the row-by-row form -- and work is skipped only where a
// multiplier is exactly zero (the same skips as the reference's own zero tests would leave
// bitwise: x - w * y with w = +-0 returns x unless x is a zero, and the accumulators of the
// substitutions are never -0).  Above the cloud the matrix is tridiagonal (diffusion only), so
// most of the O(n^3) inverse becomes O(n^2).
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
constexpr int NMAX = 64;

struct CArgs {
    DV m, q[4];
    DV entu, detu, entd, detd, dkg;
    const int32_t *top, *lfs;
    int64_t ts0, ts1;
    const int32_t *cols;  // (i, j) pairs
    int ncol, n, nt;
    double dt;
    double *inv;         // ncol * n * n: the inverses (the cache's, or the work space's)
    double *ubuf;        // ncol * n * n work space: U of the columns factorised in this call
    int32_t *fresh;      // ncol work space: 1 where this call factorised the column
    double *cache_m;     // ncol * n, or null (no reuse)
    int32_t *cache_tag;  // ncol
    const int32_t *epoch;
    int cols_per_block;  // k_convec_apply: whole columns of n threads
};

__device__ __forceinline__ double &AT(const DV &v, int64_t i, int64_t j, int64_t l) {
    return v.p[i * v.s0 + j * v.s1 + l * v.s2];
}
__device__ __forceinline__ double &AT4(const DV &v, int64_t i, int64_t j, int64_t l, int64_t t) {
    return v.p[i * v.s0 + j * v.s1 + l * v.s2 + t * v.s3];
}
__device__ __forceinline__ double max0(double x) { return isnan(x) ? x : (0.0 > x ? 0.0 : x); }

// shared memory of one warp (doubles): A n*n (conv1, then LU), Y (n+1)*n (f, then L^-1), vectors
// m, amu, amd, zu, zd and the quotients qeu, qed, qamu, qamd, qdk1, qdk2 (n+1 each)
__host__ __device__ __forceinline__ size_t warp_doubles(int n) {
    return (size_t)n * n + (size_t)(n + 1) * n + 11 * (size_t)(n + 1);
}

__global__ void __launch_bounds__(WARPS * 32) k_convec_lu(CArgs A) {
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
    double *qeu = zd + (n + 1), *qed = qeu + (n + 1), *qamu = qed + (n + 1), *qamd = qamu + (n + 1);
    double *qdk1 = qamd + (n + 1), *qdk2 = qdk1 + (n + 1);
    const int i = A.cols[2 * c], j = A.cols[2 * c + 1];

    for (int l = lane; l < n; l += 32) mc[l] = AT(A.m, i, j, l);
    __syncwarp();

    // ---- the kept inverse, when this column's inputs are bitwise those it was made from
    if (A.cache_m) {
        const double *cm = A.cache_m + (size_t)c * n;
        bool same = A.cache_tag[c] == *A.epoch;
        for (int l = lane; l < n; l += 32)
            same = same && (__double_as_longlong(cm[l]) == __double_as_longlong(mc[l]));
        if (__all_sync(FULL_MASK, same)) {
            if (lane == 0) A.fresh[c] = 0;
            return;
        }
    }

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
    // ---- every division of the matrix once, lanes across levels k = 1..n
    for (int k = 1 + lane; k <= n; k += 32) {
        qeu[k] = AT(A.entu, i, j, k - 1) / mc[k - 1];
        qed[k] = -AT(A.entd, i, j, k - 1) / mc[k - 1];
        if (k <= n - 1) {
            qamu[k] = amu[k] / mc[k];
            qamd[k] = amd[k] / mc[k - 1];
            qdk1[k] = AT(A.dkg, i, j, k - 1) / mc[k - 1];
            qdk2[k] = AT(A.dkg, i, j, k - 1) / mc[k];
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
                v = act ? qed[k] * z : 0.0;
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
                u = act ? qeu[k] * z : 0.0;
            else
                u = 0.0;
            if (k <= n - 1) {
                double f = u + Y[(size_t)k * n + l];
                if (l == k) f = f - qamu[k];
                if (l == k - 1) {
                    f = f - qamd[k];
                    f = f + qdk1[k];
                }
                if (l == k) f = f - qdk2[k];
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
    // ---- Crout LU, column by column: column cj receives the terms k = 0..cj-1 in order, each on
    // the rows below k (packed onto the lanes); then its part below the diagonal / the diagonal
    for (int cj = 0; cj < n; ++cj) {
        for (int k = 0; k < cj; ++k) {
            const double v = LU[(size_t)k * n + cj];  // U(k, cj), final
            if (v == 0.0) continue;                   // warp-uniform
            for (int r = k + 1 + lane; r < n; r += 32) LU[(size_t)r * n + cj] = LU[(size_t)r * n + cj] - LU[(size_t)r * n + k] * v;
            __syncwarp();
        }
        const double d = LU[(size_t)cj * n + cj];
        for (int r = cj + 1 + lane; r < n; r += 32) LU[(size_t)r * n + cj] = LU[(size_t)r * n + cj] / d;
        __syncwarp();
    }
    // ---- forward substitution of the identity: Y = L^-1.  Row k is final once the terms of
    // rows < k are in; its term then goes to every later row r with L(r, k) != 0 at once, the
    // (r, column <= k) elements packed onto the lanes -- each element still in k order.
    for (int e = lane; e < n * n; e += 32) Y[e] = (e / n == e % n) ? 1.0 : 0.0;
    __syncwarp();
    for (int k = 0; k < n - 1; ++k) {
        // the rows below k with a non-zero multiplier, in order
        uint32_t rows0 = __ballot_sync(FULL_MASK, k + 1 + lane < n && LU[(size_t)(k + 1 + lane) * n + k] != 0.0);
        uint32_t rows1 = __ballot_sync(FULL_MASK, k + 33 + lane < n && LU[(size_t)(k + 33 + lane) * n + k] != 0.0);
        const int nr = __popc(rows0) + __popc(rows1);
        if (nr == 0) continue;
        const int w = k + 1;  // the columns 0..k
        for (int e = lane; e < nr * w; e += 32) {
            int q = e / w;
            const int col = e % w;
            // the q-th set bit of (rows1:rows0)
            int r;
            const int n0 = __popc(rows0);
            if (q < n0) {
                uint32_t b = rows0;
                for (int s = 0; s < q; ++s) b &= b - 1;
                r = k + 1 + __ffs(b) - 1;
            } else {
                uint32_t b = rows1;
                for (int s = 0; s < q - n0; ++s) b &= b - 1;
                r = k + 33 + __ffs(b) - 1;
            }
            Y[(size_t)r * n + col] = Y[(size_t)r * n + col] - LU[(size_t)r * n + k] * Y[(size_t)k * n + col];
        }
        __syncwarp();
    }
    // ---- out: U (the upper triangle with the diagonal) and L^-1; the air mass it is made from
    double *U = A.ubuf + (size_t)c * n * n, *X = A.inv + (size_t)c * n * n;
    for (int e = lane; e < n * n; e += 32) {
        U[e] = LU[e];
        X[e] = Y[e];
    }
    if (lane == 0) A.fresh[c] = 1;
    if (A.cache_m) {
        for (int l = lane; l < n; l += 32) A.cache_m[(size_t)c * n + l] = mc[l];
        if (lane == 0) A.cache_tag[c] = *A.epoch;
    }
}

__global__ void k_convec_apply(CArgs A) {
    const int n = A.n;
    const int cl = threadIdx.x / n, x = threadIdx.x % n;  // column in the block, its thread
    const int c = blockIdx.x * A.cols_per_block + cl;
    const bool live = cl < A.cols_per_block && c < A.ncol;
    double *X = live ? A.inv + (size_t)c * n * n : nullptr;
    // ---- back substitution of inverse column x: rows from the bottom, terms k in order
    if (live && A.fresh[c]) {
        const double *U = A.ubuf + (size_t)c * n * n;
        for (int r = n - 1; r >= 0; --r) {
            double a = X[(size_t)r * n + x];
            for (int k = r + 1; k < n; ++k) {
                const double w = U[(size_t)r * n + k];
                if (w == 0.0) continue;
                a = a - w * X[(size_t)k * n + x];
            }
            X[(size_t)r * n + x] = a / U[(size_t)r * n + r];
        }
    }
    __syncthreads();
    // ---- apply: the slopes times the diagonal; rm(l) = sum over k of C(l, k) rm(k), in k order.
    // Threads without a column stay for the block's barriers.
    const int l = x;
    const int i = live ? A.cols[2 * c] : 0, j = live ? A.cols[2 * c + 1] : 0;
    const double *C = live ? X + (size_t)l * n : nullptr;
    if (live) {
        const double dg = C[l];
        for (int w = 1; w < 4; ++w)
            for (int t = 0; t < A.nt; ++t) AT4(A.q[w], i, j, l, t) = dg * AT4(A.q[w], i, j, l, t);
    }
    for (int t = 0; t < A.nt; ++t) {
        double zr = 0.0;
        if (live)
            for (int k = 0; k < n; ++k) zr = zr + C[k] * AT4(A.q[0], i, j, k, t);
        __syncthreads();  // every thread of the column has read rm(., t)
        if (live) AT4(A.q[0], i, j, l, t) = zr;
    }
}

int gcd(int a, int b) { return b == 0 ? a : gcd(b, a % b); }

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
    const size_t nn = (size_t)lmax * lmax;
    // work space: U of every column, the fresh flags, and the inverses when there is no cache
    const size_t doubles = nn * ncol + ((size_t)ncol + 1) / 2 + (cache_inv ? 0 : nn * ncol);
    double *w = gb_work(ctx, doubles * sizeof(double));
    if (!w) return GB_ECUDA;
    A.ubuf = w;
    A.fresh = reinterpret_cast<int32_t *>(w + nn * ncol);
    A.inv = cache_inv ? cache_inv : w + nn * ncol + ((size_t)ncol + 1) / 2;
    A.cache_m = cache_inv ? cache_m : nullptr;
    A.cache_tag = cache_tag;
    A.epoch = epoch;
    const size_t smem = (size_t)WARPS * warp_doubles(lmax) * sizeof(double);
    GB_CHECK_CUDA(cudaFuncSetAttribute(k_convec_lu, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_convec_lu<<<(ncol + WARPS - 1) / WARPS, WARPS * 32, smem, ctx->stream>>>(A);
    if (int rc = gb_after_launch(ctx, "convec_lu")) return rc;
    // whole columns per block, as many as make the block a whole number of warps (<= 1024 threads)
    int per = 32 / gcd(lmax, 32);
    while (per > 1 && per * lmax > 1024) per /= 2;
    if (per * lmax < 128) per = (128 + lmax - 1) / lmax;
    A.cols_per_block = per;
    const int threads = ((per * lmax + 31) / 32) * 32;
    k_convec_apply<<<(ncol + per - 1) / per, threads, 0, ctx->stream>>>(A);
    return gb_after_launch(ctx, "convec_apply");
}
