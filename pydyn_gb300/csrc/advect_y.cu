// dynamv: meridional slopes advection, one sub-cycle count per layer.
//
// Two launches.  k_y_search: one CTA per layer runs the layer's CFL search exactly as the
// reference does -- every column of the layer tried at n = 1, 2, ... until all pass -- with
// the progressively rescaled faces recomputed from the untouched bm (the rescale is a fixed
// chain per face), and rescales the faces of the halo'd layer that the columns do not own.
// k_y_steps: one thread per (column, cell) over blocks of whole columns of one layer stages the
// columns in shared memory, runs the layer's sub-steps on chip and writes the columns and their
// faces (rescaled, then times nloop) once.
// Two column kinds:
//   polar  region 1: jm cells, jm+1 faces with the polar ones closed; flow out of a pole cell
//          carries no slope; the pole cells keep rxm and rym
//   held   a child: n cells whose two ends are held (the parent's, put there by put_yedges),
//          n-1 interior faces at shared-memory indices 1 .. n-1
// Reference: pydyn kernels.py:223-291 (advect_y, _advect_layer_y), ops.py:315-341
// (subcycles, _trial), zoom/advect.py:201-226 (_dynamv_region1, _rescale_layer_halo),
// zoom/advect.py:348-412 (_dynamv_child), cfl.py:170-183 (dynamvm) and zoom/check_cfl.py:162-193
// (_dynamvm_child).
#include <atomic>

#include "gb_common.cuh"

namespace {

constexpr int SEARCH_THREADS = 256;
constexpr int STEP_WARPS = 4;

struct YArgs {
    DV m, q[4], bm, full;
    int ni, nc, nl, nt;       // columns (i), cells per column, levels
    int full_l0;              // level of `full` that is bm's level 0
    int own_i0, own_i1, own_j0, own_j1;  // faces of `full` the columns own (inclusive data indices)
    int full_mode;            // 0: chain * nloop outside; 1: * nloop only (a child's dynamvm)
    int limits, nmax;
    int ncell;                // nc + 2
    int tc;                   // tracers staged at once (launch_y)
    int P;                    // k_y_steps: columns (one layer's) per block
    int held;
    int32_t *nloop;           // nl, written by the search
    int32_t *nloop_out;
    gb_ctl *ctl;
    int mass_only;
};

__device__ __forceinline__ double &AT(const DV &v, int64_t i, int64_t j, int64_t l) {
    return v.p[i * v.s0 + j * v.s1 + l * v.s2];
}
__device__ __forceinline__ double &AT4(const DV &v, int64_t i, int64_t j, int64_t l, int64_t t) {
    return v.p[i * v.s0 + j * v.s1 + l * v.s2 + t * v.s3];
}

// the face of shared-memory index k of column (i, l) in bm
__device__ __forceinline__ double &BF(const YArgs &A, int i, int k, int l) {
    return AT(A.bm, i, A.held ? k - 1 : k, l);
}

// One column's trial (ops.py:330-341; zoom/advect.py:366-376): n sub-steps of its mass with the
// faces rescaled n-1 times, the Courant number of each interior face checked before each.
__device__ bool column_trial(const YArgs &A, int i, int l, int n, double *mx, double *bf, int lane) {
    const int nc = A.nc;
    const int k0 = 1, k1 = nc - 1;                              // interior faces
    const int c0 = A.held ? 1 : 0, c1 = A.held ? nc - 1 : nc;  // cells that move
    for (int k = (A.held ? 1 : 0) + lane; k <= (A.held ? nc - 1 : nc); k += GB_WARP)
        bf[k] = progressive_chain(BF(A, i, k, l), n);
    for (int k = lane; k < nc; k += GB_WARP) mx[k] = AT(A.m, i, k, l);
    __syncwarp();
    for (int s = 0; s < n; ++s) {
        bool lok = true;
        for (int k = k0 + lane; k <= k1 - (A.held ? 0 : 0) && k < nc; k += GB_WARP) {
            double f = bf[k];
            double mu = ge_zero(f) ? mx[k - 1] : mx[k];
            lok = lok && cfl_pass(f, mu);
        }
        if (!__all_sync(FULL_MASK, lok)) return false;
        for (int k = c0 + lane; k < c1; k += GB_WARP) mx[k] = (mx[k] + bf[k]) - bf[k + 1];
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
    // every exit writes the layer's count, so that k_y_steps never reads one of an earlier call;
    // a count above nmax leaves the layer untouched
    if (s_abort) {
        if (threadIdx.x == 0) A.nloop[l] = A.nmax + 1;
        return;
    }

    // region 1's polar outer faces must carry nothing (kernels.py:233-234); dynamvm does not check
    if (!A.mass_only && !A.held)
        for (int i = threadIdx.x; i < A.ni; i += SEARCH_THREADS)
            if (AT(A.bm, i, 0, l) != 0.0 || AT(A.bm, i, A.nc, l) != 0.0) s_halo = 1;
    __syncthreads();
    if (s_halo) {
        if (threadIdx.x == 0) {
            A.nloop[l] = A.nmax + 1;
            raise_status(A.ctl, GB_EHALO);
        }
        return;
    }

    int nloop = 1;
    while (true) {
        if (threadIdx.x == 0) s_fail = 0;
        __syncthreads();
        for (int i = warp; i < A.ni; i += nwarps) {
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
    if (nloop > A.nmax || nloop == 1) return;

    // the faces of the halo'd layer outside the columns' own: rescaled and restored alike
    if (A.full.p) {
        const int64_t ni = A.full.n0, nj = A.full.n1;
        const int lf = l + A.full_l0;
        for (int64_t k = threadIdx.x; k < ni * nj; k += SEARCH_THREADS) {
            int64_t fi = k / nj, fj = k % nj;
            bool inside = fi >= A.own_i0 && fi <= A.own_i1 && fj >= A.own_j0 && fj <= A.own_j1;
            if (inside) continue;
            double &b = AT(A.full, fi, fj, lf);
            b = (A.full_mode == 0 ? progressive_chain(b, nloop) : b) * (double)nloop;
        }
    }
}

// ------------------------------------------------------------------ the search, column-parallel
// The same smallest n every column of a layer passes, found with every (i, l) column working at
// once: round 0, each column its own smallest passing n (into coln) and the layer's candidate
// their maximum (integer atomic); round r >= 1, the columns below the layer's candidate try it,
// and one that fails pushes the next candidate to its own next passing n.  A layer's count is
// the first candidate no column moved.  No assumption that passing is monotone in n.
constexpr int YROUNDS = 3;

struct YSearch {
    int32_t *cand;     // [YROUNDS + 1][nl], zeroed
    int32_t *changed;  // [YROUNDS][nl], zeroed
    int32_t *coln;     // [ni][nl]
};

__global__ void __launch_bounds__(STEP_WARPS * 32) k_y_search_cols(YArgs A, YSearch S, int round) {
    extern __shared__ double smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t col = (int64_t)blockIdx.x * STEP_WARPS + warp;
    if (col >= (int64_t)A.ni * A.nl) return;
    if (A.mass_only && __shfl_sync(FULL_MASK, *(volatile int *)&A.ctl->cfl_failed, 0)) return;
    const int i = (int)(col / A.nl), l = (int)(col % A.nl);
    if (round >= 2 && !S.changed[(round - 1) * A.nl + l]) return;  // the layer has settled
    double *mx = smem + (size_t)warp * 2 * A.ncell;
    double *bf = mx + A.ncell;
    int n;
    if (round == 0) {
        n = 1;
        while (n <= A.nmax && !column_trial(A, i, l, n, mx, bf, lane)) ++n;
        if (lane == 0) {
            S.coln[col] = n;
            atomicMax(&S.cand[1 * A.nl + l], n);
        }
        return;
    }
    const int cand = S.cand[round * A.nl + l];
    if (cand > A.nmax || S.coln[col] == cand) return;
    if (column_trial(A, i, l, cand, mx, bf, lane)) {
        if (lane == 0) S.coln[col] = cand;
        return;
    }
    n = cand + 1;
    while (n <= A.nmax && !column_trial(A, i, l, n, mx, bf, lane)) ++n;
    if (lane == 0) {
        S.coln[col] = n;
        atomicMax(&S.cand[(round + 1) * A.nl + l], n);
        atomicExch(&S.changed[round * A.nl + l], 1);
    }
}

// one CTA per layer: the layer's settled count (or the errors), then the faces of the halo'd
// layer outside the columns' own, rescaled and restored alike (as k_y_search does)
__global__ void __launch_bounds__(SEARCH_THREADS) k_y_search_done(YArgs A, YSearch S) {
    __shared__ int s_nloop;
    __shared__ int s_halo;
    const int l = blockIdx.x;
    if (threadIdx.x == 0) s_halo = 0;
    __syncthreads();
    // region 1's polar outer faces must carry nothing (kernels.py:233-234), checked before the
    // count as the reference does; dynamvm does not check
    if (!A.mass_only && !A.held)
        for (int i = threadIdx.x; i < A.ni; i += SEARCH_THREADS)
            if (AT(A.bm, i, 0, l) != 0.0 || AT(A.bm, i, A.nc, l) != 0.0) s_halo = 1;
    __syncthreads();
    if (threadIdx.x == 0) {
        int nloop = -1;
        if (s_halo) {
            nloop = A.nmax + 1;
            raise_status(A.ctl, GB_EHALO);
        } else if (A.mass_only && *(volatile int *)&A.ctl->cfl_failed) {
            nloop = A.nmax + 1;
        } else {
            for (int r = 1; r < YROUNDS; ++r)
                if (!S.changed[r * A.nl + l]) {
                    nloop = S.cand[r * A.nl + l];
                    break;
                }
            if (nloop < 0) {  // did not settle in its rounds
                nloop = A.nmax + 1;
                raise_status(A.ctl, GB_ESEARCH);
            } else if (nloop > A.nmax) {
                if (A.mass_only)
                    atomicExch(&A.ctl->cfl_failed, 1);
                else
                    raise_status(A.ctl, GB_ECFL);
            }
            if (A.nloop_out) A.nloop_out[l] = nloop;
        }
        A.nloop[l] = nloop;
        s_nloop = nloop;
    }
    __syncthreads();
    const int nloop = s_nloop;
    if (nloop > A.nmax || nloop == 1 || !A.full.p) return;
    const int64_t ni = A.full.n0, nj = A.full.n1;
    const int lf = l + A.full_l0;
    for (int64_t k = threadIdx.x; k < ni * nj; k += SEARCH_THREADS) {
        int64_t fi = k / nj, fj = k % nj;
        bool inside = fi >= A.own_i0 && fi <= A.own_i1 && fj >= A.own_j0 && fj <= A.own_j1;
        if (inside) continue;
        double &b = AT(A.full, fi, fj, lf);
        b = (A.full_mode == 0 ? progressive_chain(b, nloop) : b) * (double)nloop;
    }
}

// Lines per block of k_y_steps for columns of nc cells: P = 32 / gcd(nc, 32), halved while the
// block exceeds YMAX_THREADS -- a whole number of warps where it fits (8 held columns of 70
// cells are 17.5 warps of which the last is half full, against 70 cells on 3 warps of 32)
constexpr int YMAX_THREADS = 576;  // two blocks an SM at <= 56 registers a thread
int y_lines_per_block(int nc) {
    int g = 32, a = nc;
    while (a % 2 == 0 && g > 1) { a /= 2; g /= 2; }  // g = 32 / gcd(nc, 32)
    int P = g;
    while (P > 1 && P * nc > YMAX_THREADS) P /= 2;
    return P;
}

// One thread per (column, cell) over blocks of P columns of one layer (so the layer's nloop is
// the block's): each block stages its columns in shared memory, runs the layer's sub-steps on
// chip and writes the columns and their faces (rescaled, then times nloop) once.  A column's
// threads meet at block barriers; the faces are staged and written back spread over the
// block's threads.
template <bool MASS_ONLY>
__global__ void __launch_bounds__(YMAX_THREADS, 2) k_y_steps(YArgs A) {
    extern __shared__ double smem[];
    __shared__ int s_skip;
    const int nc = A.nc, P = A.P, NC = A.ncell;
    const int bpl = (A.ni + P - 1) / P;  // blocks per layer
    const int l = blockIdx.x / bpl, i0 = (blockIdx.x % bpl) * P;
    const int nlines = min(P, A.ni - i0);
    const int p = threadIdx.x / nc, k = threadIdx.x % nc;  // the block's column, the thread's cell
    const bool live = p < nlines;
    const int i = i0 + p;
    if (threadIdx.x == 0) s_skip = MASS_ONLY && *(volatile int *)&A.ctl->cfl_failed;  // block-uniform
    __syncthreads();
    if (s_skip) return;
    const int nloop = A.nloop[l];
    if (nloop > A.nmax) return;
    const bool held = A.held != 0;
    const int nt = MASS_ONLY ? 0 : A.nt;
    const int tc = MASS_ONLY ? 0 : A.tc;  // tracers staged at once (a chunk)
    const int kf0 = held ? 1 : 0, kf1 = held ? nc - 1 : nc;  // faces held in smem (inclusive)
    const int c0 = held ? 1 : 0, c1 = held ? nc - 1 : nc;    // cells that move
    const int nf = kf1 - kf0 + 1;
    const bool moves = live && k >= c0 && k < c1;
    const size_t per = (size_t)NC * (3 + 8 * tc);  // doubles of one column's shared memory
    double *m_s = smem + p * per;
    double *b_s = m_s + NC;
    double *m0_s = b_s + NC;           // the staged mass, each chunk's start
    double *q_s = m0_s + NC;           // [4][tc]: rm, rxm, rym, rzm
    double *f_s = q_s + 4 * tc * NC;   // [4][tc]: f, pf, fx, fz
    auto Q = [&](int w, int t) { return q_s + (size_t)(w * tc + t) * NC; };
    auto F = [&](int w, int t) { return f_s + (size_t)(w * tc + t) * NC; };

    for (int e = threadIdx.x; e < nlines * nf; e += blockDim.x) {  // every column's faces
        const int q = e / nf, kk = kf0 + e % nf;
        smem[q * per + NC + kk] = progressive_chain(BF(A, i0 + q, kk, l), nloop);
    }
    if (live) {
        m_s[k] = AT(A.m, i, k, l);
        m0_s[k] = m_s[k];
    }
    __syncthreads();

    if constexpr (MASS_ONLY) {  // dynamvm: the layer's nloop advances, then b * nloop
        for (int s = 0; s < nloop; ++s)  // each thread its own cell
            if (moves) m_s[k] = (m_s[k] + b_s[k]) - b_s[k + 1];
        if (moves) AT(A.m, i, k, l) = m_s[k];
        if (nloop > 1)
            for (int e = threadIdx.x; e < nlines * nf; e += blockDim.x) {
                const int q = e / nf, kk = kf0 + e % nf;
                BF(A, i0 + q, kk, l) = smem[q * per + NC + kk] * (double)nloop;
            }
    } else {
        // the tracers, tc at a time: each chunk restarts from the staged mass and repeats the same
        // mass updates; tracers never mix, so the chunking changes no value
        for (int t0 = 0; t0 < nt; t0 += tc) {
            const int ntc = min(tc, nt - t0);
            if (live) {
                m_s[k] = m0_s[k];
                for (int w = 0; w < 4; ++w)
                    for (int t = 0; t < ntc; ++t) Q(w, t)[k] = AT4(A.q[w], i, k, l, t0 + t);
                if (A.limits)  // every cell of the column, the poles / held ends included
                    for (int t = 0; t < ntc; ++t) Q(2, t)[k] = np_limit(Q(2, t)[k], Q(0, t)[k]);
                if (!held && k == 0)  // closed polar faces
                    for (int w = 0; w < 4; ++w)
                        for (int t = 0; t < ntc; ++t) F(w, t)[0] = F(w, t)[nc] = 0.0;
            }
            __syncthreads();

            for (int s = 0; s < nloop; ++s) {
                if (live && k >= 1) {  // the interior faces 1 .. nc-1
                    const double bk = b_s[k];
                    const int up = ge_zero(bk) ? k - 1 : k;
                    const double beta = div_ip(bk, m_s[up]);
                    for (int t = 0; t < ntc; ++t) {
                        double f, pf, fx, fz;
                        // the along slope is rym, the cross slopes rxm, rzm
                        slopes_flux(bk, beta, Q(0, t)[up], Q(2, t)[up], Q(1, t)[up], Q(3, t)[up], f, pf, fx, fz);
                        if (!held) {  // flow out of a pole cell carries no slope (Fortran faces 2 and jmr)
                            if (k == 1 && ge_zero(bk)) {
                                f = beta * Q(0, t)[0];
                                pf = (-3.0 * bk) * f;
                                fx = 0.0;
                                fz = beta * Q(3, t)[0];
                            }
                            if (k == nc - 1 && lt_zero(bk)) {
                                f = beta * Q(0, t)[nc - 1];
                                pf = (-3.0 * bk) * f;
                                fx = 0.0;
                                fz = beta * Q(3, t)[nc - 1];
                            }
                        }
                        F(0, t)[k] = f; F(1, t)[k] = pf; F(2, t)[k] = fx; F(3, t)[k] = fz;
                    }
                }
                __syncthreads();
                if (moves) {
                    const int j = k;
                    const double mo = m_s[j], blo = b_s[j], bhi = b_s[j + 1];
                    const double mn = (mo + blo) - bhi;
                    const double inv = div_ip(1.0, mn);  // production dynamv hoists the reciprocal
                    const double fc = blo - bhi;
                    const double fm = 3.0 * (blo + bhi);
                    const double mx3 = 3.0 * mo;
                    const bool pole = !held && ((j == 0) || (j == nc - 1));
                    for (int t = 0; t < ntc; ++t) {
                        const double *f = F(0, t), *pf = F(1, t), *fx = F(2, t), *fz = F(3, t);
                        // region 1: rm - (f(j+1) - f(j)); a child: rm + (f(j) - f(j+1))
                        const double rmn = held ? Q(0, t)[j] + (f[j] - f[j + 1]) : Q(0, t)[j] - (f[j + 1] - f[j]);
                        const double ry = Q(2, t)[j];
                        double ryn = ry + ((((pf[j] - pf[j + 1]) - fc * ry) + fm * rmn) - mx3 * (f[j] + f[j + 1])) * inv;
                        if (A.limits) ryn = np_limit(ryn, rmn);
                        const double rx = Q(1, t)[j], rz = Q(3, t)[j];
                        const double rxn = held ? rx + (fx[j] - fx[j + 1]) : rx - (fx[j + 1] - fx[j]);
                        Q(3, t)[j] = held ? rz + (fz[j] - fz[j + 1]) : rz - (fz[j + 1] - fz[j]);
                        Q(0, t)[j] = rmn;
                        if (!pole) {  // the poles keep rxm, rym (only rm, rzm are updated there)
                            Q(2, t)[j] = ryn;
                            Q(1, t)[j] = rxn;
                        }
                    }
                    m_s[j] = mn;
                }
                __syncthreads();
            }
            if (moves)
                for (int w = 0; w < 4; ++w)
                    for (int t = 0; t < ntc; ++t) AT4(A.q[w], i, k, l, t0 + t) = Q(w, t)[k];
            if (live && held && A.limits && k == 0)  // the held ends keep their limited rym
                for (int t = 0; t < ntc; ++t) {
                    AT4(A.q[2], i, 0, l, t0 + t) = Q(2, t)[0];
                    AT4(A.q[2], i, nc - 1, l, t0 + t) = Q(2, t)[nc - 1];
                }
            __syncthreads();  // the next chunk overwrites the staged tracers
        }
        if (moves) AT(A.m, i, k, l) = m_s[k];
        for (int e = threadIdx.x; e < nlines * nf; e += blockDim.x) {
            const int q = e / nf, kk = kf0 + e % nf;
            BF(A, i0 + q, kk, l) = smem[q * per + NC + kk] * (double)nloop;
        }
    }
}

// tracers a warp stages at once: as many as fit in the block's shared memory (all when they do)
int tracer_chunk(int warps, int ncell, int fixed, int per_tracer, int nt) {
    const size_t cap = 227 * 1024;
    int tc = nt;
    while (tc > 1 && (size_t)warps * ncell * (fixed + per_tracer * tc) * sizeof(double) > cap) --tc;
    return tc;
}

int launch_y(gb_ctx *ctx, YArgs &A, int32_t *scratch = nullptr) {
    A.ncell = A.nc + 2;
    const int64_t cols = (int64_t)A.ni * A.nl;
    const int blocks = (int)((cols + STEP_WARPS - 1) / STEP_WARPS);
    // the column-parallel search needs the per-layer candidates and a count per column: in the
    // context's scratch when it holds them; the fixed scratch of gb_advect_y_noalloc (and a
    // scratch too small) take the CTA-per-layer search, which needs the layer counts only
    const size_t need = (size_t)A.nl * (1 + (YROUNDS + 1) + YROUNDS) + (size_t)cols;
    int32_t *wide = scratch ? nullptr : gb_scratch_i(ctx, need);
    A.nloop = scratch ? scratch : (wide ? wide : gb_scratch_i(ctx, A.nl));
    if (!A.nloop) {
        gb_set_error("gb_advect_y: too many levels for the scratch");
        return GB_EARG;
    }
    if (wide) {
        YSearch S;
        S.cand = wide + A.nl;
        S.changed = S.cand + (YROUNDS + 1) * A.nl;
        S.coln = S.changed + YROUNDS * A.nl;
        GB_CHECK_CUDA(cudaMemsetAsync(S.cand, 0, (size_t)(2 * YROUNDS + 1) * A.nl * sizeof(int32_t), ctx->stream));
        const size_t smem_c = (size_t)STEP_WARPS * 2 * A.ncell * sizeof(double);
        GB_CHECK_CUDA(cudaFuncSetAttribute(k_y_search_cols, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_c));
        // with a cap of one (Check_CFL's rehearsal) round 0 decides: a column passes at n = 1 or
        // records 2, so round 1 finds every column at the candidate or the candidate over the cap
        // and round 2 finds nothing changed -- both would return at once
        const int rounds = A.nmax <= 1 ? 1 : YROUNDS;
        for (int r = 0; r < rounds; ++r) {
            k_y_search_cols<<<blocks, STEP_WARPS * 32, smem_c, ctx->stream>>>(A, S, r);
            if (int rc = gb_after_launch(ctx, "y_search_cols")) return rc;
        }
        k_y_search_done<<<A.nl, SEARCH_THREADS, 0, ctx->stream>>>(A, S);
        if (int rc = gb_after_launch(ctx, "y_search_done")) return rc;
    } else {
        size_t smem_s = (size_t)(SEARCH_THREADS / 32) * 2 * A.ncell * sizeof(double);
        GB_CHECK_CUDA(cudaFuncSetAttribute(k_y_search, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_s));
        k_y_search<<<A.nl, SEARCH_THREADS, smem_s, ctx->stream>>>(A);
        if (int rc = gb_after_launch(ctx, "y_search")) return rc;
    }
    if (A.nc > YMAX_THREADS) {
        gb_set_error("gb_advect_y: at most 576 cells a column");
        return GB_EARG;
    }
    A.P = y_lines_per_block(A.nc);
    A.tc = A.mass_only ? 0 : tracer_chunk(A.P, A.ncell, 3, 8, A.nt);
    const size_t smem = (size_t)A.P * A.ncell * (3 + 8 * A.tc) * sizeof(double);
    if (smem > 227 * 1024) {
        gb_set_error("gb_advect_y: the columns of a block do not fit in shared memory");
        return GB_EARG;
    }
    const int sthreads = (A.P * A.nc + 31) / 32 * 32;
    const int sblocks = A.nl * ((A.ni + A.P - 1) / A.P);
    if (A.mass_only) {
        GB_CHECK_CUDA(cudaFuncSetAttribute(k_y_steps<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_y_steps<true><<<sblocks, sthreads, smem, ctx->stream>>>(A);
    } else {
        GB_CHECK_CUDA(cudaFuncSetAttribute(k_y_steps<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_y_steps<false><<<sblocks, sthreads, smem, ctx->stream>>>(A);
    }
    return gb_after_launch(ctx, A.mass_only ? "cfl_y" : "y_steps");
}

int setup(YArgs &A, const gb_view *m, const gb_view *bm, const gb_view *full, int full_l0, const int32_t *own,
          int held) {
    A.m = dv(m);
    A.bm = dv(bm);
    A.full = full ? dv(full) : DV{};
    A.full_l0 = full_l0;
    A.ni = (int)m->n[0]; A.nc = (int)m->n[1]; A.nl = (int)m->n[2];
    A.held = held;
    if (!held && bm->n[1] != A.nc + 1) {
        gb_set_error("gb_advect_y: bm must have jm+1 faces");
        return GB_EARG;
    }
    if (held && (bm->n[1] != A.nc - 1 || A.nc < 3)) {
        gb_set_error("gb_advect_y_held: a held column of n >= 3 cells has n-1 faces");
        return GB_EARG;
    }
    if (full) {
        if (!own) {
            gb_set_error("gb_advect_y: the owned face box of the full layer is needed");
            return GB_EARG;
        }
        A.own_i0 = own[0]; A.own_i1 = own[1]; A.own_j0 = own[2]; A.own_j1 = own[3];
    }
    return GB_OK;
}

}  // namespace

extern "C" int gb_advect_y(gb_ctx *ctx, const gb_view *m, const gb_view *rm, const gb_view *rxm,
                           const gb_view *rym, const gb_view *rzm, const gb_view *bm,
                           const gb_view *bm_full, int bm_full_l0, int limits, int max_nloop,
                           int32_t *nloop_out) {
    if (!ctx || !m || !rm || !rxm || !rym || !rzm || !bm) return GB_EARG;
    YArgs A{};
    // region 1: the columns own bm(1:im, 1:jm+1) of the halo'd (0:im+1, 0:jm+1) layer
    const int32_t own[4] = {1, (int32_t)m->n[0], 1, (int32_t)m->n[1] + 1};
    if (int rc = setup(A, m, bm, bm_full, bm_full_l0, own, 0)) return rc;
    A.q[0] = dv(rm); A.q[1] = dv(rxm); A.q[2] = dv(rym); A.q[3] = dv(rzm);
    A.nt = (int)rm->n[3];
    A.limits = limits; A.nmax = max_nloop - 1;
    A.nloop_out = nloop_out;
    A.ctl = ctx->ctl;
    return launch_y(ctx, A);
}

// ------------------------------------------------------------------ gb_advect_y_noalloc
// The per-layer sub-cycle counts live in this array, compiled into the library, instead of in
// the context's scratch.  Nothing in it has to start at zero: the search kernel writes the count
// of every layer of a call (on every exit) before the steps kernel of that call reads it.
namespace {
__device__ __align__(256) int32_t g_y_nloop_static[GB_NOALLOC_MAX_LEVELS];

constexpr int MAX_DEVICES = 64;
std::atomic<int32_t *> g_y_nloop_addr[MAX_DEVICES];

// the array's device address on the current device, looked up on the first call there
int y_static_scratch(gb_ctx *ctx, int32_t **out) {
    int cur = -1;
    GB_CHECK_CUDA(cudaGetDevice(&cur));
    if (cur != ctx->device || cur < 0 || cur >= MAX_DEVICES) {
        gb_set_error("gb_advect_y_noalloc: the current device is not the context's (or above 63)");
        return GB_EARG;
    }
    int32_t *p = g_y_nloop_addr[cur].load(std::memory_order_acquire);
    if (!p) {
        void *addr = nullptr;
        GB_CHECK_CUDA(cudaGetSymbolAddress(&addr, g_y_nloop_static));
        p = static_cast<int32_t *>(addr);
        g_y_nloop_addr[cur].store(p, std::memory_order_release);
    }
    *out = p;
    return GB_OK;
}
}  // namespace

extern "C" int gb_advect_y_noalloc(gb_ctx *ctx, const gb_view *m, const gb_view *rm, const gb_view *rxm,
                                   const gb_view *rym, const gb_view *rzm, const gb_view *bm,
                                   const gb_view *bm_full, int bm_full_l0, int limits, int max_nloop,
                                   int32_t *nloop_out) {
    if (!ctx || !m || !rm || !rxm || !rym || !rzm || !bm) return GB_EARG;
    if (m->n[2] < 1 || m->n[2] > GB_NOALLOC_MAX_LEVELS) {
        gb_set_error("gb_advect_y_noalloc: " + std::to_string(m->n[2]) + " levels; this entry point takes 1 to " +
                     std::to_string(GB_NOALLOC_MAX_LEVELS));
        return GB_EARG;
    }
    int32_t *scratch = nullptr;
    if (int rc = y_static_scratch(ctx, &scratch)) return rc;
    YArgs A{};
    const int32_t own[4] = {1, (int32_t)m->n[0], 1, (int32_t)m->n[1] + 1};
    if (int rc = setup(A, m, bm, bm_full, bm_full_l0, own, 0)) return rc;
    A.q[0] = dv(rm); A.q[1] = dv(rxm); A.q[2] = dv(rym); A.q[3] = dv(rzm);
    A.nt = (int)rm->n[3];
    A.limits = limits; A.nmax = max_nloop - 1;
    A.nloop_out = nloop_out;
    A.ctl = ctx->ctl;
    return launch_y(ctx, A, scratch);
}

extern "C" int gb_advect_y_held(gb_ctx *ctx, const gb_view *m, const gb_view *rm, const gb_view *rxm,
                                const gb_view *rym, const gb_view *rzm, const gb_view *bm,
                                const gb_view *bm_full, int bm_full_l0, const int32_t *own, int limits,
                                int max_nloop) {
    if (!ctx || !m || !rm || !rxm || !rym || !rzm || !bm) return GB_EARG;
    YArgs A{};
    if (int rc = setup(A, m, bm, bm_full, bm_full_l0, own, 1)) return rc;
    A.q[0] = dv(rm); A.q[1] = dv(rxm); A.q[2] = dv(rym); A.q[3] = dv(rzm);
    A.nt = (int)rm->n[3];
    A.limits = limits; A.nmax = max_nloop - 1;
    A.ctl = ctx->ctl;
    return launch_y(ctx, A);
}

extern "C" int gb_cfl_y(gb_ctx *ctx, const gb_view *m, const gb_view *bm, int max_nloop) {
    if (!ctx || !m || !bm) return GB_EARG;
    YArgs A{};
    if (int rc = setup(A, m, bm, nullptr, 0, nullptr, 0)) return rc;
    for (int w = 0; w < 4; ++w) A.q[w] = A.m;
    A.nt = 0;
    A.nmax = max_nloop;  // dynamvm gives up once nloop would exceed max_nloop (cfl.py:175)
    A.ctl = ctx->ctl;
    A.mass_only = 1;
    return launch_y(ctx, A);
}

extern "C" int gb_cfl_y_held(gb_ctx *ctx, const gb_view *m, const gb_view *bm, const gb_view *bm_full,
                             int bm_full_l0, const int32_t *own, int max_nloop) {
    if (!ctx || !m || !bm) return GB_EARG;
    YArgs A{};
    if (int rc = setup(A, m, bm, bm_full, bm_full_l0, own, 1)) return rc;
    for (int w = 0; w < 4; ++w) A.q[w] = A.m;
    A.nt = 0;
    A.nmax = max_nloop;  // the child's dynamvm: nloop > max_nloop fails (check_cfl.py:185)
    A.full_mode = 1;     // the whole layer is only restored, times nloop (check_cfl.py:189-190)
    A.ctl = ctx->ctl;
    A.mass_only = 1;
    return launch_y(ctx, A);
}
