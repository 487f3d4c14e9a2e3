// dynamu: zonal slopes advection of every (j, l) row of a region, one warp per row.
//
// A row is staged in shared memory (lanes across its cells), clustered onto the reduced grid
// when its latitude is reduced, searched for its smallest CFL-safe sub-cycle count (warp
// vote), advanced through all its sub-steps on chip, split back onto the uniform cells and
// written once.  Two row kinds:
//   periodic  region 1: n cells, n+1 faces, face 0 the seam copy of face n
//   held      a child: n cells of which the two ends are held (the parent's, put there by
//             put_xedges), n-1 interior faces; shared memory keeps the periodic indexing (face
//             k between cells k-1 and k, k = 1 .. n-1)
// Reference: pydyn kernels.py:129-220 (_advect_rows_x, subcycle_rows, _substeps_x),
// redgrid.py:56-110 (uni2red, uni2red_mf, red2uni), zoom/advect.py:237-345 (_dynamu_region1's
// halos, _dynamu_child, _rows_child, _substeps_child), cfl.py:140-167 (dynamum) and
// zoom/check_cfl.py:113-137 (_dynamum_child).
#include "gb_adjoint.cuh"
#include "gb_common.cuh"

namespace {

constexpr int WARPS = 4;

struct XArgs {
    DV m, q[4], am;
    const int32_t *clust;
    int n0, nj, nl, nt;  // view extents: cells per row, rows (j), levels
    int halo, js, je;    // halo writes on rows js..je (1-based, inclusive)
    int limits, nmax;    // nmax = max_nloop - 1
    int restore_am;      // 1: am = a * nloop written back; 0: am untouched (reduced grid)
    int held;            // child rows
    int ncell;           // smem cells per array (n0 + 2)
    int tc;              // tracers staged at once (launch_x)
    int32_t *nloop_out;
    double *amax_out;
    gb_ctl *ctl;
};

__device__ __forceinline__ double &AT(const DV &v, int64_t i, int64_t j, int64_t l) {
    return v.p[i * v.s0 + j * v.s1 + l * v.s2];
}
__device__ __forceinline__ double &AT4(const DV &v, int64_t i, int64_t j, int64_t l, int64_t t) {
    return v.p[i * v.s0 + j * v.s1 + l * v.s2 + t * v.s3];
}

// The per-row CFL search (kernels.py:169-199): the smallest nloop for which nloop trial
// sub-steps of the mass stay under |Courant| < 1 on every face (division form,
// ops.py:267-270), the faces rescaled by (n-1)/n per retry.  Faces k0..k1, cells i0..i1 move.
// Returns nloop, or nmax + 1.  want_amax: also the largest |Courant| of the passing trial (the
// division on every face); without it the test is cfl_pass's.
__device__ int row_search(double *m_s, double *mx_s, double *a_s, int n, bool held, int nmax, int lane,
                          double &amax_out, bool want_amax) {
    const int k0 = held ? 1 : 0, k1 = held ? n - 1 : n;
    const int i0 = held ? 1 : 0, i1 = held ? n - 1 : n;  // cells [i0, i1)
    int nloop = 1;
    while (true) {
        for (int k = lane; k < n; k += GB_WARP) mx_s[k] = m_s[k];
        __syncwarp();
        bool ok = true;
        double amax = 0.0;
        for (int s = 0; s < nloop; ++s) {
            bool lok = true;
            double cmax = 0.0;
            for (int k = k0 + lane; k <= k1; k += GB_WARP) {
                double f = a_s[k];
                int up = ge_zero(f) ? (k == 0 ? n - 1 : k - 1) : (k == n ? 0 : k);
                if (want_amax) {
                    double c = gb_abs(div_ip(f, mx_s[up]));
                    lok = lok && (c < 1.0);
                    cmax = (c > cmax) ? c : cmax;
                } else {
                    lok = lok && cfl_pass(f, mx_s[up]);
                }
            }
            ok = __all_sync(FULL_MASK, lok);
            if (!ok) break;
            if (want_amax) {
                for (int o = 16; o > 0; o >>= 1) {
                    double other = __shfl_xor_sync(FULL_MASK, cmax, o);
                    cmax = (other > cmax) ? other : cmax;
                }
                amax = (amax > cmax) ? amax : cmax;
            }
            __syncwarp();
            for (int k = i0 + lane; k < i1; k += GB_WARP) mx_s[k] = (mx_s[k] + a_s[k]) - a_s[k + 1];
            __syncwarp();
        }
        if (ok) {
            amax_out = amax;
            return nloop;
        }
        nloop += 1;
        for (int k = k0 + lane; k <= k1; k += GB_WARP) a_s[k] = div_ip(a_s[k] * (double)(nloop - 1), (double)nloop);
        __syncwarp();
        if (nloop > nmax) {
            amax_out = 0.0;
            return nloop;
        }
    }
}

template <bool MASS_ONLY>
__global__ void __launch_bounds__(WARPS * 32) k_advect_x(XArgs A) {
    extern __shared__ double smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t row = (int64_t)blockIdx.x * WARPS + warp;
    if (row >= (int64_t)A.nj * A.nl) return;
    if (MASS_ONLY && __shfl_sync(FULL_MASK, *(volatile int *)&A.ctl->cfl_failed, 0)) return;
    const int j = (int)(row / A.nl), l = (int)(row % A.nl);
    const int nt = MASS_ONLY ? 0 : A.nt;
    const int tc = MASS_ONLY ? 0 : A.tc;  // tracers staged at once (a chunk)
    const int NC = A.ncell;
    const int per_warp = NC * (4 + 8 * tc);
    const bool held = A.held != 0;
    double *m_s = smem + (size_t)warp * per_warp;
    double *mx_s = m_s + NC;
    double *minv_s = mx_s + NC;
    double *a_s = minv_s + NC;
    double *q_s = a_s + NC;          // [4][tc][NC]: rm, rxm, rym, rzm
    double *f_s = q_s + 4 * tc * NC; // [4][tc][NC]: f, pf, fy, fz
    auto Q = [&](int w, int t) { return q_s + (size_t)(w * tc + t) * NC; };
    auto F = [&](int w, int t) { return f_s + (size_t)(w * tc + t) * NC; };

    const int c = (!held && A.clust && A.clust[j] > 1) ? A.clust[j] : 1;
    const int n = A.n0 / c;
    const bool reduced = c > 1;

    // ---- stage the row's mass: cluster sums onto the reduced cells (uni2red, seqsum in order)
    for (int k = lane; k < n; k += GB_WARP) {
        double acc = AT(A.m, (int64_t)k * c, j, l);
        for (int cc = 1; cc < c; ++cc) acc = acc + AT(A.m, (int64_t)k * c + cc, j, l);
        m_s[k] = acc;
    }
    if (held) {  // n-1 interior faces, face k between cells k-1 and k
        for (int k = 1 + lane; k < n; k += GB_WARP) a_s[k] = AT(A.am, k - 1, j, l);
    } else {     // a(i) = am(i c), i = 1..n; a(0) = a(n) on a reduced row (uni2red_mf)
        for (int k = lane; k <= n; k += GB_WARP) {
            int src = (k == 0) ? (reduced ? n * c : 0) : k * c;
            a_s[k] = AT(A.am, src, j, l);
        }
    }
    __syncwarp();

    double amax = 0.0;
    const int nloop = row_search(m_s, mx_s, a_s, n, held, A.nmax, lane, amax, A.amax_out != nullptr);
    if (nloop > A.nmax) {
        if (lane == 0) {
            if (MASS_ONLY)
                atomicExch(&A.ctl->cfl_failed, 1);
            else
                raise_status(A.ctl, GB_ECFL);
            if (A.nloop_out) A.nloop_out[row] = nloop;
        }
        return;
    }

    const int i0 = held ? 1 : 0, i1 = held ? n - 1 : n;  // the cells that move
    const bool in_scope = (j + 1 >= A.js) && (j + 1 <= A.je);
    const int im = A.n0;
    if (MASS_ONLY) {
        for (int s = 0; s < nloop; ++s) {
            for (int k = i0 + lane; k < i1; k += GB_WARP) m_s[k] = (m_s[k] + a_s[k]) - a_s[k + 1];
            __syncwarp();
        }
    } else {
        // the tracers, tc at a time: every chunk restarts from the staged mass (kept in mx_s) and
        // repeats the same mass updates; tracers never mix, so each sees exactly what it would
        // with all of them staged together
        for (int k = lane; k < n; k += GB_WARP) mx_s[k] = m_s[k];
        __syncwarp();
        for (int t0 = 0; t0 < nt; t0 += tc) {
            const int ntc = min(tc, nt - t0);
            for (int k = lane; k < n; k += GB_WARP) {
                m_s[k] = mx_s[k];
                minv_s[k] = div_ip(1.0, mx_s[k]);
                for (int w = 0; w < 4; ++w)
                    for (int t = 0; t < ntc; ++t) {
                        double v = AT4(A.q[w], (int64_t)k * c, j, l, t0 + t);
                        for (int cc = 1; cc < c; ++cc) v = v + AT4(A.q[w], (int64_t)k * c + cc, j, l, t0 + t);
                        Q(w, t)[k] = v;
                    }
                if (A.limits)  // every cell of the row, a child's held ends included
                    for (int t = 0; t < ntc; ++t) Q(1, t)[k] = np_limit(Q(1, t)[k], Q(0, t)[k]);
            }
            __syncwarp();
            const int k0 = 1, k1 = held ? n - 1 : n;  // periodic: face 0 is the seam copy of face n
            for (int s = 0; s < nloop; ++s) {
                for (int k = k0 + lane; k <= k1; k += GB_WARP) {
                    double f = a_s[k];
                    int up = ge_zero(f) ? k - 1 : (k == n ? 0 : k);
                    double alpha = f * minv_s[up];  // the reciprocal form of production dynamu
                    for (int t = 0; t < ntc; ++t) {
                        double ff, pf, fy, fz;
                        slopes_flux(f, alpha, Q(0, t)[up], Q(1, t)[up], Q(2, t)[up], Q(3, t)[up], ff, pf, fy, fz);
                        F(0, t)[k] = ff; F(1, t)[k] = pf; F(2, t)[k] = fy; F(3, t)[k] = fz;
                    }
                }
                __syncwarp();
                for (int i = i0 + lane; i < i1; i += GB_WARP) {
                    const int lo = (i == 0) ? n : i;
                    const double mo = m_s[i], alo = a_s[i], ahi = a_s[i + 1];
                    const double mn = (mo + alo) - ahi;
                    // 1 / mn, the next sub-step's Courant factor, also gives the slope's quotient
                    const double inv = div_ip(1.0, mn), y = recip_mark(mn, inv);
                    for (int t = 0; t < ntc; ++t) {
                        double *f = F(0, t), *pf = F(1, t), *fy = F(2, t), *fz = F(3, t);
                        double rmn = Q(0, t)[i] - (f[i + 1] - f[lo]);
                        double rxn = along_slope_y(Q(1, t)[i], pf[lo], pf[i + 1], alo, ahi, rmn, f[lo], f[i + 1], mo,
                                                   mn, y);
                        if (A.limits) rxn = np_limit(rxn, rmn);
                        Q(0, t)[i] = rmn;
                        Q(1, t)[i] = rxn;
                        Q(2, t)[i] = Q(2, t)[i] - (fy[i + 1] - fy[lo]);
                        Q(3, t)[i] = Q(3, t)[i] - (fz[i + 1] - fz[lo]);
                    }
                    m_s[i] = mn;
                    minv_s[i] = inv;
                }
                __syncwarp();
            }
            // ---- the chunk's tracers out
            if (!reduced) {
                for (int i = i0 + lane; i < i1; i += GB_WARP)
                    for (int w = 0; w < 4; ++w)
                        for (int t = 0; t < ntc; ++t) AT4(A.q[w], i, j, l, t0 + t) = Q(w, t)[i];
                if (held && A.limits && lane == 0)  // the held ends keep their limited rxm
                    for (int t = 0; t < ntc; ++t) {
                        AT4(A.q[1], 0, j, l, t0 + t) = Q(1, t)[0];
                        AT4(A.q[1], n - 1, j, l, t0 + t) = Q(1, t)[n - 1];
                    }
                if (A.halo && in_scope && lane == 0)  // q(0) = q(im), q(im+1) = q(1)
                    for (int w = 0; w < 4; ++w)
                        for (int t = 0; t < ntc; ++t) {
                            AT4(A.q[w], -1, j, l, t0 + t) = Q(w, t)[n - 1];
                            AT4(A.q[w], n, j, l, t0 + t) = Q(w, t)[0];
                        }
            } else {
                // red2uni: every cell of a cluster given its share m_uni(i) / m(cluster) of the
                // cluster's tracers, m_uni the uniform mass updated with the untouched am
                for (int i = lane; i < im; i += GB_WARP) {
                    const int k = i / c;
                    const double mun = (AT(A.m, i, j, l) + AT(A.am, i, j, l)) - AT(A.am, i + 1, j, l);
                    const double sc = div_ip(mun, m_s[k]);
                    for (int w = 0; w < 4; ++w)
                        for (int t = 0; t < ntc; ++t) AT4(A.q[w], i, j, l, t0 + t) = sc * Q(w, t)[k];
                    if (A.halo && i == im - 1)  // q(0) = q(im) after red2uni
                        for (int w = 0; w < 4; ++w)
                            for (int t = 0; t < ntc; ++t) AT4(A.q[w], -1, j, l, t0 + t) = sc * Q(w, t)[k];
                }
            }
            __syncwarp();  // the next chunk overwrites the staged tracers
        }
    }

    if (A.nloop_out && lane == 0) A.nloop_out[row] = nloop;
    if (A.amax_out && lane == 0) A.amax_out[row] = amax;

    if (A.restore_am) {  // "restore old am": a * nloop, not an exact round trip
        if (held)
            for (int k = 1 + lane; k < n; k += GB_WARP) AT(A.am, k - 1, j, l) = a_s[k] * (double)nloop;
        else
            for (int k = lane; k <= n; k += GB_WARP) AT(A.am, k, j, l) = a_s[k] * (double)nloop;
    }

    // ---- the mass out, after every chunk (red2uni's shares read the uniform mass)
    if (!reduced) {
        for (int i = i0 + lane; i < i1; i += GB_WARP) AT(A.m, i, j, l) = m_s[i];
        if (A.halo && in_scope && lane == 0) {
            AT(A.m, -1, j, l) = m_s[n - 1];
            AT(A.m, n, j, l) = m_s[0];
        }
    } else {
        for (int i = lane; i < im; i += GB_WARP) {
            const double mun = (AT(A.m, i, j, l) + AT(A.am, i, j, l)) - AT(A.am, i + 1, j, l);
            AT(A.m, i, j, l) = mun;
            if (A.halo && i == im - 1 && (MASS_ONLY ? in_scope : true)) AT(A.m, -1, j, l) = mun;
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

int launch_x(gb_ctx *ctx, XArgs &A, bool mass_only) {
    A.ncell = A.n0 + 2;
    A.tc = mass_only ? 0 : tracer_chunk(WARPS, A.ncell, 4, 8, A.nt);
    size_t smem = (size_t)WARPS * A.ncell * (4 + 8 * A.tc) * sizeof(double);
    int64_t rows = (int64_t)A.nj * A.nl;
    int blocks = (int)((rows + WARPS - 1) / WARPS);
    if (blocks == 0) return GB_OK;
    if (mass_only) {
        GB_CHECK_CUDA(cudaFuncSetAttribute(k_advect_x<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_advect_x<true><<<blocks, WARPS * 32, smem, ctx->stream>>>(A);
    } else {
        GB_CHECK_CUDA(cudaFuncSetAttribute(k_advect_x<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_advect_x<false><<<blocks, WARPS * 32, smem, ctx->stream>>>(A);
    }
    return gb_after_launch(ctx, mass_only ? "cfl_x" : "advect_x");
}

// The adjoint of dynamu on region 1's rows (unlimited slopes): one warp per (j, l) row.  The
// row is staged and searched exactly as k_advect_x does it (the same sub-cycle count and rescaled
// faces), then the transposes run in reverse: red2uni's (a reduced row's cells gather their
// cluster's adjoints with the shares m_uni'(i) / m(cluster)), the sub-steps', uni2red's (every
// cell of a cluster receives the cluster's adjoint).  A.m / A.am: the mass and faces before the
// forward operator; A.q: the tracer adjoints, overwritten with the adjoints before it.
__global__ void __launch_bounds__(WARPS * 32) k_adj_x(XArgs A) {
    extern __shared__ double smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t row = (int64_t)blockIdx.x * WARPS + warp;
    if (row >= (int64_t)A.nj * A.nl) return;
    const int j = (int)(row / A.nl), l = (int)(row % A.nl);
    const int NC = A.ncell;
    double *base = smem + (size_t)warp * adj_doubles_per_line(NC);
    const AdjLine L = adj_line(base, NC);
    double *mx = base + 14 * NC;
    const int c = (A.clust && A.clust[j] > 1) ? A.clust[j] : 1;
    const int n = A.n0 / c;
    const bool reduced = c > 1;

    for (int k = lane; k < n; k += GB_WARP) {
        double acc = AT(A.m, (int64_t)k * c, j, l);
        for (int cc = 1; cc < c; ++cc) acc = acc + AT(A.m, (int64_t)k * c + cc, j, l);
        L.m0[k] = acc;
    }
    for (int k = lane; k <= n; k += GB_WARP) L.a[k] = AT(A.am, k == 0 ? (reduced ? n * c : 0) : k * c, j, l);
    __syncwarp();
    double amax = 0.0;
    const int nloop = row_search(L.m0, mx, L.a, n, false, A.nmax, lane, amax, false);
    if (nloop > A.nmax) {
        if (lane == 0) raise_status(A.ctl, GB_ECFL);
        return;
    }
    if (reduced) {  // red2uni's transpose: the reduced mass after the sub-steps first
        for (int k = lane; k < n; k += GB_WARP) L.mw[k] = L.m0[k];
        __syncwarp();
        for (int s = 0; s < nloop; ++s) {
            for (int k = lane; k < n; k += GB_WARP) L.mw[k] = (L.mw[k] + L.a[k]) - L.a[k + 1];
            __syncwarp();
        }
        for (int k = lane; k < n; k += GB_WARP)
            for (int w = 0; w < 4; ++w) {
                double acc = 0.0;
                for (int p = 0; p < c; ++p) {
                    const int64_t i = (int64_t)k * c + p;
                    const double mun = (AT(A.m, i, j, l) + AT(A.am, i, j, l)) - AT(A.am, i + 1, j, l);
                    acc = acc + div_ip(mun, L.mw[k]) * AT4(A.q[w], i, j, l, 0);
                }
                L.q[w][k] = acc;
            }
    } else {
        for (int k = lane; k < n; k += GB_WARP)
            for (int w = 0; w < 4; ++w) L.q[w][k] = AT4(A.q[w], k, j, l, 0);
    }
    __syncwarp();
    adj_line_substeps(L, n, nloop, LINE_PERIODIC, true, lane);
    for (int i = lane; i < A.n0; i += GB_WARP)  // uni2red's transpose
        for (int w = 0; w < 4; ++w) AT4(A.q[w], i, j, l, 0) = L.q[w][i / c];
}

int setup(XArgs &A, const gb_view *m, const gb_view *am, int held) {
    A.m = dv(m);
    A.am = dv(am);
    A.n0 = (int)m->n[0]; A.nj = (int)m->n[1]; A.nl = (int)m->n[2];
    A.held = held;
    if (!held && am->n[0] != A.n0 + 1) {
        gb_set_error("gb_advect_x: a periodic row has im+1 faces");
        return GB_EARG;
    }
    if (held && (am->n[0] != A.n0 - 1 || A.n0 < 3)) {
        gb_set_error("gb_advect_x_held: a held row of n >= 3 cells has n-1 faces");
        return GB_EARG;
    }
    return GB_OK;
}

}  // namespace

extern "C" int gb_advect_x(gb_ctx *ctx, const gb_view *m, const gb_view *rm, const gb_view *rxm,
                           const gb_view *rym, const gb_view *rzm, const gb_view *am,
                           const int32_t *clust, int halo, int js, int je, int limits, int max_nloop,
                           int32_t *nloop_out, double *amax_out) {
    if (!ctx || !m || !rm || !rxm || !rym || !rzm || !am) return GB_EARG;
    XArgs A{};
    if (int rc = setup(A, m, am, 0)) return rc;
    A.q[0] = dv(rm); A.q[1] = dv(rxm); A.q[2] = dv(rym); A.q[3] = dv(rzm);
    A.clust = clust;
    A.nt = (int)rm->n[3];
    A.halo = halo; A.js = js; A.je = je;
    A.limits = limits; A.nmax = max_nloop - 1;
    A.restore_am = clust ? 0 : 1;
    A.nloop_out = nloop_out; A.amax_out = amax_out;
    A.ctl = ctx->ctl;
    return launch_x(ctx, A, false);
}

extern "C" int gb_advect_x_held(gb_ctx *ctx, const gb_view *m, const gb_view *rm, const gb_view *rxm,
                                const gb_view *rym, const gb_view *rzm, const gb_view *am, int limits,
                                int max_nloop) {
    if (!ctx || !m || !rm || !rxm || !rym || !rzm || !am) return GB_EARG;
    XArgs A{};
    if (int rc = setup(A, m, am, 1)) return rc;
    A.q[0] = dv(rm); A.q[1] = dv(rxm); A.q[2] = dv(rym); A.q[3] = dv(rzm);
    A.nt = (int)rm->n[3];
    A.limits = limits; A.nmax = max_nloop - 1;
    A.restore_am = 1;
    A.js = 1; A.je = 0;
    A.ctl = ctx->ctl;
    return launch_x(ctx, A, false);
}

extern "C" int gb_cfl_x(gb_ctx *ctx, const gb_view *m, const gb_view *am, const int32_t *clust, int halo,
                        int js, int je, int max_nloop) {
    if (!ctx || !m || !am) return GB_EARG;
    XArgs A{};
    if (int rc = setup(A, m, am, 0)) return rc;
    for (int w = 0; w < 4; ++w) A.q[w] = A.m;
    A.clust = clust;
    A.nt = 0;
    A.halo = halo; A.js = js; A.je = je;
    A.limits = 0; A.nmax = max_nloop - 1;
    A.restore_am = clust ? 0 : 1;
    A.ctl = ctx->ctl;
    return launch_x(ctx, A, true);
}

extern "C" int gb_cfl_x_held(gb_ctx *ctx, const gb_view *m, const gb_view *am, int max_nloop) {
    if (!ctx || !m || !am) return GB_EARG;
    XArgs A{};
    if (int rc = setup(A, m, am, 1)) return rc;
    for (int w = 0; w < 4; ++w) A.q[w] = A.m;
    A.nt = 0;
    A.limits = 0; A.nmax = max_nloop - 1;
    A.restore_am = 1;
    A.js = 1; A.je = 0;
    A.ctl = ctx->ctl;
    return launch_x(ctx, A, true);
}

extern "C" int gb_adjoint_x(gb_ctx *ctx, const gb_view *m, const gb_view *rm_b, const gb_view *rxm_b,
                            const gb_view *rym_b, const gb_view *rzm_b, const gb_view *am, const int32_t *clust,
                            int max_nloop) {
    if (!ctx || !m || !rm_b || !rxm_b || !rym_b || !rzm_b || !am) return GB_EARG;
    XArgs A{};
    if (int rc = setup(A, m, am, 0)) return rc;
    A.q[0] = dv(rm_b); A.q[1] = dv(rxm_b); A.q[2] = dv(rym_b); A.q[3] = dv(rzm_b);
    if (rm_b->n[3] != 1) {
        gb_set_error("gb_adjoint_x: one tracer");
        return GB_EARG;
    }
    A.clust = clust;
    A.nt = 1;
    A.nmax = max_nloop - 1;
    A.ctl = ctx->ctl;
    A.ncell = A.n0 + 2;
    const size_t smem = (size_t)WARPS * 15 * A.ncell * sizeof(double);
    const int64_t rows = (int64_t)A.nj * A.nl;
    if (rows == 0) return GB_OK;
    GB_CHECK_CUDA(cudaFuncSetAttribute(k_adj_x, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_adj_x<<<(unsigned)((rows + WARPS - 1) / WARPS), WARPS * 32, smem, ctx->stream>>>(A);
    return gb_after_launch(ctx, "adjoint_x");
}
