// The transpose of the slopes scheme's sub-steps on one line of cells (unlimited slopes), for
// the adjoint of dynamu / dynamv / dynamw.
//
// With the limiter off, one sub-step is linear in the tracer moments (rm, the slope along the
// line, two cross slopes) for a given air mass and face fluxes: the Courant numbers and the mass
// update depend on the mass only.  The forward statements (pydyn kernels.py:75-92, 202-220,
// 246-291, 324-346), for face k between cells L = k-1 and R = k with flux a_k, Courant number
// c_k and upwind cell u:
//   f  = c (r_u + (1 - c) s_u)  (a >= 0)   or   c (r_u - (1 + c) s_u)  (a < 0)
//   pf = a (c^2 s_u - 3 f),   fA = c tA_u,   fB = c tB_u
//   r_i'  = r_i - (f_hi - f_lo),  tA_i' = tA_i - (fA_hi - fA_lo),  tB_i' likewise
//   s_i'  = s_i + ((pf_lo - pf_hi) - (a_lo - a_hi) s_i + 3 (a_lo + a_hi) r_i' - 3 m_i (f_lo + f_hi)) / m_i'
// and, on a polar line (region 1's dynamv), flow out of a pole cell carries no slope
// (f = c r_u, pf = -3 a f, fA = 0, fB = c tB_u) and the pole cells keep s and tA.
// The transpose, for output adjoints (R, S, TA, TB) of a cell:
//   q_i = S_i / m_i',  rt_i = R_i + 3 (a_lo + a_hi) q_i          (rt: the adjoint of r_i')
//   face k: F = (rt_R - rt_L) - 3 m_R q_R - 3 m_L q_L,  P = q_R - q_L,  A = TA_R - TA_L, ...
//           F += -3 a P;  to the upwind cell: r += c F,  s += a c^2 P + c (1 -+ c) F,
//           tA += c A,  tB += c B
//   cell:   r = rt_i + ...,  s = S_i (1 - (a_lo - a_hi) / m_i') + ...,  tA = TA_i + ...
// Sub-steps run backwards; the mass before sub-step s is recomputed from the line's mass
// before the operator by s forward mass updates, exactly as the forward made it.
#pragma once

#include "gb_common.cuh"

enum { LINE_PERIODIC = 0, LINE_CLOSED = 1, LINE_POLAR = 2 };

// One warp's shared memory for a line of n cells (faces 0..n): NC = n + 2 doubles per array.
struct AdjLine {
    double *m0;     // mass before the operator (read only)
    double *mw;     // mass before the current sub-step
    double *a;      // faces: a[0..n] (periodic: a[0] is the seam copy of a[n]; closed: a[0] = a[n] = 0)
    double *q[4];   // adjoints: rm, along slope, cross slope A, cross slope B
    double *qs, *rt, *g;  // per cell: S / m', rt, 3 m q
    double *d[4];   // per face: what goes to its upwind cell
};

__device__ __forceinline__ int adj_doubles_per_line(int NC) { return 15 * NC; }

__device__ __forceinline__ AdjLine adj_line(double *base, int NC) {
    AdjLine L;
    L.m0 = base; L.mw = base + NC; L.a = base + 2 * NC;
    for (int w = 0; w < 4; ++w) L.q[w] = base + (3 + w) * NC;
    L.qs = base + 7 * NC; L.rt = base + 8 * NC; L.g = base + 9 * NC;
    for (int w = 0; w < 4; ++w) L.d[w] = base + (10 + w) * NC;
    return L;  // 14 NC used; one spare for the caller
}

// the upwind cell of face k and its Courant number (recip: a * (1 / m), production dynamu's
// form; else a / m)
__device__ __forceinline__ int adj_upwind(int kind, int n, int k, double ak) {
    return ak >= 0.0 ? k - 1 : ((kind == LINE_PERIODIC && k == n) ? 0 : k);
}

// The transpose of `nloop` sub-steps on the line, in place on L.q.  All 32 lanes call it.
static __device__ void adj_line_substeps(const AdjLine &L, int n, int nloop, int kind, bool recip, int lane) {
    const int k0 = 1, k1 = (kind == LINE_PERIODIC) ? n : n - 1;  // the faces that carry flux
    for (int s = nloop - 1; s >= 0; --s) {
        // the mass before sub-step s
        for (int i = lane; i < n; i += GB_WARP) L.mw[i] = L.m0[i];
        __syncwarp();
        for (int r = 0; r < s; ++r) {
            for (int i = lane; i < n; i += GB_WARP) L.mw[i] = (L.mw[i] + L.a[i]) - L.a[i + 1];
            __syncwarp();
        }
        // cells: q, rt, 3 m q
        for (int i = lane; i < n; i += GB_WARP) {
            const double mo = L.mw[i], mn = (mo + L.a[i]) - L.a[i + 1];
            const bool pole = kind == LINE_POLAR && (i == 0 || i == n - 1);
            const double qq = pole ? 0.0 : L.q[1][i] / mn;
            L.qs[i] = qq;
            L.rt[i] = L.q[0][i] + (3.0 * (L.a[i] + L.a[i + 1])) * qq;
            L.g[i] = (3.0 * mo) * qq;
        }
        __syncwarp();
        // faces: the adjoints of the face's fluxes, handed to the upwind cell
        for (int k = k0 + lane; k <= k1; k += GB_WARP) {
            const int lc = k - 1, rc = (kind == LINE_PERIODIC && k == n) ? 0 : k;
            const double ak = L.a[k];
            const int up = adj_upwind(kind, n, k, ak);
            const double c = recip ? ak * (1.0 / L.mw[up]) : ak / L.mw[up];
            double F = ((L.rt[rc] - L.rt[lc]) - L.g[rc]) - L.g[lc];
            const double P = L.qs[rc] - L.qs[lc];
            const bool pole_r = kind == LINE_POLAR && (rc == 0 || rc == n - 1);
            const bool pole_l = kind == LINE_POLAR && (lc == 0 || lc == n - 1);
            const double A = (pole_r ? 0.0 : L.q[2][rc]) - (pole_l ? 0.0 : L.q[2][lc]);
            const double B = L.q[3][rc] - L.q[3][lc];
            F = F - (3.0 * ak) * P;
            const bool slope_free = kind == LINE_POLAR && ((k == 1 && ak >= 0.0) || (k == n - 1 && ak < 0.0));
            L.d[0][k] = c * F;
            L.d[1][k] = slope_free ? 0.0 : (ak * (c * c)) * P + (ak >= 0.0 ? c * (1.0 - c) : -(c * (1.0 + c))) * F;
            L.d[2][k] = slope_free ? 0.0 : c * A;
            L.d[3][k] = c * B;
        }
        __syncwarp();
        // cells: the direct terms plus the faces this cell is upwind of
        for (int i = lane; i < n; i += GB_WARP) {
            const int lo = (kind == LINE_PERIODIC && i == 0) ? n : i, hi = i + 1;
            const bool pole = kind == LINE_POLAR && (i == 0 || i == n - 1);
            const bool from_hi = hi >= k0 && hi <= k1 && L.a[hi] >= 0.0;
            const bool from_lo = lo >= k0 && lo <= k1 && L.a[lo] < 0.0;
            double v[4];
            v[0] = L.rt[i];
            v[1] = pole ? L.q[1][i] : L.q[1][i] - (L.a[i] - L.a[i + 1]) * L.qs[i];
            v[2] = L.q[2][i];
            v[3] = L.q[3][i];
            for (int w = 0; w < 4; ++w) {
                if (from_hi) v[w] = v[w] + L.d[w][hi];
                if (from_lo) v[w] = v[w] + L.d[w][lo];
            }
            for (int w = 0; w < 4; ++w) L.q[w][i] = v[w];  // this cell's own entries only
        }
        __syncwarp();
    }
}
