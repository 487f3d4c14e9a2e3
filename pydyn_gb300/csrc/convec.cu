// convec: implicit convection with Kzz diffusion folded into one matrix per column, inverted
// by Crout LU without pivoting, applied to the tracer mass and (by its diagonal) the slopes.
//
// Seven launches, shaped so that the FP64 pipe -- GB300's scarcest unit -- issues with its
// lanes full:
//   k_convec_chains  three threads per owned column: whether its kept inverse still holds, the
//                    updraft and the downdraft mass fluxes carried level to level
//   k_convec_ratios  one thread per (column, level): the chains' ratios (a division each), which
//                    the carried fluxes do not wait for
//   k_convec_matrix  one thread per (column, column l of its matrix): the quotients that column
//                    uses (each division once), conv1(., l) = I - dt (f(k-1, l) - f(k, l)), the
//                    downdraft chain of f down from the diagonal and the updraft chain up from
//                    it -- into a work space
//   k_convec_tri     one thread per cloudless column (tridiagonal conv1): the same LU and L^-1
//                    by the recurrence their non-zero elements follow
//   k_convec_lu      a group of 8, 16 or 32 lanes per other column whose inverse is made
//                    (beside k_convec_tri, on the context's side stream), on the leading block
//                    of its matrix that holds every off-band non-zero (the cloud's levels): LU
//                    right-looking (each step's trailing (row, column) elements packed onto the
//                    lanes), then L^-1 by forward substitution in place of L (row k's terms
//                    applied to every later row at once, the (row, column) elements packed onto
//                    the lanes).  U goes to the work space, L^-1 to the inverse's place.
//   k_convec_tail    one thread per column k_convec_lu split: the band recurrence of the rows
//                    above its block (tridiagonal there), continued from the block's last pivot
//   k_convec_apply   one thread per (column, column of the inverse): the band rows of L^-1,
//                    then the back substitution U X = L^-1; then, whole columns per block, one
//                    thread per (column, level): the slopes times the inverse's diagonal and
//                    rm = C rm accumulated in k.
// The reference's operation order is kept element by element -- every element receives its
// terms in the same k order as in the row-by-row form -- and work is skipped only where a
// multiplier is exactly zero (x - w * y with w = +-0 returns x unless x is a zero, and the
// accumulators of the substitutions are never -0).  Above the cloud the matrix is tridiagonal
// (diffusion only), so most of the O(n^3) inverse becomes O(n^2).
//
// The inverse of a column is kept (with the air mass it was made from) and reused by the next
// call in the same convection epoch when that air mass is bitwise unchanged -- the two `v` of
// a step's half steps, between which only sources and chemistry (tracers) run.
//
// Reference: pydyn kernels.py:350-396 (convection_matrix), :399-420 (fastminv), :423-457
// (convec), zoom/physics.py:33-52 (convec_region).
#include "gb_common.cuh"

namespace {

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
    double *abuf;        // ncol * n * n work space: conv1, then U, of the columns made here
    double *chain;       // ncol * 4 (n+1) work space: the updraft and downdraft chains
    int32_t *fresh;      // ncol work space: 1 where this call makes the column's inverse
    int32_t *rend;       // ncol * n work space: per row of U, one past its last non-zero
    double *tband;       // ncol * 2n work space: a tridiagonal column's U diagonal, then L's band
    int32_t *eblk;       // ncol work space: the leading block k_convec_lu factorised (n: all of it)
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
__device__ __forceinline__ double max0(double x) { return gb_isnan(x) ? x : (lt_zero(x) ? 0.0 : x); }  // 0.0 > x: lt_zero
// x == 0.0 (either sign), tested on the integer pipe: the FP64 pipe is kept for arithmetic
__device__ __forceinline__ bool is_zero(double x) { return (__double_as_longlong(x) << 1) == 0; }

// the work space's per-column chains amu, zu, amd, zd (n+1 each, indexed by level k = 0..n)
constexpr int NCHAIN = 4;
__device__ __forceinline__ double *chains(const CArgs &A, int c) { return A.chain + (size_t)c * NCHAIN * (A.n + 1); }

// The chain loops read their inputs CB levels at a time into registers before using them, so
// that a batch's loads are in flight together (one column a thread: few warps hide little latency).
constexpr int CB = 12;

// whether column c's kept inverse still holds: its air mass bitwise the one it was made from
__device__ void chain_cache(const CArgs &A, int c, int i, int j) {
    const int n = A.n;
    if (A.cache_m) {
        double *cm = A.cache_m + (size_t)c * n;
        bool same = A.cache_tag[c] == *A.epoch;
        for (int l0 = 0; l0 < n; l0 += CB) {
            double mb[CB], cb[CB];
#pragma unroll
            for (int u = 0; u < CB; ++u)
                if (l0 + u < n) {
                    mb[u] = AT(A.m, i, j, l0 + u);
                    cb[u] = cm[l0 + u];
                }
#pragma unroll
            for (int u = 0; u < CB; ++u)
                if (l0 + u < n) {
                    same = same && (__double_as_longlong(cb[u]) == __double_as_longlong(mb[u]));
                    cm[l0 + u] = mb[u];  // unchanged bits where the column's mass is the kept one
                }
        }
        if (same) {
            A.fresh[c] = 0;
            return;
        }
        A.cache_tag[c] = *A.epoch;
    }
    A.fresh[c] = 1;
    A.eblk[c] = A.n;
}

// The chains' carried part: the updraft mass flux amu of column c (levels 1..n from the bottom)
// and the downdraft's amd.  Each level's ratio z (a division, which the carried value does not
// wait for) is k_convec_ratios', one thread a level, from the stored amu(k-1) / amd(k): the same
// statements on the same values.
__device__ void chain_up(const CArgs &A, int c, int i, int j) {
    const int n = A.n;
    double *amu = chains(A, c);
    const int top = A.top[i * A.ts0 + j * A.ts1];
    double mu = 0.0;
    amu[0] = 0.0;
    for (int k0 = 1; k0 <= n; k0 += CB) {
        double eb[CB], db[CB];
#pragma unroll
        for (int u = 0; u < CB; ++u)
            if (k0 + u <= n) {
                eb[u] = AT(A.entu, i, j, k0 + u - 1);
                db[u] = AT(A.detu, i, j, k0 + u - 1);
            }
#pragma unroll
        for (int u = 0; u < CB; ++u) {
            const int k = k0 + u;
            if (k > n) break;
            const double eu = eb[u], du = db[u];
            const bool act = top >= k;
            const double a = mu + eu - du;
            mu = (act && gb_gt0(a)) ? a : 0.0;
            amu[k] = mu;
        }
    }
}

// the downdraft's carried part, amd of column c (levels n down to 2)
__device__ void chain_down(const CArgs &A, int c, int i, int j) {
    const int n = A.n;
    double *amd = chains(A, c) + 2 * (n + 1);
    const int lfs = A.lfs[i * A.ts0 + j * A.ts1];
    double md = 0.0;
    amd[n] = 0.0;
    amd[0] = 0.0;
    for (int k0 = n; k0 >= 2; k0 -= CB) {
        double eb[CB], db[CB];
#pragma unroll
        for (int u = 0; u < CB; ++u)
            if (k0 - u >= 2) {
                eb[u] = AT(A.entd, i, j, k0 - u - 1);
                db[u] = AT(A.detd, i, j, k0 - u - 1);
            }
#pragma unroll
        for (int u = 0; u < CB; ++u) {
            const int k = k0 - u;
            if (k < 2) break;
            const double ed = eb[u], dd = db[u];
            const bool act = lfs >= k;
            const double a = md - ed + dd;
            md = (act && lt_zero(a)) ? a : 0.0;
            amd[k - 1] = md;
        }
    }
}

// thread per (column made fresh, level k = 1..n): the chains' ratios.  Updraft at k:
// a = amu(k-1) + entu - detu, z = 1 - detu / (amu(k-1) + entu) clipped at 0 where a > 0, else 0;
// the downdraft at k >= 2 from amd(k) alike; -1 marks an inactive level (above the cloud top, or
// the level of free sinking).
__global__ void __launch_bounds__(GB_TUNE_MAX_CELL) k_convec_ratios(CArgs A) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int n = A.n;
    if (t >= (int64_t)A.ncol * n) return;
    const int c = (int)(t / n), k = (int)(t % n) + 1;
    if (!A.fresh[c]) return;
    const int i = A.cols[2 * c], j = A.cols[2 * c + 1];
    double *amu = chains(A, c), *zu = amu + (n + 1), *amd = zu + (n + 1), *zd = amd + (n + 1);
    {  // a level above the cloud top is inactive whatever its ratio: its division is not made
        const bool act = A.top[i * A.ts0 + j * A.ts1] >= k;
        double z = -1.0;
        if (act) {
            const double mu = amu[k - 1], eu = AT(A.entu, i, j, k - 1), du = AT(A.detu, i, j, k - 1);
            const double a = mu + eu - du;
            z = gb_gt0(a) ? max0(1.0 - div_ip(du, mu + eu)) : 0.0;
        }
        zu[k] = z;
    }
    if (k >= 2) {
        const bool act = A.lfs[i * A.ts0 + j * A.ts1] >= k;
        double z = -1.0;
        if (act) {
            const double md = amd[k], ed = AT(A.entd, i, j, k - 1), dd = AT(A.detd, i, j, k - 1);
            const double a = md - ed + dd;
            z = lt_zero(a) ? max0(1.0 + div_ip(dd, md - ed)) : 0.0;
        }
        zd[k] = z;
    } else {
        zd[0] = zd[1] = -1.0;
    }
}

// three threads per column, one part each (threadIdx.y, a warp's threads all take the same):
// 0 whether the kept inverse still holds, 1 the updraft chains, 2 the downdraft chains.  The
// chains are made whether or not the inverse is kept (k_convec_matrix reads them only for the
// columns made fresh), so the three parts run side by side.
__global__ void __launch_bounds__(3 * GB_TUNE_MAX_COLUMN) k_convec_chains(CArgs A) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= A.ncol) return;
    const int i = A.cols[2 * c], j = A.cols[2 * c + 1];
    if (threadIdx.y == 0)
        chain_cache(A, c, i, j);
    else if (threadIdx.y == 1)
        chain_up(A, c, i, j);
    else
        chain_down(A, c, i, j);
}

// thread per (column, column l of its matrix): conv1(., l).  f(k, l), k = 0..n: the downdraft
// chain fd(k, l) for k = l down to 1 (zero elsewhere), plus the updraft chain fu(k, l) for
// k = l+1 up, plus the diagonal terms; f(0, l) = f(n, l) = 0.  conv1(k-1, l) =
// -dt (f(k-1, l) - f(k, l)), plus 1 on the diagonal.
__global__ void __launch_bounds__(GB_TUNE_MAX_CELL) k_convec_matrix(CArgs A) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int n = A.n;
    if (t >= (int64_t)A.ncol * n) return;
    const int c = (int)(t / n), l = (int)(t % n);
    if (!A.fresh[c]) return;
    const double *amu = chains(A, c), *zu = amu + (n + 1), *amd = zu + (n + 1), *zd = amd + (n + 1);
    const int i = A.cols[2 * c], j = A.cols[2 * c + 1];
    // the quotients this column of the matrix uses, each divided once: at level k = l + 1 the
    // chain starts (qed, qeu) and the sub-diagonal terms (qamd, qdk1); at k = l the diagonal's
    // (qamu, qdk2).  They share the divisor m(l): one reciprocal, each quotient correctly
    // rounded from it (div_by_recip: the division's bits)
    const double ml = AT(A.m, i, j, l);
    const double yl = recip_for(ml);
    const bool sub = l + 1 <= n - 1, dia = l >= 1;
    const double qamd = sub ? div_by_recip(amd[l + 1], ml, yl) : 0.0;
    const double qdk1 = sub ? div_by_recip(AT(A.dkg, i, j, l), ml, yl) : 0.0;
    const double qamu = dia ? div_by_recip(amu[l], ml, yl) : 0.0;
    const double qdk2 = dia ? div_by_recip(AT(A.dkg, i, j, l - 1), ml, yl) : 0.0;
    double *out = A.abuf + (size_t)c * n * n;
    const double mdt = -A.dt;
    const int top = A.top[i * A.ts0 + j * A.ts1], lfs = A.lfs[i * A.ts0 + j * A.ts1];
    // every element of rows k >= kend (1-based) is -dt (+0 - +0): above both the cloud and the
    // diagonal's two levels, the updraft chain u is +0 (its ratios are inactive), the downdraft
    // chain ends at the diagonal, and f(k - 1, l), f(k, l) are (+0 - +0) + -0 = +0
    const double off = mdt * (0.0 - 0.0);
    // The band of matrix column l where the chains are +0: f(l, l) and f(l+1, l) are the
    // general statements below with u = fd = +0, (+0 - qamu) + (-qdk2) and (+0 - qamd) + qdk1
    // (x - y = x + (-y) exactly), and the rows k = l, l+1, l+2 take -dt (f(k-1, l) - f(k, l)),
    // plus 1 at k = l+1; every other row of such a stretch is -dt (+0 - +0).  The band's values
    // are made once a lane and each row picks its own, so that no FP64 instruction is issued
    // row by row for the few lanes whose band that row is.
    const double nqdk2 = -qdk2;
    const double fl = dia ? (0.0 - qamu) + nqdk2 : 0.0;  // f(0, l) = 0: the surface
    const double fl1 = sub ? (0.0 - qamd) + qdk1 : 0.0;
    const double eb1 = mdt * (fl - fl1) + 1.0, eb2 = mdt * (fl1 - 0.0);
    if (top <= 0 && lfs <= 1) {
        // no cloud: every chain level is inactive, so u and fd are +0 throughout; f(l-1, l) = +0
        const double eb0 = mdt * (0.0 - fl);
        for (int k = 1; k <= n; ++k) {
            const int b = k - l;
            out[(size_t)(k - 1) * n + l] = b == 0 ? eb0 : (b == 1 ? eb1 : (b == 2 ? eb2 : off));
        }
        return;
    }
    const int kend = min(n, max(top, l + 1) + 1);  // the last row with terms of its own
    // R: the chains reach no row past it.  Above the cloud top the updraft's ratios are inactive
    // (u is +0, assigned), and fd(r, l) is +0, assigned, wherever r >= lfs (the downdraft's ratio
    // at r + 1 inactive); so in rows k > R both chains are +0 and only the band is left.  The
    // chain loops stop there: a warp's trip is then R, not the l + 2 of its highest lane.
    const int R = max(top, lfs) + 1;
    const int kg = min(kend, R);  // rows 1 .. kg by the chains' statements
    // the chains' first quotients, used only when a chain starts at or below R
    const double qed = l <= R ? div_by_recip(-AT(A.entd, i, j, l), ml, yl) : 0.0;
    const double qeu = l <= R ? div_by_recip(AT(A.entu, i, j, l), ml, yl) : 0.0;
    double fd[NMAX];
    double fprev = 0.0;
    {
        // Each statement below is one instruction for every lane of the warp (a lane's l selects its
        // operands, not its branch): the FP64 pipe issues per instruction, whatever its lanes.
        // fd(r, l) for r from l down: +0 from l down to R (each such ratio inactive), so the loop
        // starts at min(l, R) with the carried +0.
        double v = 0.0;
        for (int r = min(l, R); r >= 1; --r) {  // fd(r, l), r = k - 1 with k from l + 1 down to 2
            const double z = zd[r + 1];
            v = ge_zero(z) ? ((r == l) ? qed : v) * z : 0.0;
            fd[r] = v;
        }
        // the diagonal's terms (l == k: - qamu, then - qdk2) and the sub-diagonal's (l == k - 1:
        // - qamd, then + qdk1) as f = (f - s1) + s2, where the other lanes' s1 = +0 and s2 = -0
        // leave every f as it is (x - +0 = x, x + -0 = x, zeros and NaNs included)
        // The diagonal element (row k = l + 1, 1-based) takes e + 1.0: its e is kept and the sum made
        // once after the loop -- a sum inside it would be issued every row for the warp, its other
        // lanes predicated off.
        double u = 0.0, ediag = 0.0;
        for (int k = 1; k <= kg; ++k) {
            const double z = zu[k];
            // the updraft chain from l + 1 up: qeu z at k = l + 1, then u z; zero below
            u = (ge_zero(z) && l <= k - 1) ? ((l == k - 1) ? qeu : u) * z : 0.0;
            double fk = 0.0;
            if (k <= n - 1) {
                double f = u + (k <= l ? fd[k] : 0.0);
                const double s1 = (l == k) ? qamu : ((l == k - 1) ? qamd : 0.0);
                const double s2 = (l == k) ? nqdk2 : ((l == k - 1) ? qdk1 : -0.0);
                f = (f - s1) + s2;
                fk = f;
            }
            const double e = mdt * (fprev - fk);
            if (l == k - 1) ediag = e;
            else out[(size_t)(k - 1) * n + l] = e;
            fprev = fk;
        }
        if (l + 1 <= kg) out[(size_t)l * n + l] = ediag + 1.0;
    }
    // rows kg+1 .. kend (a lane whose band lies above R): f(k, l) is the band's, +0 below row l;
    // f(l-1, l) is the chains' last value when row l-1 is kg, else +0
    if (kend > kg) {
        const double eb0 = mdt * ((l - 1 == kg ? fprev : 0.0) - fl);
        for (int k = kg + 1; k <= kend; ++k) {
            const int b = k - l;
            out[(size_t)(k - 1) * n + l] = b == 0 ? eb0 : (b == 1 ? eb1 : (b == 2 ? eb2 : off));
        }
    }
    for (int k = kend + 1; k <= n; ++k) out[(size_t)(k - 1) * n + l] = off;
}

// thread per cloudless column: conv1 is tridiagonal.  When its three bands are finite and
// non-zero, the general Crout LU does, in its non-zero elements, exactly the recurrence
//   L(c, c-1) = A(c, c-1) / U(c-1, c-1),   U(c, c) = A(c, c) - L(c, c-1) A(c-1, c),
// U(c-1, c) = A(c-1, c): every other term it applies has a zero multiplier or multiplicand and
// only changes zeros, which are never used but as zero-tested multipliers.  Written here over
// its own band buffer (conv1 is left as it is, so that k_convec_lu, running beside it, reads the
// bands it tests unchanged): U's diagonal and L's band below (U's band above is conv1's); and the
// rows' term ends.  fresh = 2 tells k_convec_apply to take them from there and that L^-1 is still
// to be made from that band.  A column with a zero or non-finite band entry is left to the warp
// kernel, which makes the same test.

// whether k_convec_tri takes column c: a cloudless column made fresh whose three bands are all
// finite and non-zero (k_convec_lu takes the other fresh columns; the two run side by side)
__device__ __forceinline__ bool band_ok(double v) {
    const int64_t mag = __double_as_longlong(v) & 0x7fffffffffffffffLL;
    return mag != 0 && mag < 0x7ff0000000000000LL;  // neither zero, infinite nor NaN
}
__device__ __forceinline__ bool cloudless(const CArgs &A, int c) {
    const int i = A.cols[2 * c], j = A.cols[2 * c + 1];
    return A.top[i * A.ts0 + j * A.ts1] <= 0 && A.lfs[i * A.ts0 + j * A.ts1] <= 1;
}
__device__ __forceinline__ bool band_row_ok(const double *G, int n, int r) {
    return band_ok(G[(size_t)r * n + r]) &&
           (r + 1 >= n || (band_ok(G[(size_t)r * n + r + 1]) && band_ok(G[(size_t)(r + 1) * n + r])));
}

__global__ void __launch_bounds__(GB_TUNE_MAX_COLUMN) k_convec_tri(CArgs A) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= A.ncol || A.fresh[c] != 1 || !cloudless(A, c)) return;
    const int n = A.n;
    double *G = A.abuf + (size_t)c * n * n;
    int32_t *rend = A.rend + (size_t)c * n;
    double *ud = A.tband + (size_t)c * 2 * n, *lb = ud + n;
    // The bands are tested as the recurrence reads them (band_row_ok of every row): the band
    // buffer is this kernel's alone, so what it writes for a column that fails the test is never
    // read (fresh stays 1 and k_convec_lu makes that column); rend and fresh are written after.
    double uprev = G[0];  // U(r-1, r-1)
    bool ok = band_ok(uprev);
    ud[0] = uprev;
    constexpr int B = 8;  // rows whose bands are read into registers at once (loads in flight together)
    for (int r0 = 1; r0 < n; r0 += B) {
        double sub[B], dia[B], sup[B];
#pragma unroll
        for (int u = 0; u < B; ++u)
            if (r0 + u < n) {
                const int r = r0 + u;
                sub[u] = G[(size_t)r * n + r - 1];
                dia[u] = G[(size_t)r * n + r];
                sup[u] = G[(size_t)(r - 1) * n + r];
            }
#pragma unroll
        for (int u = 0; u < B; ++u) {
            const int r = r0 + u;
            if (r >= n) break;
            ok = ok && band_ok(sub[u]) && band_ok(dia[u]) && band_ok(sup[u]);
            const double l = div_ip(sub[u], uprev);
            const double v = dia[u] - l * sup[u];
            ud[r] = v;
            lb[r] = l;  // L(r, r-1): k_convec_apply builds L^-1 from it
            uprev = v;
        }
    }
    if (!ok) return;
    for (int r = 0; r < n; ++r) rend[r] = r + 1 < n ? r + 2 : r + 1;
    A.fresh[c] = 2;
}

// shared memory of one column of the LU (doubles): the matrix (conv1, then LU, then U over L^-1's
// strict lower triangle), one step's multipliers (n), and one step's list of the columns (or
// rows) it updates (NMAX int32)
__host__ __device__ __forceinline__ size_t warp_doubles(int n) { return (size_t)n * n + n + NMAX / 2; }

// e / d for 0 <= e < 2^16 and 1 <= d <= NMAX: the high word of e * (floor((2^32 - 1) / d) + 1),
// exact in that range (the multiplier exceeds 2^32 / d by less than 1, which moves e / d by
// less than 2^-16, below the 1 / d that separates it from the next integer)
__device__ __forceinline__ unsigned div_magic(int d) { return d > 1 ? 0xffffffffu / (unsigned)d + 1u : 0u; }
__device__ __forceinline__ int div_by(int e, int d, unsigned magic) {
    return d > 1 ? (int)__umulhi((unsigned)e, magic) : e;
}

// Where the warp LU stops: above its cloud a column's conv1 is tridiagonal (diffusion alone), and
// Crout's LU there does, in its non-zero elements, only the band recurrence of k_convec_tri.  E is
// one past the last row or column of an off-band non-zero of conv1: the LU of the leading E x E
// block is the reference's on those elements (no step k < E - 1 reaches a column >= E, and the rows
// >= E take only terms with a +-0 multiplier L(r, k), which leave a finite value as it is up to
// the sign of a zero -- never read again: the inverse's tail rows are built from the band), and
// from row E on the band recurrence continues from the block's last pivot (k_convec_tail).  The
// split is taken when the band from row E on passes k_convec_tri's test (finite, non-zero) and
// the block's elements and pivots stay finite and non-zero; otherwise E = n (the whole LU here).
// G lanes per column (32 / G columns a warp): every step's divisions and ballots serve the warp's
// columns at once.  Lanes of a group whose column is not made here (reused, k_convec_tri's, or past
// the list) take part in the warp's ballots with false predicates and do nothing else.
template <int G>
__device__ __forceinline__ int group_max(int v) {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(FULL_MASK, v, o, G));
    return v;
}
template <int G>
__device__ __forceinline__ bool group_all(bool p, unsigned gmask_shifted) {
    return (__ballot_sync(FULL_MASK, !p) & gmask_shifted) == 0;
}
__device__ __forceinline__ bool finite(double v) {
    return (__double_as_longlong(v) & 0x7fffffffffffffffLL) < 0x7ff0000000000000LL;
}

template <int G>
__global__ void __launch_bounds__(GB_TUNE_MAX_LU_WARPS * 32) k_convec_lu(CArgs A) {
    extern __shared__ double smem[];
    constexpr int MPW = 32 / G, NCH = NMAX / G;
    constexpr unsigned GMASK = G == 32 ? 0xffffffffu : ((1u << (G % 32)) - 1u);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int h = lane / G, gl = lane % G;  // the group (column) in the warp, the lane in the group
    const unsigned gshift = G == 32 ? 0xffffffffu : (GMASK << (h * G));
    const int c = (blockIdx.x * (blockDim.x >> 5) + warp) * MPW + h;
    const int n = A.n;
    // made in this call (k_convec_tri, beside this kernel, turns its columns' 1 into 2: the test
    // reads 0 or not, which that write does not change), and not k_convec_tri's: a cloudless
    // column is its unless a band entry is zero or not finite
    bool mine = c < A.ncol && A.fresh[c] != 0;
    const bool cand = mine && cloudless(A, c);
    bool ok = true;
    if (cand) {
        const double *G0 = A.abuf + (size_t)c * n * n;
        for (int r = gl; r < n; r += G) ok = ok && band_row_ok(G0, n, r);
    }
    const unsigned bad = (__ballot_sync(FULL_MASK, cand && !ok) >> (h * G)) & GMASK;
    mine = mine && !(cand && bad == 0);
    if (__ballot_sync(FULL_MASK, mine) == 0) return;  // the whole warp
    double *LU = smem + ((size_t)warp * MPW + h) * warp_doubles(n);  // n x n
    double *mult = LU + (size_t)n * n;                                 // n: step k's multipliers L(r, k)
    int32_t *list = reinterpret_cast<int32_t *>(mult + n);             // NMAX: a step's columns or rows
    double *Gm = A.abuf + (size_t)c * n * n;
    // ---- the leading block: E from conv1's off-band non-zeros, then the band's test from row E on
    if (mine)
        for (int e = gl; e < n * n; e += G) LU[e] = Gm[e];
    __syncwarp();
    int last = -1;
    if (mine)
        for (int e = gl; e < n * n; e += G) {
            const int r = e / n, col = e - r * n;
            if ((r - col > 1 || col - r > 1) && !is_zero(LU[e])) last = max(last, max(r, col));
        }
    int E = group_max<G>(last) + 1;
    {
        bool tail_ok = true;
        if (mine)
            for (int r = E + gl; r < n; r += G)  // rows >= E: the diagonal, and the band's two entries to row r - 1
                tail_ok = tail_ok && band_ok(LU[(size_t)r * n + r]) &&
                          (r == 0 || (band_ok(LU[(size_t)r * n + r - 1]) && band_ok(LU[(size_t)(r - 1) * n + r])));
        bool block_ok = true;
        if (mine)
            for (int e = gl; e < E * n; e += G) block_ok = block_ok && (e % n >= E || finite(LU[e]));
        if (!group_all<G>(tail_ok && block_ok, gshift)) E = n;
    }
    // Every loop below runs the warp's largest count (its ballots and __syncwarp take every lane);
    // a group acts on its own column's steps only (act, k < E).
    bool act = mine;
    for (int pass = 0; pass < 2; ++pass) {
        const int Ew = __reduce_max_sync(FULL_MASK, act ? E : 0);
        // ---- LU of the leading E x E block, right-looking: at step k, L's column k (its rows below
        // k divided by U(k, k), final after the steps before k), then every later element (r, c)
        // receives its term k, A(r, c) - L(r, k) U(k, c) -- the (row, column) elements packed onto
        // the group's lanes.  Each element receives its terms in k order, each skipped exactly where
        // Crout's column-by-column form skips it (the multiplier U(k, c) a zero: above a column's
        // first non-zero such zeros stay zero), and L's column is divided after all its terms: the
        // same operations on every element, the same bits.
        for (int k = 0; k < Ew; ++k) {
            const bool on = act && k < E;
            if (on) {
                const double d = LU[(size_t)k * n + k];
                for (int r = k + 1 + gl; r < E; r += G) LU[(size_t)r * n + k] = div_ip(LU[(size_t)r * n + k], d);
            }
            // row k's non-zeros right of the diagonal inside the block, listed in order: the
            // columns step k updates
            int ncols = 0;
#pragma unroll
            for (int s = 0; s < NCH; ++s) {
                const int col = s * G + gl;
                const bool p = on && col > k && col < E && !is_zero(LU[(size_t)k * n + col]);
                const unsigned b = (__ballot_sync(FULL_MASK, p) >> (h * G)) & GMASK;
                if (p) list[ncols + __popc(b & ((1u << gl) - 1u))] = col;
                ncols += __popc(b);
            }
            __syncwarp();
            if (on) {
                const int nrow = E - k - 1;
                const unsigned magic = div_magic(nrow);
                for (int e = gl; e < nrow * ncols; e += G) {
                    const int q = div_by(e, nrow, magic), r = k + 1 + (e - q * nrow);
                    const int col = list[q];
                    LU[(size_t)r * n + col] = LU[(size_t)r * n + col] - LU[(size_t)r * n + k] * LU[(size_t)k * n + col];
                }
            }
            __syncwarp();
        }
        // a split block keeps finite values and non-zero pivots, or the column is made whole
        bool fine = true;
        if (act && E < n)
            for (int e = gl; e < E * n; e += G) {
                const int r = e / n, col = e - r * n;
                if (col < E) fine = fine && finite(LU[e]) && (col != r || !is_zero(LU[e]));
            }
        const bool all_fine = group_all<G>(fine, gshift);  // every lane: a ballot
        const bool redo = act && E < n && !all_fine;
        if (pass == 1 || __ballot_sync(FULL_MASK, redo) == 0) break;
        // a singular or overflowing block: the whole LU over conv1 again, for those columns alone
        act = redo;
        if (redo) {
            E = n;
            for (int e = gl; e < n * n; e += G) LU[e] = Gm[e];
        }
        __syncwarp();
    }
    // ---- forward substitution of the identity: Y = L^-1, in place of L's strict lower triangle
    // (Y's diagonal is 1 and its upper triangle +0, U stays where it is), on the block's rows.
    // Row k of Y is final once the terms of rows < k are in; its term then goes to every later
    // row r with L(r, k) != 0 at once, Y(r, c) = Y(r, c) - L(r, k) Y(k, c) for the columns c <= k,
    // the (r, c) elements packed onto the group's lanes -- each element still in k order.  Step k
    // is the first to touch column k of Y: its elements start as the identity's +0 (Y(k, k) is the
    // identity's 1), and L(r, k) is taken into `mult` first, since the step overwrites it.
    const int Ew = __reduce_max_sync(FULL_MASK, mine ? E : 0);
    for (int k = 0; k < Ew - 1; ++k) {
        const bool on = mine && k < E - 1;
        // the rows below k with L(r, k) != 0, listed in order
        int nr = 0;
#pragma unroll
        for (int s = 0; s < NCH; ++s) {
            const int r = k + 1 + s * G + gl;
            const bool p = on && r < E && !is_zero(LU[(size_t)r * n + k]);
            const unsigned b = (__ballot_sync(FULL_MASK, p) >> (h * G)) & GMASK;
            if (p) list[nr + __popc(b & ((1u << gl) - 1u))] = r;
            nr += __popc(b);
        }
        if (on)
            for (int r = k + 1 + gl; r < E; r += G) {  // the lane that tested row r above
                mult[r] = LU[(size_t)r * n + k];
                LU[(size_t)r * n + k] = 0.0;  // Y(r, k) before its terms: the identity's +0
            }
        __syncwarp();
        if (on) {
            const int w = k + 1;  // the columns 0..k
            const unsigned magic = div_magic(w);
            for (int e = gl; e < nr * w; e += G) {
                const int q = div_by(e, w, magic), col = e - q * w;
                const int r = list[q];
                const double ykc = col == k ? 1.0 : LU[(size_t)k * n + col];  // Y(k, col)
                LU[(size_t)r * n + col] = LU[(size_t)r * n + col] - mult[r] * ykc;
            }
        }
        __syncwarp();
    }
    // ---- out: the block's rows -- U (the upper triangle with the diagonal) over conv1, L^-1 into
    // the inverse's place -- and for each of them one past its last non-zero right of the diagonal
    // (the back substitution's terms end there: the rest are zeros it would skip).  The rows from
    // E on are k_convec_tail's and the apply's (their conv1 band stays in place).
    if (mine) {
        double *X = A.inv + (size_t)c * n * n;
        for (int e = gl; e < E * n; e += G) {
            const int r = e / n, col = e % n;
            Gm[e] = LU[e];  // the back substitution reads U only (the diagonal and right of it)
            X[e] = r > col ? LU[e] : (r == col ? 1.0 : 0.0);
        }
        if (gl == 0) A.eblk[c] = E;
    }
    int32_t *rend = A.rend + (size_t)c * n;
    for (int r = 0; r < Ew; ++r) {  // (the lists are done with: their last readers passed a __syncwarp)
        const bool on = mine && r < E;
        int lastc = r;
#pragma unroll
        for (int s = 0; s < NCH; ++s) {
            const int col = s * G + gl;
            const bool p = on && col > r && col < n && !is_zero(LU[(size_t)r * n + col]);
            const unsigned b = (__ballot_sync(FULL_MASK, p) >> (h * G)) & GMASK;
            if (b) lastc = s * G + 31 - __clz(b);
        }
        if (on && gl == 0) rend[r] = lastc + 1;
    }
}

// thread per column k_convec_lu split (E < n): the band recurrence of k_convec_tri from row E on,
// continued from the block's last pivot U(E - 1, E - 1) (conv1's own U(0, 0) when E = 0): U's
// diagonal and L's band for the rows >= E into the band buffer, and their rows' term ends.
__global__ void __launch_bounds__(GB_TUNE_MAX_COLUMN) k_convec_tail(CArgs A) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= A.ncol || A.fresh[c] != 1) return;
    const int n = A.n, E = A.eblk[c];
    if (E >= n) return;
    const double *G = A.abuf + (size_t)c * n * n;
    int32_t *rend = A.rend + (size_t)c * n;
    double *ud = A.tband + (size_t)c * 2 * n, *lb = ud + n;
    int r0 = E;
    double uprev;
    if (E == 0) {
        uprev = G[0];
        ud[0] = uprev;
        r0 = 1;
    } else {
        uprev = G[(size_t)(E - 1) * n + E - 1];
    }
    constexpr int B = 8;  // rows whose bands are read into registers at once (loads in flight together)
    for (; r0 < n; r0 += B) {
        double sub[B], dia[B], sup[B];
#pragma unroll
        for (int u = 0; u < B; ++u)
            if (r0 + u < n) {
                const int r = r0 + u;
                sub[u] = G[(size_t)r * n + r - 1];
                dia[u] = G[(size_t)r * n + r];
                sup[u] = G[(size_t)(r - 1) * n + r];
            }
#pragma unroll
        for (int u = 0; u < B; ++u) {
            const int r = r0 + u;
            if (r >= n) break;
            const double l = div_ip(sub[u], uprev);
            const double v = dia[u] - l * sup[u];
            ud[r] = v;
            lb[r] = l;
            uprev = v;
        }
    }
    for (int r = E; r < n; ++r) rend[r] = r + 1 < n ? r + 2 : r + 1;
}

__global__ void k_convec_apply(CArgs A) {
    extern __shared__ double recip[];  // cols_per_block x n: RN(1 / U(r, r)) of each column's rows
    const int n = A.n;
    const int cl = threadIdx.x / n, x = threadIdx.x % n;  // column in the block, its thread
    const int c = blockIdx.x * A.cols_per_block + cl;
    const bool live = cl < A.cols_per_block && c < A.ncol;
    double *X = live ? A.inv + (size_t)c * n * n : nullptr;
    // the rows from E on are band rows (k_convec_tri's columns: all of them; a column k_convec_lu
    // split: those past its block): U's diagonal and L's band in the band buffer
    const int fr = live ? A.fresh[c] : 0;
    const int E = fr == 2 ? 0 : (fr == 1 ? A.eblk[c] : n);
    const double *ud = E < n ? A.tband + (size_t)c * 2 * n : nullptr;
    const double *U = live ? A.abuf + (size_t)c * n * n : nullptr;
    // ---- the reciprocals of U's diagonal, one a thread: every quotient of row r shares U(r, r)
    if (fr) recip[cl * n + x] = recip_for(x >= E ? ud[x] : U[(size_t)x * n + x]);
    // ---- the band rows of L^-1, column x: the forward substitution of the identity with L's
    // single band there, Y(r, x) = +0 - L(r, r-1) Y(r-1, x) below the diagonal (the terms of a
    // zero L(r, r-1) it skips leave the +0 that this writes), 1 on it, +0 above; from Y(E - 1, x)
    // (the block's last row, k_convec_lu's) in the block's columns
    if (fr && E < n) {
        const double *lb = ud + n;
        double y;
        int r0;
        if (x >= E) {
            for (int r = E; r < x; ++r) X[(size_t)r * n + x] = 0.0;
            X[(size_t)x * n + x] = 1.0;
            y = 1.0;
            r0 = x + 1;
        } else {
            y = X[(size_t)(E - 1) * n + x];
            r0 = E;
        }
        for (int r = r0; r < n; ++r) {
            y = zero_minus(lb[r] * y);  // 0.0 - lb[r] y
            X[(size_t)r * n + x] = y;
        }
    }
    __syncthreads();
    // ---- back substitution of inverse column x: rows from the bottom, terms k in order; each
    // quotient by the row's shared reciprocal, correctly rounded (div_by_recip)
    if (fr) {
        const int32_t *rend = A.rend + (size_t)c * n;
        const double *rc = recip + cl * n;
        for (int r = n - 1; r >= 0; --r) {
            double a = X[(size_t)r * n + x];
            for (int k = r + 1; k < rend[r]; ++k) {
                const double w = U[(size_t)r * n + k];
                if (is_zero(w)) continue;
                a = sub_ip(a, w * X[(size_t)k * n + x]);
            }
            X[(size_t)r * n + x] = div_by_recip(a, r >= E ? ud[r] : U[(size_t)r * n + r], rc[r]);
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
            for (int k = 0; k < n; ++k) zr = add_ip(zr, C[k] * AT4(A.q[0], i, j, k, t));
        __syncthreads();  // every thread of the column has read rm(., t)
        if (live) AT4(A.q[0], i, j, l, t) = zr;
    }
}

int gcd(int a, int b) { return b == 0 ? a : gcd(b, a % b); }

// Columns per block of k_convec_apply (whole columns: a column's threads share its reciprocals
// and meet at the block's barriers).  least > 0: at least `least` threads, as many columns as
// make whole warps, and a call of few columns spread over the device.  least == 0: the count
// that evens out the FP64 work over the SMs -- a block issues as many warp instructions as it
// has warps (a part-filled warp issues as a full one), and the busiest SM runs ceil(blocks /
// SMs) of them; the fewest such warps, with the most columns a block among equals.
int apply_columns_per_block(int ncol, int lmax, int least, int sms) {
    const int whole = 32 / gcd(lmax, 32);  // columns that fill whole warps
    int per = whole;
    while (per > 1 && per * lmax > 1024) per /= 2;
    if (least > 0) {
        if (per * lmax < least) per = (least + lmax - 1) / lmax;
        while (per > 1 && ((per * lmax + 31) / 32) * 32 > 1024) --per;
        // a call of few columns (a segment along a child's footprint) spread over the device: its
        // FP64 work would otherwise queue on the few multiprocessors its few blocks land on
        while (per > 1 && (ncol + per - 1) / per < sms) per /= 2;
        return per;
    }
    int best = per;
    long long best_cost = -1;
    for (int p = per; p >= 1; --p) {
        const long long blocks = (ncol + p - 1) / p;
        const long long cost = ((blocks + sms - 1) / sms) * ((p * lmax + 31) / 32);
        if (best_cost < 0 || cost < best_cost) {
            best_cost = cost;
            best = p;
        }
    }
    return best;
}

template <int G>
int launch_lu_g(gb_ctx *ctx, const CArgs &A) {
    constexpr int MPW = 32 / G;
    int warps = ctx->tune[GB_TUNE_LU_WARPS];
    while (warps > 1 && (size_t)warps * MPW * warp_doubles(A.n) * sizeof(double) > 227 * 1024) warps /= 2;
    const size_t smem = (size_t)warps * MPW * warp_doubles(A.n) * sizeof(double);
    GB_CHECK_CUDA(cudaFuncSetAttribute(k_convec_lu<G>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_convec_lu<G><<<gb_blocks(A.ncol, warps * MPW), warps * 32, smem, ctx->stream>>>(A);
    return gb_after_launch(ctx, "convec_lu");
}

int launch_lu(gb_ctx *ctx, const CArgs &A, int lanes) {
    switch (lanes) {
        case 8: return launch_lu_g<8>(ctx, A);
        case 16: return launch_lu_g<16>(ctx, A);
        default: return launch_lu_g<32>(ctx, A);
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
    const size_t nn = (size_t)lmax * lmax;
    // work space: conv1 / U of every column, the chains, the fresh flags, and the inverses
    // without a cache
    const size_t nchain = (size_t)NCHAIN * (lmax + 1) * ncol, nflag = ((size_t)ncol + 1) / 2;
    const size_t nrend = ((size_t)ncol * lmax + 1) / 2;
    const size_t ntband = (size_t)ncol * 2 * lmax;
    const size_t doubles = nn * ncol + nchain + 2 * nflag + nrend + ntband + (cache_inv ? 0 : nn * ncol);
    double *w = gb_work(ctx, doubles * sizeof(double));
    if (!w) return GB_ECUDA;
    A.abuf = w;
    A.chain = w + nn * ncol;
    A.fresh = reinterpret_cast<int32_t *>(A.chain + nchain);
    A.eblk = reinterpret_cast<int32_t *>(A.chain + nchain + nflag);
    A.rend = reinterpret_cast<int32_t *>(A.chain + nchain + 2 * nflag);
    A.tband = A.chain + nchain + 2 * nflag + nrend;
    A.inv = cache_inv ? cache_inv : A.tband + ntband;
    A.cache_m = cache_inv ? cache_m : nullptr;
    A.cache_tag = cache_tag;
    A.epoch = epoch;
    const int tcol = ctx->tune[GB_TUNE_COLUMN_THREADS], tcell = ctx->tune[GB_TUNE_CELL_THREADS];
    k_convec_chains<<<gb_blocks(ncol, tcol), dim3(tcol, 3), 0, ctx->stream>>>(A);
    if (int rc = gb_after_launch(ctx, "convec_chains")) return rc;
    k_convec_ratios<<<gb_blocks((int64_t)ncol * lmax, tcell), tcell, 0, ctx->stream>>>(A);
    if (int rc = gb_after_launch(ctx, "convec_ratios")) return rc;
    k_convec_matrix<<<gb_blocks((int64_t)ncol * lmax, tcell), tcell, 0, ctx->stream>>>(A);
    if (int rc = gb_after_launch(ctx, "convec_matrix")) return rc;
    // the cloudless columns' recurrence on the side stream, beside the LU of the others: each
    // kernel decides the same split (cloudless with regular bands: tri's), so they share nothing
    GB_CHECK_CUDA(cudaEventRecord(ctx->fork, ctx->stream));
    GB_CHECK_CUDA(cudaStreamWaitEvent(ctx->side, ctx->fork, 0));
    k_convec_tri<<<gb_blocks(ncol, tcol), tcol, 0, ctx->side>>>(A);
    if (int rc = gb_after_launch(ctx, "convec_tri")) return rc;
    // warps per LU block and lanes per column: the tuned counts, fewer warps where their shared
    // memory would not fit
    if (int rc = launch_lu(ctx, A, ctx->tune[GB_TUNE_LU_LANES])) return rc;
    // the band rows above the blocks k_convec_lu split off, thread per column
    k_convec_tail<<<gb_blocks(ncol, tcol), tcol, 0, ctx->stream>>>(A);
    if (int rc = gb_after_launch(ctx, "convec_tail")) return rc;
    GB_CHECK_CUDA(cudaEventRecord(ctx->join, ctx->side));
    GB_CHECK_CUDA(cudaStreamWaitEvent(ctx->stream, ctx->join, 0));
    // whole columns per block, as many as make the block a whole number of warps (<= 1024
    // threads), and at least the tuned block size
    A.cols_per_block = apply_columns_per_block(ncol, lmax, ctx->tune[GB_TUNE_APPLY_THREADS], ctx->sms);
    const int per = A.cols_per_block;
    const int threads = ((per * lmax + 31) / 32) * 32;
    k_convec_apply<<<(ncol + per - 1) / per, threads, (size_t)per * lmax * sizeof(double), ctx->stream>>>(A);
    return gb_after_launch(ctx, "convec_apply");
}
