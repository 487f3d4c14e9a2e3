// Shared pieces of the gbdyn kernels: the context, device views, the status word, and the
// per-element arithmetic of the slopes scheme in NumPy's evaluation order.
//
// Every kernel is float64 and compiled with -fmad=false: no multiply-add contraction, no
// reassociation, IEEE division and square root.  That is what makes each element's value the
// one the NumPy reference computes.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>

#include "../../include/gbdyn.h"

// ------------------------------------------------------------------ context
struct gb_ctl {         // device-resident control block, one per context
    int status;         // GB_* error bits, or-ed by kernels
    int cfl_failed;     // Check_CFL rehearsal: an operator exceeded its cap
    int zsearch_n[8];   // z search rounds: candidate n_advz after each round
    int zsearch_changed[8];
    int ysearch_fail;   // scratch
    int pad[5];
    double stats[4];
};

struct gb_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;   // a second stream an operator forks independent work onto
    cudaEvent_t fork = nullptr, join = nullptr;  // (timing disabled) its fork and join
    gb_ctl *ctl = nullptr;         // device
    int32_t *scratch_i = nullptr;  // per-op integer scratch (layer nloops, ...)
    size_t scratch_i_n = 0;
    double *work = nullptr;        // per-op float64 work space, grown outside capture (gb_work)
    size_t work_bytes = 0;
    int64_t launches = 0;
    int tune[GB_TUNE_N] = {64, 128, 2, 0, 32};  // launch shapes (GB_TUNE_*)
    bool capturing = false;
    int64_t capture_launches = 0;
    int sms = 1;  // the device's multiprocessors (grids of small calls are spread over them)
};

void gb_set_error(const std::string &msg);
int gb_cuda_fail(cudaError_t e, const char *what);
int gb_after_launch(gb_ctx *ctx, const char *what);
int32_t *gb_scratch_i(gb_ctx *ctx, size_t n);
double *gb_work(gb_ctx *ctx, size_t bytes);  // nullptr (error set) if it cannot be had

#define GB_CHECK_CUDA(call)                                   \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return gb_cuda_fail(e_, #call); \
    } while (0)

// ------------------------------------------------------------------ views
struct DV {  // device view of a float64 array, rank <= 4
    double *p;
    int64_t n0, n1, n2, n3;
    int64_t s0, s1, s2, s3;
};

static inline DV dv(const gb_view *v) {
    DV d;
    d.p = (double *)v->p;
    d.n0 = v->n[0]; d.n1 = v->n[1]; d.n2 = v->n[2]; d.n3 = v->n[3];
    d.s0 = v->s[0]; d.s1 = v->s[1]; d.s2 = v->s[2]; d.s3 = v->s[3];
    return d;
}

// ------------------------------------------------------------------ bit tests
// isnan, |x| and -x on the integer pipe: on this GPU the FP64 pipe is the scarce unit, and a
// compare or a sign change issued there costs as much as a multiply.  Exact for every input.
__device__ __forceinline__ bool gb_isnan(double x) {
    return (unsigned long long)(__double_as_longlong(x) & 0x7fffffffffffffffLL) > 0x7ff0000000000000ULL;
}
__device__ __forceinline__ double gb_abs(double x) {
    return __longlong_as_double(__double_as_longlong(x) & 0x7fffffffffffffffLL);
}
__device__ __forceinline__ double gb_neg(double x) {
    return __longlong_as_double(__double_as_longlong(x) ^ (long long)0x8000000000000000ULL);
}

// The ordered compares a < b, a <= b, a > b, a >= b, x > 0 on the integer pipe, true and false
// exactly where the FP64 compares are: false when either operand is a NaN, +0 equal to -0.  The
// sign-magnitude image of the bit patterns (the bits where the sign is clear, INT64_MIN - bits
// where it is set) orders every non-NaN double as its value, both zeros at 0.
__device__ __forceinline__ long long gb_ord(double x) {
    const long long b = __double_as_longlong(x);
    return b >= 0 ? b : (long long)(0x8000000000000000ULL - (unsigned long long)b);
}
__device__ __forceinline__ bool gb_lt(double a, double b) {
    return !gb_isnan(a) && !gb_isnan(b) && gb_ord(a) < gb_ord(b);
}
__device__ __forceinline__ bool gb_le(double a, double b) {
    return !gb_isnan(a) && !gb_isnan(b) && gb_ord(a) <= gb_ord(b);
}
__device__ __forceinline__ bool gb_gt(double a, double b) { return gb_lt(b, a); }
__device__ __forceinline__ bool gb_ge(double a, double b) { return gb_le(b, a); }
__device__ __forceinline__ bool gb_gt0(double x) {  // x > 0.0: positive, not a zero, not a NaN
    const long long b = __double_as_longlong(x);
    return b > 0 && b <= 0x7ff0000000000000LL;
}

// abs(c / mu) < 1.0 (the sub-cycle searches' Courant test, ops.py:330-341) without the division
// where the answer is certain: |c| < fl(0.9999 |mu|) puts the quotient below 0.9999 (1 + 2^-53)
// < 1 - 2^-54, so it rounds below 1 (for subnormal |mu| too); |c| > |mu| puts it above 1.  The
// band between, zeros, NaNs and infinities take the division itself.
__device__ __forceinline__ bool cfl_pass(double c, double mu) {
    const double ac = gb_abs(c), am = gb_abs(mu);
    if (ac < am * 0.9999) return true;
    if (ac > am) return false;
    return gb_abs(c / mu) < 1.0;
}

// a / d, correctly rounded, from y = RN(1 / d) shared by many quotients of one divisor
// (Markstein's correction, IBM J. Res. Develop. 34(1), 1990): q0 = RN(a y), then twice
// r = a - d q (exact by FMA while q is within an ulp of a / d) and q = RN(q + r y).  q0 is within
// 1.5 ulp of a / d, the first correction brings it within half an ulp plus a few 2^-52 ulp, and
// from within one ulp Markstein's theorem makes the second exact: RN(a / d).  One multiply and
// four FMAs on the FP64 pipe, where a division costs eight.  The proof needs normal operands
// and results away from overflow and underflow: a zero a (whose quotient is a y, signed as a / d),
// and anything outside |a| >= 2^-960, |d| in [2^-1000, 2^1000], |a / d| in [2^-1001, 2^1001],
// take the division itself, as does y = 0 (the caller's mark for a divisor outside that range).
__device__ __forceinline__ double recip_for(double d) {
    const int ed = (int)((__double_as_longlong(d) >> 52) & 0x7ff);
    return (ed >= 23 && ed <= 2023) ? 1.0 / d : 0.0;
}
// recip_for(d) from an inv = 1.0 / d the caller makes anyway (an integer test, no division)
__device__ __forceinline__ double recip_mark(double d, double inv) {
    const int ed = (int)((__double_as_longlong(d) >> 52) & 0x7ff);
    return (ed >= 23 && ed <= 2023) ? inv : 0.0;
}
__device__ __forceinline__ double div_by_recip(double a, double d, double y) {
    const unsigned long long ab = (unsigned long long)__double_as_longlong(a);
    if (((unsigned long long)__double_as_longlong(y) << 1) != 0) {
        if ((ab << 1) == 0) return a * y;
        const int ea = (int)((ab >> 52) & 0x7ff), ed = (int)((__double_as_longlong(d) >> 52) & 0x7ff);
        const int diff = ea - ed;
        if (ea >= 63 && ea <= 2023 && diff >= -1000 && diff <= 1000) {
            const double q0 = a * y;
            const double q1 = __fma_rn(__fma_rn(-q0, d, a), y, q0);
            return __fma_rn(__fma_rn(-q1, d, a), y, q1);
        }
    }
    return a / d;
}

// x >= 0.0 and x < 0.0 on the integer pipe (an FP64 compare issues on the FP64 pipe): >= holds
// from +0 to +inf and at -0; < from the smallest negative to -inf; a NaN fails both
__device__ __forceinline__ bool ge_zero(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    return b <= 0x7ff0000000000000ULL || b == 0x8000000000000000ULL;
}
__device__ __forceinline__ bool lt_zero(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    return b > 0x8000000000000000ULL && b <= 0xfff0000000000000ULL;
}

// ------------------------------------------------------------------ NumPy's element rules
// np.clip(s, -|r|, |r|) exactly as NumPy evaluates it: a NaN in s wins, then max with the lower
// bound ((s > lo) ? s : lo), then a NaN wins again, then min with the upper bound.  Both compares
// are made on the integer pipe from the magnitudes' bit patterns (which order as the values do):
// with lo = -|r|, s > lo holds for a negative s (either zero included) where |s| < |r|, and for
// a non-negative s unless s and r are both zeros (+0 > -0 is false); t < hi = |r| holds for a
// negative t where t and r are not both zeros, for a non-negative t where |t| < |r|.  A NaN r
// makes lo a NaN: s > lo fails, and t = lo is returned.
__device__ __forceinline__ double np_limit(double s, double r) {
    const unsigned long long MAG = 0x7fffffffffffffffULL, INF = 0x7ff0000000000000ULL;
    const unsigned long long bs = (unsigned long long)__double_as_longlong(s);
    const unsigned long long as = bs & MAG, ar = (unsigned long long)__double_as_longlong(r) & MAG;
    const double hi = __longlong_as_double((long long)ar), lo = __longlong_as_double((long long)(ar | ~MAG));
    if (as > INF) return s;
    if (ar > INF) return lo;
    const bool sneg = (bs >> 63) != 0;
    const bool gt = sneg ? as < ar : (as | ar) != 0;  // s > lo
    const unsigned long long at = gt ? as : ar;      // |t|, t = gt ? s : lo
    const bool tneg = gt ? sneg : true;
    const bool lt = tneg ? (at | ar) != 0 : at < ar;  // t < hi
    return lt ? (gt ? s : lo) : hi;
}

// np.maximum(a, b): NaN in a, else NaN in b, else (a > b ? a : b), the compare on the integer pipe
// (gb_ord; neither is a NaN by then).
__device__ __forceinline__ double np_max(double a, double b) {
    return gb_isnan(a) ? a : (gb_isnan(b) ? b : (gb_ord(a) > gb_ord(b) ? a : b));
}
__device__ __forceinline__ double np_min(double a, double b) {
    return gb_isnan(a) ? a : (gb_isnan(b) ? b : (gb_ord(a) < gb_ord(b) ? a : b));
}

// Tracer fluxes of the slopes scheme through one face (pydyn kernels.py:75-84): the flux,
// its Courant number c and the upwind cell's mass rm_u, along-slope s_u and cross slopes.
__device__ __forceinline__ void slopes_flux(double flux, double c, double rm_u, double s_u,
                                            double t_u, double w_u, double &f, double &pf,
                                            double &ft, double &fw) {
    double ff;
    if (ge_zero(flux))
        ff = c * (rm_u + (1.0 - c) * s_u);
    else
        ff = c * (rm_u - (1.0 + c) * s_u);
    f = ff;
    pf = flux * (c * c * s_u - 3.0 * ff);
    ft = c * t_u;
    fw = c * w_u;
}

// The along-flow slope after one sub-step (kernels.py:87-92):
// s + (pf_lo - pf_hi - (lo - hi) s + 3 ((lo + hi) rm_new - (f_lo + f_hi) m_old)) / m_new
__device__ __forceinline__ double along_slope(double s, double pf_lo, double pf_hi, double lo,
                                              double hi, double rm_new, double f_lo, double f_hi,
                                              double m_old, double m_new) {
    double num = ((pf_lo - pf_hi) - (lo - hi) * s) + 3.0 * ((lo + hi) * rm_new - (f_lo + f_hi) * m_old);
    return s + num / m_new;
}
// the same with the division num / m_new made from y_new = recip_for(m_new) (div_by_recip: the
// division's bits), where the caller has the reciprocal of the new mass for other uses
__device__ __forceinline__ double along_slope_y(double s, double pf_lo, double pf_hi, double lo,
                                                double hi, double rm_new, double f_lo, double f_hi,
                                                double m_old, double m_new, double y_new) {
    double num = ((pf_lo - pf_hi) - (lo - hi) * s) + 3.0 * ((lo + hi) * rm_new - (f_lo + f_hi) * m_old);
    return s + div_by_recip(num, m_new, y_new);
}

// The progressive rescale of dynamu / dynamv (ops.py:304-307): f * (n - 1) / n, evaluated
// left to right, applied once per retry n = 2 .. nloop.
__device__ __forceinline__ double progressive_chain(double f, int nloop) {
    for (int n = 2; n <= nloop; ++n) f = (f * (double)(n - 1)) / (double)n;
    return f;
}

__device__ __forceinline__ void raise_status(gb_ctl *ctl, int bits) { atomicOr(&ctl->status, bits); }

// max of non-negative doubles through their bit patterns (order-free)
__device__ __forceinline__ void atomic_max_nonneg(double *addr, double v) {
    atomicMax((unsigned long long *)addr, (unsigned long long)__double_as_longlong(v));
}

// the largest block a tunable kernel is compiled for (its __launch_bounds__)
constexpr int GB_TUNE_MAX_COLUMN = 256, GB_TUNE_MAX_CELL = 512, GB_TUNE_MAX_LU_WARPS = 4;
static inline unsigned gb_blocks(int64_t n, int threads) { return (unsigned)((n + threads - 1) / threads); }

#define GB_WARP 32
#define FULL_MASK 0xffffffffu
