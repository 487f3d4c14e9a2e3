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
// isnan, |x| and -x on the integer pipe: on GB300 the FP64 pipe is the scarce unit, and a
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

// a / d, correctly rounded, from y = RN(1 / d) shared by many quotients of one divisor: one
// multiply on the FP64 pipe, the rest on the integer pipe.  q0 = RN(a y) carries a relative
// error below 2^-52 ((1 + 2^-53)^2), so it lies within 2 ulp of a / d.  Where q0's significand
// mq is at least 1 and 5 ulp inside its binade, a / d lies in that binade, and the correctly
// rounded quotient is q0 + k ulp for k in -2..2: k = round(R / md), R = a - q0 d in units of
// ulp(q0) d / md.  With a = ma 2^Ea, d = md 2^Ed, q0 = mq 2^Eq (53-bit integer significands),
// R = ma 2^t - mq md for t = Ea - Eq - Ed (52 or 53 when q0 d is that close to a), an integer
// below 2 md < 2^54 in magnitude: its low 64 bits, (ma << t) - mq md, are all of it.  Rounding
// to nearest even compares 2|R| with md and 3 md (a tie -- which a quotient of two doubles
// never is -- goes to the even neighbour), and the neighbour is q0's bit pattern plus or minus k
// (the patterns of one sign run in the order of their magnitudes).  A zero a gives a y, signed
// as a / d.  y = 0 (the caller's mark for a divisor whose reciprocal is not a normal number),
// and any a, d or q0 outside that -- a zero d, subnormal, infinite or NaN operands, q0 at a
// binade's edge or not normal -- take the division itself, on the FP64 pipe, through a call
// (a predicated-off division beside the integer path would hold the FP64 pipe on every call).
// recip_for(d) from an inv = 1.0 / d the caller makes anyway (an integer test, no division)
__device__ __forceinline__ double recip_mark(double d, double inv) {
    const int ed = (int)((__double_as_longlong(d) >> 52) & 0x7ff);
    return (ed >= 23 && ed <= 2023) ? inv : 0.0;
}
static __device__ __noinline__ double div_fp64_pipe(double a, double d) { return a / d; }
__device__ __forceinline__ double div_by_recip(double a, double d, double y) {
    constexpr unsigned long long SIGN = 0x8000000000000000ULL, FRAC = 0xfffffffffffffULL, ONE = 0x10000000000000ULL;
    const double q0 = a * y;
    const unsigned long long ua = (unsigned long long)__double_as_longlong(a),
                             ud = (unsigned long long)__double_as_longlong(d),
                             uq = (unsigned long long)__double_as_longlong(q0);
    const int ea = (int)((ua >> 52) & 0x7ff), ed = (int)((ud >> 52) & 0x7ff), eq = (int)((uq >> 52) & 0x7ff);
    const int t = ea - eq - ed + 1075;
    const unsigned long long fq = uq & FRAC;
    const bool az = (ua << 1) == 0 && ((unsigned long long)__double_as_longlong(y) << 1) != 0;
    const bool fast = (unsigned)(ea - 1) < 2046u && (unsigned)(ed - 1) < 2046u && (unsigned)(eq - 1) < 2046u &&
                      (t == 52 || t == 53) && fq - 1 < FRAC - 4;  // 1 <= fq <= 2^52 - 5
    const unsigned long long ma = (ua & FRAC) | ONE, md = (ud & FRAC) | ONE, mq = fq | ONE;
    // (unsigned arithmetic throughout: outside the fast path the values are unused, and wrap)
    const unsigned long long Ru = (ma << (t & 63)) - mq * md;
    const long long R = (long long)Ru;
    const unsigned long long v = (R < 0 ? 0ULL - Ru : Ru) << 1, m3 = md * 3, odd = mq & 1;
    const unsigned long long k = (unsigned long long)(v > md || (v == md && odd)) +
                                 (unsigned long long)(v > m3 || (v == m3 && !odd));
    const unsigned long long mag = (uq & ~SIGN) + (R < 0 ? 0ULL - k : k);
    double r = __longlong_as_double((long long)((uq & SIGN) | mag));
    if (az) r = q0;
    else if (!fast) r = div_fp64_pipe(a, d);
    return r;
}

// a / d, correctly rounded, with three FP64 instructions where the FP64 pipe's own division
// issues eight.  The seed is an FP32 reciprocal: d truncated to FP32 (relative error below
// 2^-23) and rcp.approx.f32 (within one FP32 ulp, 2^-23), so y0 = 1 / d to within 2^-22.
// q0 = RN(a y0) then carries a relative error below 2^-21.9, and one correction
// q1 = RN(q0 + RN(a - q0 d) y0) squares it: below 2^-43.7, within 2^9.3 ulp of a / d.  Where
// q1's significand is 2048 ulp or more inside its binade, a / d lies in that binade and the
// correctly rounded quotient is q1 + k ulp, k = round(R / md), with R = ma 2^t - mq md the exact
// residual in units of ulp(q1) d / md (as in div_by_recip: t = Ea - Eq - Ed, 52 or 53, and
// |R| < 2^62.3, so the low 64 bits are all of it).  k comes from the top bits of R and md in FP32
// (within 0.16 of R / md), then is made exact by one test of the integer remainder R - k md
// against md / 2 (a tie would go to the even neighbour; a quotient of two doubles is never
// one).  A zero a gives a y0, signed as a / d.  Outside d in [2^-125, 2^125] (where the FP32
// seed and its reciprocal are normal), or with a, q1 not normal, or q1 near a binade's edge, the
// division is the FP64 pipe's own, through a call (a quotient that is always near a power of two,
// such as a midpoint's fraction 1/2, is better left to the plain division).
static __device__ __noinline__ double div_fp64_call(double a, double d) { return a / d; }
__device__ __forceinline__ double div_ip(double a, double d) {
    constexpr unsigned long long SIGN = 0x8000000000000000ULL, FRAC = 0xfffffffffffffULL, ONE = 0x10000000000000ULL;
    const unsigned long long ua = (unsigned long long)__double_as_longlong(a),
                             ud = (unsigned long long)__double_as_longlong(d);
    const int ea = (int)((ua >> 52) & 0x7ff), ed = (int)((ud >> 52) & 0x7ff);
    const bool seed_ok = (unsigned)(ed - 898) <= 250u;  // the FP32 image of d and its reciprocal normal
    const uint32_t fd = ((uint32_t)(ed - 896) << 23) | ((uint32_t)(ud >> 29) & 0x7fffffu);
    float rf;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rf) : "f"(__uint_as_float(fd)));
    const uint32_t ur = __float_as_uint(rf);
    const double y0 = __longlong_as_double((long long)((ud & SIGN) | ((unsigned long long)(((ur >> 23) & 0xffu) + 896u) << 52) |
                                                       ((unsigned long long)(ur & 0x7fffffu) << 29)));
    const double q0 = a * y0;
    const double q1 = __fma_rn(__fma_rn(-q0, d, a), y0, q0);
    const unsigned long long uq = (unsigned long long)__double_as_longlong(q1);
    const int eq = (int)((uq >> 52) & 0x7ff);
    const int t = ea - eq - ed + 1075;
    const unsigned long long fq = uq & FRAC;
    const bool fast = seed_ok && (unsigned)(ea - 1) < 2046u && (unsigned)(eq - 1) < 2046u && (t == 52 || t == 53) &&
                      fq - 2048 < FRAC - 4095;  // 2048 <= fq <= 2^52 - 2049
    const unsigned long long ma = (ua & FRAC) | ONE, md = (ud & FRAC) | ONE, mq = fq | ONE;
    // (the remainders in unsigned arithmetic, read as signed: outside the fast path the values are
    // unused, and wrap)
    const unsigned long long Ru = (ma << (t & 63)) - mq * md;
    const long long R = (long long)Ru, smd = (long long)md;
    unsigned long long k = (unsigned long long)(long long)__float2int_rn(
        __fdividef((float)(int)(R >> 40), (float)(int)(md >> 40)));
    const long long r2 = (long long)((Ru - k * md) << 1);
    k += (unsigned long long)((long long)(r2 > smd) - (long long)(r2 < -smd));
    const long long t2 = (long long)((Ru - k * md) << 1);
    if ((t2 == smd || t2 == -smd) && ((mq + k) & 1) != 0) k += t2 > 0 ? 1ULL : 0ULL - 1ULL;
    double r = __longlong_as_double((long long)((uq & SIGN) | ((uq & ~SIGN) + k)));
    if ((ua << 1) == 0 && seed_ok) r = q0;
    else if (!fast) r = div_fp64_call(a, d);
    return r;
}

// sqrt(x), correctly rounded, with two FP64 instructions where the FP64 pipe's own square root
// issues eight.  x = 1.f 2^(2q + p): the seed is the correctly rounded FP32 root of 1.f 2^p
// (significand truncated to FP32: s0 within 2^-23 of sqrt(x) once scaled by 2^q) and the FP32
// reciprocal of that root (rcp.approx.f32, within one ulp) for h0 = 1 / (2 s0).  One Newton step
// s1 = RN(s0 + RN(x - s0^2) h0) leaves a relative error below 2^-44.6, within 2^8.4 ulp.  Where
// s1's significand is 1024 ulp or more inside its binade, the root lies in that binade; with
// x 2^-2Es = X = mx 2^t (t = Ex - 2 Es, 52 or 53) and c = ms + k the candidate significand, c is
// the correctly rounded root exactly when (c - 1/2)^2 < X < (c + 1/2)^2, i.e. -c < X - c^2 <= c
// for the integer X - c^2 (a root of a double is never a midpoint).  X - ms^2 is below 2^62.4 in
// magnitude: its low 64 bits are all of it; k starts from its top bits over 2 ms in FP32 and is
// moved by one until the test holds.  A zero is its own root.  Negative, subnormal, infinite and
// NaN x, and s1 near a binade's edge, take the FP64 pipe's square root through a call.
static __device__ __noinline__ double sqrt_fp64_call(double x) { return sqrt(x); }
__device__ __forceinline__ double sqrt_ip(double x) {
    constexpr unsigned long long FRAC = 0xfffffffffffffULL, ONE = 0x10000000000000ULL;
    const unsigned long long ux = (unsigned long long)__double_as_longlong(x);
    const int ex = (int)(ux >> 52);  // the sign bit included: >= 2048 for a negative x
    const int E = ex - 1023, p = E & 1, q = (E - p) / 2;
    const uint32_t fx = ((uint32_t)(127 + p) << 23) | ((uint32_t)(ux >> 29) & 0x7fffffu);
    float sf, rf;
    asm("sqrt.rn.f32 %0, %1;" : "=f"(sf) : "f"(__uint_as_float(fx)));
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rf) : "f"(sf));
    const uint32_t us = __float_as_uint(sf), ur = __float_as_uint(rf);
    const double s0 = __longlong_as_double((long long)(((unsigned long long)((int)((us >> 23) & 0xffu) + 896 + q) << 52) |
                                                       ((unsigned long long)(us & 0x7fffffu) << 29)));
    const double h0 = __longlong_as_double((long long)(((unsigned long long)((int)((ur >> 23) & 0xffu) + 895 - q) << 52) |
                                                       ((unsigned long long)(ur & 0x7fffffu) << 29)));
    const double s1 = __fma_rn(__fma_rn(-s0, s0, x), h0, s0);
    const unsigned long long us1 = (unsigned long long)__double_as_longlong(s1);
    const int es = (int)((us1 >> 52) & 0x7ff);
    const int t = ex - 2 * es + 1075;
    const unsigned long long fs = us1 & FRAC;
    const bool fast = ex >= 1 && ex <= 2046 && (t == 52 || t == 53) && fs - 1024 < FRAC - 2047;  // 1024 <= fs <= 2^52 - 1025
    const unsigned long long mx = (ux & FRAC) | ONE, ms = fs | ONE;
    const unsigned long long Ru = (mx << (t & 63)) - ms * ms;  // X - ms^2 (unsigned: wraps off the fast path)
    unsigned long long k = (unsigned long long)(long long)__float2int_rn(
        __fdividef((float)(int)((long long)Ru >> 40), (float)(int)(ms >> 39)));
#pragma unroll
    for (int it = 0; it < 2; ++it) {
        const unsigned long long c = ms + k;
        const long long D = (long long)(Ru - 2 * ms * k - k * k);  // X - c^2
        k += (unsigned long long)((long long)(D > (long long)c) - (long long)(D <= -(long long)c));
    }
    double r = __longlong_as_double((long long)(us1 + k));
    if ((ux << 1) == 0) r = x;  // sqrt(+-0) = +-0
    else if (!fast) r = sqrt_fp64_call(x);
    return r;
}

// RN(1 / d) for div_by_recip where d is in [2^-1000, 2^1000]; else 0, the mark that makes
// div_by_recip divide
__device__ __forceinline__ double recip_for(double d) {
    const int ed = (int)((__double_as_longlong(d) >> 52) & 0x7ff);
    return (ed >= 23 && ed <= 2023) ? div_ip(1.0, d) : 0.0;
}

// ------------------------------------------------------------------ addition on the integer pipe
// a + b, IEEE binary64 round to nearest even, bit for bit the FP64 pipe's sum.  On GB300 the
// FP64 pipe issues a warp instruction about every 76 cycles of a sub-partition while the integer
// ALU issues one every two: a chain of products and sums (x = x + c q) that keeps the multiply on
// the FP64 pipe and moves the sum here runs well above the rate of both on the FP64 pipe.
//
// The integer path takes the operand of the larger exponent, x, normal and below the top binade,
// and y a zero (of either sign), or a normal or subnormal number of x's sign -- the sums of
// like-signed terms -- and two zeros.  y's significand (53 bits; a subnormal's without the
// implicit bit, at the exponent of the smallest normal) is shifted right by the exponents'
// difference d (63 at most: further down it only sets the sticky bit, as at 63) across three
// 32-bit words, the third a guard word, with the bits that fall below it kept as a sticky bit;
// the two significands are added, the sum put back in [2^52, 2^53) by at most one right shift
// (its bit kept as sticky), and rounded to nearest even on the guard word: up when it exceeds
// half, or is half and the last kept bit is odd.  A carry out of the rounding lands in the
// exponent field, which is the representation of the rounded value (the largest finite x
// rounding up gives infinity, as the FP64 pipe's overflow does).  A zero y adds nothing: the sum
// is x.  Two zeros sum to -0 when both are -0, else +0.  Everything else -- signs that differ on
// non-zero operands, a subnormal, infinite or NaN x, x in the top binade -- is the FP64 pipe's,
// through a call: a fallback inlined beside the integer path is issued on every call, its lanes
// predicated off, and a predicated-off FP64 instruction holds the FP64 pipe as long as a live one.
static __device__ __noinline__ double add_fp64_pipe(double a, double b) { return a + b; }
__device__ __forceinline__ double add_ip(double a, double b) {
    const uint32_t ha = (uint32_t)__double2hiint(a), la = (uint32_t)__double2loint(a);
    const uint32_t hb = (uint32_t)__double2hiint(b), lb = (uint32_t)__double2loint(b);
    const uint32_t fa = ha & 0x7ff00000u, fb = hb & 0x7ff00000u;  // the exponent fields
    const bool sw = fa < fb;
    const uint32_t hx = sw ? hb : ha, lx = sw ? lb : la, hy = sw ? ha : hb, ly = sw ? la : lb;
    const uint32_t fx = sw ? fb : fa, fy = sw ? fa : fb;
    const bool yz = ((hy << 1) | ly) == 0, bz = yz && ((hx << 1) | lx) == 0;
    const bool fast = (fx - 0x00100000u < 0x7fd00000u && (yz || ((ha ^ hb) >> 31) == 0)) || bz;
    const uint32_t d = min((fx - max(fy, 0x00100000u)) >> 20, 63u), s = d & 31;
    const uint32_t mxh = (hx & 0xfffffu) | 0x100000u, myh = (hy & 0xfffffu) | (fy != 0 ? 0x100000u : 0u);
    // y >> d over (yh, yl, g): the words (myh, ly, 0), or (0, myh, ly) for d >= 32, shifted by d mod 32
    const bool big = d >= 32;
    const uint32_t w2 = big ? 0u : myh, w1 = big ? myh : ly, w0 = big ? ly : 0u;
    const uint32_t yh = w2 >> s, yl = __funnelshift_r(w1, w2, s);
    uint32_t g = __funnelshift_r(w0, w1, s) | (uint32_t)(__funnelshift_r(0u, w0, s) != 0u);
    const uint64_t S = (((uint64_t)mxh << 32) | lx) + (((uint64_t)yh << 32) | yl);
    uint32_t sh = (uint32_t)(S >> 32), sl = (uint32_t)S;
    const uint32_t c = sh >> 21;  // 1 where the sum reached 2^53
    g = __funnelshift_r(g, sl, c) | (g & c);
    sl = __funnelshift_r(sl, sh, c);
    sh >>= c;
    const uint32_t up = (g | (sl & 1u)) > 0x80000000u;
    const uint64_t M = (((uint64_t)sh << 32) | sl) + up;
    const uint32_t hr = (hx & 0xfff00000u) + (c << 20) - 0x100000u + (uint32_t)(M >> 32);
    double r = __hiloint2double((int)(bz ? ha & hb : hr), bz ? 0 : (int)(uint32_t)M);
    if (!fast) r = add_fp64_pipe(a, b);
    return r;
}
// a - b as a + (-b): the same bits (IEEE subtraction is addition of the negated operand)
__device__ __forceinline__ double sub_ip(double a, double b) {
    return add_ip(a, __longlong_as_double(__double_as_longlong(b) ^ (long long)0x8000000000000000ULL));
}
// +0.0 + p and +0.0 - p, the first term of a sum or a difference that starts from +0: p (or -p)
// itself, +0 where p is a zero of either sign, the FP64 pipe's own result for a NaN
__device__ __forceinline__ double zero_plus(double p) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(p);
    if ((b << 1) == 0) return 0.0;
    if ((b << 1) > 0xffe0000000000000ULL) return add_fp64_pipe(0.0, p);
    return p;
}
__device__ __forceinline__ double zero_minus(double p) { return zero_plus(gb_neg(p)); }

// ------------------------------------------------------------------ 0/1 flags (Calc_Kzz's jqif)
// jqif(x, y) = nint(0.5 + sign(0.5, x - y)) (1 where x - y has a clear sign bit) on the integer
// pipe, for the Kzz column sweep's serial chain (where the subtraction's latency is on the
// path): for finite x and y the sign of x - y is their order (x - x = +0; an
// overflowing difference keeps its sign), but for two zeros, where only -0 - +0 = -0 has it set.
// An infinite or NaN operand takes the subtraction itself.  (Where the FP64 pipe's throughput,
// not its latency, is the bound, the plain subtraction measured better.)
static __device__ __noinline__ double jqif_fp64(double x, double y) { return signbit(x - y) ? 0.0 : 1.0; }
__device__ __forceinline__ double jqif_ip(double x, double y) {
    const unsigned long long bx = (unsigned long long)__double_as_longlong(x), by = (unsigned long long)__double_as_longlong(y);
    if (((bx >> 52) & 0x7ff) == 0x7ff || ((by >> 52) & 0x7ff) == 0x7ff) return jqif_fp64(x, y);
    if (((bx | by) << 1) == 0) return (bx >> 63) && !(by >> 63) ? 0.0 : 1.0;  // two zeros
    return gb_ge(x, y) ? 1.0 : 0.0;
}

// Calc_Kzz's statements blend by flags that are exactly +0.0 or 1.0 (jqif's values, their
// products and complements), so the flag arithmetic runs on the integer pipe:
//   jq a jq' and jq (1 - jq')  ->  the flags' AND (+0.0 or 1.0, as the products are);
//   jq x + (1 - jq) y          ->  x or y, for finite x and y, with the zero the other product
//                                  adds: x + (+0 y) is x but for x = -0 beside a y of clear sign
//                                  (-0 + +0 = +0), and (+0 x) + y the same way round;
//   jq v                       ->  v, or the zero of v's sign, for finite v.
// A non-finite operand takes the FP64 statement itself, through a call.
__device__ __forceinline__ bool on(double f) { return __double_as_longlong(f) != 0; }  // 1.0, not +0.0
__device__ __forceinline__ double flag(bool b) { return b ? 1.0 : 0.0; }
__device__ __forceinline__ bool finite_bits(unsigned long long b) { return ((b >> 52) & 0x7ff) != 0x7ff; }
static __device__ __noinline__ double blend_fp64(double jq, double x, double y) { return jq * x + (1.0 - jq) * y; }
__device__ __forceinline__ double blend01(double jq, double x, double y) {
    const unsigned long long bx = (unsigned long long)__double_as_longlong(x), by = (unsigned long long)__double_as_longlong(y);
    constexpr unsigned long long SIGN = 0x8000000000000000ULL;
    if (!finite_bits(bx) || !finite_bits(by)) return blend_fp64(jq, x, y);
    const unsigned long long r = on(jq) ? ((bx == SIGN && (by >> 63) == 0) ? 0ULL : bx)
                                        : ((by == SIGN && (bx >> 63) == 0) ? 0ULL : by);
    return __longlong_as_double((long long)r);
}
static __device__ __noinline__ double mul_fp64(double a, double b) { return a * b; }
__device__ __forceinline__ double mul01(double jq, double v) {
    const unsigned long long bv = (unsigned long long)__double_as_longlong(v);
    if (!finite_bits(bv)) return mul_fp64(jq, v);
    return __longlong_as_double((long long)(on(jq) ? bv : (bv & 0x8000000000000000ULL)));
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
    return s + div_ip(num, m_new);
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
    for (int n = 2; n <= nloop; ++n) f = div_ip(f * (double)(n - 1), (double)n);
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
