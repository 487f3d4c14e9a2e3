// The replay's comparison of a device array with a dump's, made where the state is: only the
// report comes back to the host.
//
// Over two float64 views of one shape (rank <= 4; any strides, so the dump's array can stay in
// its file's Fortran order): the elements whose bit patterns differ, and over the whole array
// the reductions of the reference's report -- the number of differing elements; the largest ulp
// distance, |o(a) - o(b)| with o the sign-magnitude image (o(x) = x's bits as int64 where
// non-negative, INT64_MIN - bits where negative; the subtraction and the magnitude wrap as int64
// arithmetic does); the largest |a - b|; the largest |a - b| / max(|a|, |b|) over the differing
// elements (0 elsewhere); and the first differing element in row-major order.  The maxima of
// |a - b| and of the ratio propagate NaN as NumPy's max and maximum do: both are non-negative or
// a NaN with a clear sign bit, whose bit patterns order as the values do with the NaN above
// +inf, so they are reduced as unsigned bit patterns.
//
// Reference: pydyn harness.py:140-179 (_ulp_distance, bits, compare), replay.py:277-289.
#include <climits>

#include "gb_common.cuh"

namespace {

struct CmpOut {
    unsigned long long n_diff;
    long long max_ulp;
    unsigned long long max_abs;  // bit pattern
    unsigned long long max_rel;  // bit pattern
    long long first;             // row-major index, LLONG_MAX when none differs
};

__device__ __forceinline__ long long ordered(long long i) {
    return i < 0 ? (long long)((unsigned long long)LLONG_MIN - (unsigned long long)i) : i;
}
__device__ __forceinline__ double np_maximum(double a, double b) {  // NumPy maximum: NaN wins
    return (gb_isnan(a) || gb_isnan(b)) ? __longlong_as_double(0x7ff8000000000000LL) : (a >= b ? a : b);
}

__global__ void k_cmp_init(CmpOut *o) {
    o->n_diff = 0;
    o->max_ulp = LLONG_MIN;
    o->max_abs = 0;  // +0.0
    o->max_rel = 0;
    o->first = LLONG_MAX;
}

__global__ void k_compare(DV a, DV b, int64_t total, CmpOut *o) {
    unsigned long long nd = 0, mabs = 0, mrel = 0;
    long long mulp = LLONG_MIN, first = LLONG_MAX;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < total; k += stride) {
        int64_t r = k;
        const int64_t i3 = r % a.n3;
        r /= a.n3;
        const int64_t i2 = r % a.n2;
        r /= a.n2;
        const int64_t i1 = r % a.n1;
        const int64_t i0 = r / a.n1;
        const double x = a.p[i0 * a.s0 + i1 * a.s1 + i2 * a.s2 + i3 * a.s3];
        const double y = b.p[i0 * b.s0 + i1 * b.s1 + i2 * b.s2 + i3 * b.s3];
        const long long bx = __double_as_longlong(x), by = __double_as_longlong(y);
        const bool differ = bx != by;
        const long long d = (long long)((unsigned long long)ordered(bx) - (unsigned long long)ordered(by));
        const long long ulp = d < 0 ? (long long)(0ULL - (unsigned long long)d) : d;
        mulp = ulp > mulp ? ulp : mulp;
        const double diff = fabs(x - y);
        const unsigned long long db = (unsigned long long)__double_as_longlong(diff);
        mabs = db > mabs ? db : mabs;
        if (differ) {
            ++nd;
            const double rel = diff / np_maximum(fabs(x), fabs(y));
            const unsigned long long rb = (unsigned long long)__double_as_longlong(rel);
            mrel = rb > mrel ? rb : mrel;
            first = k < first ? k : first;
        }
    }
    for (int s = 16; s > 0; s >>= 1) {
        nd += __shfl_xor_sync(FULL_MASK, nd, s);
        const long long u = __shfl_xor_sync(FULL_MASK, mulp, s);
        mulp = u > mulp ? u : mulp;
        const unsigned long long ab = __shfl_xor_sync(FULL_MASK, mabs, s);
        mabs = ab > mabs ? ab : mabs;
        const unsigned long long rb = __shfl_xor_sync(FULL_MASK, mrel, s);
        mrel = rb > mrel ? rb : mrel;
        const long long f = __shfl_xor_sync(FULL_MASK, first, s);
        first = f < first ? f : first;
    }
    if ((threadIdx.x & 31) == 0) {
        if (nd) atomicAdd(&o->n_diff, nd);
        atomicMax(&o->max_ulp, mulp);
        atomicMax(&o->max_abs, mabs);
        atomicMax(&o->max_rel, mrel);
        if (first != LLONG_MAX) atomicMin(&o->first, first);
    }
}

}  // namespace

// The report of a against b (same extents) into out, a device buffer of 5 int64: n_diff, max_ulp,
// the bits of max_abs and of max_rel, and the first differing row-major index (INT64_MAX: none).
extern "C" int gb_compare(gb_ctx *ctx, const gb_view *a, const gb_view *b, long long *out) {
    if (!ctx || !a || !b || !out) return GB_EARG;
    for (int k = 0; k < 4; ++k)
        if (a->n[k] != b->n[k]) {
            gb_set_error("gb_compare: the two views differ in extent");
            return GB_EARG;
        }
    const DV va = dv(a), vb = dv(b);
    const int64_t total = va.n0 * va.n1 * va.n2 * va.n3;
    CmpOut *o = reinterpret_cast<CmpOut *>(out);
    k_cmp_init<<<1, 1, 0, ctx->stream>>>(o);
    if (int rc = gb_after_launch(ctx, "cmp_init")) return rc;
    if (total <= 0) return GB_OK;
    int64_t blocks = (total + 255) / 256;
    const int64_t cap = (int64_t)ctx->sms * 8;
    if (blocks > cap) blocks = cap;
    k_compare<<<(int)blocks, 256, 0, ctx->stream>>>(va, vb, total, o);
    return gb_after_launch(ctx, "compare");
}
