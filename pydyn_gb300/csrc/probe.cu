// FP64 issue-rate probe: the compute ceiling of the dynamic step.
//
// The step is float64 arithmetic compiled without contraction, so its pipe is the FP64 unit, not
// the tensor cores or HBM.  These kernels measure that unit's rate on the GPU they run on: each
// thread runs independent chains (enough of them to cover the pipe's latency) of one instruction
// kind and writes one value, so the kernel touches no memory but its output.  Timed with CUDA
// events on the context's stream.
#include "gb_common.cuh"

namespace {

constexpr int PROBE_BLOCKS_PER_SM = 8;
constexpr int PROBE_THREADS = 256;

// 8 chains of a multiply then an add (the pair -fmad=false emits for x * a + b): 16 instructions
__global__ void k_probe_muladd(double *out, int iters, double a, double b) {
    int tid = blockIdx.x * blockDim.x + threadIdx.x;
    double x[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) x[c] = tid * 1e-9 + c;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < 8; ++c) x[c] = x[c] * a;
#pragma unroll
        for (int c = 0; c < 8; ++c) x[c] = x[c] + b;
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < 8; ++c) s = s + x[c];
    out[tid] = s;
}

// 8 chains of a fused multiply-add: 8 instructions, 16 flops
__global__ void k_probe_fma(double *out, int iters, double a, double b) {
    int tid = blockIdx.x * blockDim.x + threadIdx.x;
    double x[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) x[c] = tid * 1e-9 + c;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < 8; ++c) x[c] = fma(x[c], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < 8; ++c) s = s + x[c];
    out[tid] = s;
}

// 4 chains of a correctly rounded division
__global__ void k_probe_div(double *out, int iters, double a) {
    int tid = blockIdx.x * blockDim.x + threadIdx.x;
    double x[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) x[c] = 1.0 + tid * 1e-9 + c;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < 4; ++c) x[c] = a / x[c];
    }
    out[tid] = ((x[0] + x[1]) + x[2]) + x[3];
}

// 8 chains of a multiply on the FP64 pipe and an add on the integer pipe (add_ip): the pair
// counted as two instructions, as kind 0 counts it
__global__ void k_probe_muladd_ip(double *out, int iters, double a, double b) {
    int tid = blockIdx.x * blockDim.x + threadIdx.x;
    double x[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) x[c] = tid * 1e-9 + c + 1.0;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < 8; ++c) x[c] = add_ip(x[c] * a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < 8; ++c) s = s + x[c];
    out[tid] = s;
}

// 4 chains of the integer-corrected division (div_ip)
__global__ void k_probe_div_ip(double *out, int iters, double a) {
    int tid = blockIdx.x * blockDim.x + threadIdx.x;
    double x[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) x[c] = 1.0 + tid * 1e-9 + c;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < 4; ++c) x[c] = div_ip(a, x[c]);
    }
    out[tid] = ((x[0] + x[1]) + x[2]) + x[3];
}

}  // namespace

// kind 0: DMUL + DADD, 1: DFMA, 2: DDIV, 3: DMUL + add_ip (counted as two instructions, as kind 0),
// 4: div_ip.  *rate = instructions (kinds 2 and 4: divisions) per second over the whole GPU.
extern "C" int gb_fp64_rate(gb_ctx *ctx, int kind, double *rate) {
    if (!ctx || !rate || kind < 0 || kind > 4) return GB_EARG;
    if (ctx->capturing) {
        gb_set_error("fp64_rate: cannot be captured");
        return GB_EARG;
    }
    int sms = 0;
    GB_CHECK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
    const int blocks = sms * PROBE_BLOCKS_PER_SM;
    const int64_t threads = (int64_t)blocks * PROBE_THREADS;
    double *out = gb_work(ctx, threads * sizeof(double));
    if (!out) return GB_ECUDA;
    const int iters = (kind == 2 || kind == 4) ? 200 : 2000;
    const double per_iter = (kind == 0 || kind == 3) ? 16.0 : kind == 1 ? 8.0 : 4.0;
    cudaEvent_t e0, e1;
    GB_CHECK_CUDA(cudaEventCreate(&e0));
    GB_CHECK_CUDA(cudaEventCreate(&e1));
    float best = 0.0f;
    int rc = GB_OK;
    for (int rep = 0; rep < 3 && rc == GB_OK; ++rep) {  // the first launch warms up; keep the fastest
        cudaEventRecord(e0, ctx->stream);
        if (kind == 0)
            k_probe_muladd<<<blocks, PROBE_THREADS, 0, ctx->stream>>>(out, iters, 0.999999, 1e-7);
        else if (kind == 1)
            k_probe_fma<<<blocks, PROBE_THREADS, 0, ctx->stream>>>(out, iters, 0.999999, 1e-7);
        else if (kind == 2)
            k_probe_div<<<blocks, PROBE_THREADS, 0, ctx->stream>>>(out, iters, 1.000001);
        else if (kind == 3)
            k_probe_muladd_ip<<<blocks, PROBE_THREADS, 0, ctx->stream>>>(out, iters, 0.999999, 1e-7);
        else
            k_probe_div_ip<<<blocks, PROBE_THREADS, 0, ctx->stream>>>(out, iters, 1.000001);
        rc = gb_after_launch(ctx, "fp64_rate");
        cudaEventRecord(e1, ctx->stream);
        cudaError_t e = cudaEventSynchronize(e1);
        if (e != cudaSuccess) rc = gb_cuda_fail(e, "fp64_rate sync");
        float ms = 0.0f;
        if (rc == GB_OK && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess && rep > 0)
            best = (best == 0.0f || ms < best) ? ms : best;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != GB_OK) return rc;
    *rate = best > 0.0f ? (double)threads * iters * per_iter / (best * 1e-3) : 0.0;
    return GB_OK;
}
