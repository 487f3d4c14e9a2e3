// The context of the C ABI: device memory, the one stream, the device status word, CUDA graph
// capture and the generic box statements (strided elementwise statements and ordered sums) that
// carry the zoom exchange.
#include "gb_common.cuh"

#include <mutex>
#include <new>

static thread_local std::string g_last_error;

void gb_set_error(const std::string &msg) { g_last_error = msg; }

int gb_cuda_fail(cudaError_t e, const char *what) {
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return GB_ECUDA;
}

int gb_after_launch(gb_ctx *ctx, const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return gb_cuda_fail(e, what);
    ctx->launches += 1;
    if (ctx->capturing) ctx->capture_launches += 1;
    return GB_OK;
}

int32_t *gb_scratch_i(gb_ctx *ctx, size_t n) {
    if (n <= ctx->scratch_i_n) return ctx->scratch_i;
    return nullptr;  // grown only outside capture, by gb_create's fixed size
}

double *gb_work(gb_ctx *ctx, size_t bytes) {
    if (bytes <= ctx->work_bytes) return ctx->work;
    if (ctx->capturing) {  // an allocation would end the capture: the first uncaptured call sizes it
        gb_set_error("work space of " + std::to_string(bytes) + " bytes needed inside a capture; run the "
                     "operator once before capturing");
        return nullptr;
    }
    cudaError_t e = cudaStreamSynchronize(ctx->stream);  // the old space may still be read
    if (e == cudaSuccess && ctx->work) e = cudaFree(ctx->work);
    ctx->work = nullptr;
    ctx->work_bytes = 0;
    if (e == cudaSuccess) e = cudaMalloc(&ctx->work, bytes);
    if (e != cudaSuccess) {
        gb_cuda_fail(e, "gb_work");
        ctx->work = nullptr;
        return nullptr;
    }
    ctx->work_bytes = bytes;
    return ctx->work;
}

extern "C" const char *gb_last_error(void) { return g_last_error.c_str(); }

extern "C" int gb_create(int device, gb_ctx **out) {
    if (!out) return GB_EARG;
    GB_CHECK_CUDA(cudaSetDevice(device));
    gb_ctx *ctx = new (std::nothrow) gb_ctx();
    if (!ctx) return GB_EARG;
    ctx->device = device;
    cudaError_t e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->join, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->ctl, sizeof(gb_ctl));
    if (e == cudaSuccess) e = cudaMemset(ctx->ctl, 0, sizeof(gb_ctl));
    ctx->scratch_i_n = 1 << 16;
    if (e == cudaSuccess) e = cudaMalloc(&ctx->scratch_i, ctx->scratch_i_n * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMemset(ctx->scratch_i, 0, ctx->scratch_i_n * sizeof(int32_t));
    if (e != cudaSuccess) {
        delete ctx;
        return gb_cuda_fail(e, "gb_create");
    }
    *out = ctx;
    return GB_OK;
}

extern "C" int gb_stream_priority(gb_ctx *ctx, int rank) {
    if (!ctx || rank < 0) return GB_EARG;
    if (ctx->capturing) {
        gb_set_error("gb_stream_priority: not while capturing");
        return GB_EARG;
    }
    int least = 0, greatest = 0;
    GB_CHECK_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    const int prio = least - rank < greatest ? greatest : least - rank;  // numerically lower: served first
    // new streams at that priority, once the old ones have drained (work enqueued later goes to them)
    cudaStream_t s = nullptr, side = nullptr;
    GB_CHECK_CUDA(cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, prio));
    cudaError_t e = cudaStreamCreateWithPriority(&side, cudaStreamNonBlocking, prio);
    if (e != cudaSuccess) {
        cudaStreamDestroy(s);
        return gb_cuda_fail(e, "gb_stream_priority");
    }
    GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
    GB_CHECK_CUDA(cudaStreamSynchronize(ctx->side));
    cudaStreamDestroy(ctx->stream);
    cudaStreamDestroy(ctx->side);
    ctx->stream = s;
    ctx->side = side;
    return GB_OK;
}

extern "C" int gb_work_reserve(gb_ctx *ctx, size_t bytes) {
    if (!ctx) return GB_EARG;
    return gb_work(ctx, bytes) ? GB_OK : GB_ECUDA;
}

extern "C" size_t gb_work_size(gb_ctx *ctx) { return ctx ? ctx->work_bytes : 0; }

extern "C" int gb_scratch_info(gb_ctx *ctx, int32_t **ptr, size_t *n) {
    if (!ctx || !ptr || !n) return GB_EARG;
    *ptr = ctx->scratch_i;
    *n = ctx->scratch_i_n;
    return GB_OK;
}

extern "C" int gb_device_name(gb_ctx *ctx, char *buf, int len) {
    if (!ctx || !buf || len <= 0) return GB_EARG;
    cudaDeviceProp prop;
    GB_CHECK_CUDA(cudaGetDeviceProperties(&prop, ctx->device));
    snprintf(buf, (size_t)len, "%s sm_%d%d x%d", prop.name, prop.major, prop.minor, prop.multiProcessorCount);
    return GB_OK;
}

extern "C" int gb_tune_set(gb_ctx *ctx, int key, int value) {
    if (!ctx || key < 0 || key >= GB_TUNE_N) return GB_EARG;
    const bool pow2 = value > 0 && (value & (value - 1)) == 0;
    bool ok = false;
    switch (key) {
        case GB_TUNE_COLUMN_THREADS: ok = pow2 && value >= 32 && value <= GB_TUNE_MAX_COLUMN; break;
        case GB_TUNE_CELL_THREADS: ok = pow2 && value >= 32 && value <= GB_TUNE_MAX_CELL; break;
        case GB_TUNE_LU_WARPS: ok = pow2 && value <= GB_TUNE_MAX_LU_WARPS; break;
        case GB_TUNE_APPLY_THREADS: ok = value == 0 || (value >= 32 && value <= 1024); break;
        case GB_TUNE_LU_LANES: ok = value == 8 || value == 16 || value == 32; break;
    }
    if (!ok) {
        gb_set_error("gb_tune_set: value " + std::to_string(value) + " outside the range of key " + std::to_string(key));
        return GB_EARG;
    }
    ctx->tune[key] = value;
    return GB_OK;
}

extern "C" int gb_tune_get(gb_ctx *ctx, int key, int *value) {
    if (!ctx || !value || key < 0 || key >= GB_TUNE_N) return GB_EARG;
    *value = ctx->tune[key];
    return GB_OK;
}

extern "C" void gb_destroy(gb_ctx *ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->ctl) cudaFree(ctx->ctl);
    if (ctx->scratch_i) cudaFree(ctx->scratch_i);
    if (ctx->work) cudaFree(ctx->work);
    if (ctx->side) cudaStreamSynchronize(ctx->side);
    if (ctx->fork) cudaEventDestroy(ctx->fork);
    if (ctx->join) cudaEventDestroy(ctx->join);
    if (ctx->side) cudaStreamDestroy(ctx->side);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

extern "C" int gb_alloc(gb_ctx *ctx, size_t bytes, void **dptr) {
    if (!ctx || !dptr) return GB_EARG;
    GB_CHECK_CUDA(cudaMalloc(dptr, bytes ? bytes : 8));
    GB_CHECK_CUDA(cudaMemset(*dptr, 0, bytes ? bytes : 8));
    return GB_OK;
}

extern "C" int gb_free(gb_ctx *ctx, void *dptr) {
    (void)ctx;
    GB_CHECK_CUDA(cudaFree(dptr));
    return GB_OK;
}

extern "C" int gb_put(gb_ctx *ctx, void *dst, const void *src, size_t bytes) {
    GB_CHECK_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
    return GB_OK;
}

extern "C" int gb_get(gb_ctx *ctx, void *dst, const void *src, size_t bytes) {
    GB_CHECK_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
    return GB_OK;
}

extern "C" int gb_get_async(gb_ctx *ctx, void *dst, const void *src, size_t bytes) {
    GB_CHECK_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    return GB_OK;
}

extern "C" int gb_copy_d2d(gb_ctx *ctx, void *dst, const void *src, size_t bytes) {
    GB_CHECK_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    return GB_OK;
}

extern "C" int gb_stream_sync(gb_ctx *ctx) {
    GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
    return GB_OK;
}

extern "C" int gb_host_alloc(size_t bytes, void **hptr) {
    GB_CHECK_CUDA(cudaMallocHost(hptr, bytes ? bytes : 8));
    return GB_OK;
}

extern "C" int gb_host_free(void *hptr) {
    GB_CHECK_CUDA(cudaFreeHost(hptr));
    return GB_OK;
}

extern "C" int gb_status_peek(gb_ctx *ctx, int *word) {
    int w = 0;
    GB_CHECK_CUDA(cudaMemcpyAsync(&w, &ctx->ctl->status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
    *word = w;
    return GB_OK;
}

extern "C" int gb_sync(gb_ctx *ctx) {
    int w = 0;
    GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
    GB_CHECK_CUDA(cudaMemcpy(&w, &ctx->ctl->status, sizeof(int), cudaMemcpyDeviceToHost));
    if (w) {
        int zero = 0;
        GB_CHECK_CUDA(cudaMemcpy(&ctx->ctl->status, &zero, sizeof(int), cudaMemcpyHostToDevice));
        std::string msg;
        if (w & GB_ECFL) msg += "sub-cycle cap reached (CFL); ";
        if (w & GB_EHALO) msg += "non-zero boundary faces; ";
        if (w & GB_ELEVELS) msg += "levels not strictly descending; ";
        if (w & GB_ESEARCH) msg += "sub-cycle search did not settle; ";
        if (w & GB_ETIMEOUT) msg += "device wait timed out; ";
        gb_set_error(msg);
    }
    return w;
}

extern "C" int64_t gb_launches(gb_ctx *ctx) { return ctx->launches; }

extern "C" void *gb_stream(gb_ctx *ctx) { return (void *)ctx->stream; }

// ------------------------------------------------------------------ graphs
struct gb_graph {
    cudaGraph_t graph;
    cudaGraphExec_t exec;
    int64_t launches;
};

extern "C" int gb_capture_begin(gb_ctx *ctx) {
    GB_CHECK_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    ctx->capturing = true;
    ctx->capture_launches = 0;
    return GB_OK;
}

extern "C" int gb_capture_end(gb_ctx *ctx, void **out) {
    gb_graph *g = new gb_graph();
    ctx->capturing = false;
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &g->graph);
    if (e != cudaSuccess) {
        delete g;
        return gb_cuda_fail(e, "cudaStreamEndCapture");
    }
    // each kernel node runs at the priority of the stream it was captured on (gb_stream_priority)
    e = cudaGraphInstantiate(&g->exec, g->graph, cudaGraphInstantiateFlagUseNodePriority);
    if (e != cudaSuccess) {
        cudaGraphDestroy(g->graph);
        delete g;
        return gb_cuda_fail(e, "cudaGraphInstantiate");
    }
    g->launches = ctx->capture_launches;
    ctx->launches -= ctx->capture_launches;  // counted when replayed
    *out = g;
    return GB_OK;
}

extern "C" int gb_graph_launch(gb_ctx *ctx, void *graph) {
    gb_graph *g = (gb_graph *)graph;
    GB_CHECK_CUDA(cudaGraphLaunch(g->exec, ctx->stream));
    ctx->launches += g->launches;
    return GB_OK;
}

extern "C" int gb_graph_destroy(void *graph) {
    gb_graph *g = (gb_graph *)graph;
    if (!g) return GB_OK;
    cudaGraphExecDestroy(g->exec);
    cudaGraphDestroy(g->graph);
    delete g;
    return GB_OK;
}

// ------------------------------------------------------------------ events
extern "C" int gb_event_create(void **ev) {
    cudaEvent_t e;
    GB_CHECK_CUDA(cudaEventCreate(&e));
    *ev = (void *)e;
    return GB_OK;
}
extern "C" int gb_event_record(gb_ctx *ctx, void *ev) {
    GB_CHECK_CUDA(cudaEventRecord((cudaEvent_t)ev, ctx->stream));
    return GB_OK;
}
extern "C" int gb_stream_wait(gb_ctx *ctx, void *ev) {
    if (!ctx || !ev) return GB_EARG;
    GB_CHECK_CUDA(cudaStreamWaitEvent(ctx->stream, (cudaEvent_t)ev, 0));
    return GB_OK;
}
extern "C" int gb_event_elapsed_ms(void *start, void *stop, float *ms) {
    GB_CHECK_CUDA(cudaEventSynchronize((cudaEvent_t)stop));
    GB_CHECK_CUDA(cudaEventElapsedTime(ms, (cudaEvent_t)start, (cudaEvent_t)stop));
    return GB_OK;
}
extern "C" int gb_event_sync(void *ev) {
    if (!ev) return GB_EARG;
    GB_CHECK_CUDA(cudaEventSynchronize((cudaEvent_t)ev));
    return GB_OK;
}
extern "C" int gb_event_destroy(void *ev) {
    GB_CHECK_CUDA(cudaEventDestroy((cudaEvent_t)ev));
    return GB_OK;
}

// ------------------------------------------------------------------ Check_CFL flag
__global__ void k_cfl_reset(gb_ctl *ctl) { ctl->cfl_failed = 0; }

extern "C" int gb_cfl_reset(gb_ctx *ctx) {
    k_cfl_reset<<<1, 1, 0, ctx->stream>>>(ctx->ctl);
    return gb_after_launch(ctx, "cfl_reset");
}

extern "C" int gb_cfl_failed(gb_ctx *ctx, int *failed) {
    int w = 0;
    GB_CHECK_CUDA(cudaMemcpyAsync(&w, &ctx->ctl->cfl_failed, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    GB_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
    *failed = w;
    return GB_OK;
}

// ------------------------------------------------------------------ box statements
__device__ __forceinline__ int64_t off4(const DV &v, int64_t i0, int64_t i1, int64_t i2, int64_t i3) {
    return i0 * v.s0 + i1 * v.s1 + i2 * v.s2 + i3 * v.s3;
}

// IDX: the flat index type -- 32-bit whenever the box has fewer than 2^31 elements, so that its
// decomposition into (i0, i1, i2, i3) takes three 32-bit divisions, not 64-bit ones
template <typename IDX>
__global__ void k_box(int op, DV d, DV a, DV b, double x, double y, IDX total) {
    IDX k = (IDX)(blockIdx.x * (int64_t)blockDim.x + threadIdx.x);
    const IDX stride = (IDX)((int64_t)gridDim.x * blockDim.x);
    const IDX n1 = (IDX)d.n1, n2 = (IDX)d.n2, n3 = (IDX)d.n3;
    for (; k < total; k += stride) {
        IDX r = k;
        const IDX i3 = r % n3; r /= n3;
        const IDX i2 = r % n2; r /= n2;
        const IDX i1 = r % n1; r /= n1;
        const IDX i0 = r;
        double va = (op != 3) ? a.p[off4(a, i0, i1, i2, i3)] : 0.0;
        double vb = (op >= 4 && op <= 7) || op == 9 ? b.p[off4(b, i0, i1, i2, i3)] : 0.0;
        double out;
        switch (op) {
            case 0: out = va; break;
            case 1: out = va * x; break;
            case 2: out = va / x; break;
            case 3: out = x; break;
            case 4: out = va + vb; break;
            case 5: out = va - vb; break;
            case 6: out = va * vb; break;
            case 7: out = va / vb; break;
            case 8: out = (va * x) / y; break;
            case 9: out = x * va + y * vb; break;
            case 10: out = x * va; break;
            default: out = va; break;
        }
        d.p[off4(d, i0, i1, i2, i3)] = out;
    }
}

static int launch_grid(int64_t total) {
    int64_t blocks = (total + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    if (blocks < 1) blocks = 1;
    return (int)blocks;
}

extern "C" int gb_box(gb_ctx *ctx, int op, const gb_view *dst, const gb_view *a, const gb_view *b,
                      double x, double y) {
    if (!dst) return GB_EARG;
    DV d = dv(dst);
    DV va = a ? dv(a) : d;
    DV vb = b ? dv(b) : d;
    int64_t total = d.n0 * d.n1 * d.n2 * d.n3;
    if (total <= 0) return GB_OK;
    if (total < (int64_t)1 << 31)
        k_box<uint32_t><<<launch_grid(total), 256, 0, ctx->stream>>>(op, d, va, vb, x, y, (uint32_t)total);
    else
        k_box<int64_t><<<launch_grid(total), 256, 0, ctx->stream>>>(op, d, va, vb, x, y, total);
    return gb_after_launch(ctx, "box");
}

// dst = w[0] a + w[1] b with the weights read from device memory (balance.time_interpolation)
__global__ void k_interp(DV d, DV a, DV b, const double *w, int64_t total) {
    int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const double w1 = w[0], w2 = w[1];
    for (; k < total; k += stride) {
        int64_t r = k;
        int64_t i3 = r % d.n3; r /= d.n3;
        int64_t i2 = r % d.n2; r /= d.n2;
        int64_t i1 = r % d.n1; r /= d.n1;
        int64_t i0 = r;
        d.p[off4(d, i0, i1, i2, i3)] = w1 * a.p[off4(a, i0, i1, i2, i3)] + w2 * b.p[off4(b, i0, i1, i2, i3)];
    }
}

__global__ void k_iadd(int32_t *p, int delta) { p[0] += delta; }

extern "C" int gb_iadd(gb_ctx *ctx, int32_t *counter, int delta) {
    if (!ctx || !counter) return GB_EARG;
    k_iadd<<<1, 1, 0, ctx->stream>>>(counter, delta);
    return gb_after_launch(ctx, "iadd");
}

// n device-to-device copies in one launch: table[3b .. 3b+2] = (dst, src, bytes) of copy b (blocks
// along y), 8-byte elements
__global__ void k_copy_many(const unsigned long long *table) {
    const int b = blockIdx.y;
    double *dst = reinterpret_cast<double *>(table[3 * b]);
    const double *src = reinterpret_cast<const double *>(table[3 * b + 1]);
    const unsigned long long cnt = table[3 * b + 2] / 8;
    for (unsigned long long e = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; e < cnt;
         e += (unsigned long long)gridDim.x * blockDim.x)
        dst[e] = src[e];
}

extern "C" int gb_copy_many(gb_ctx *ctx, const uint64_t *table, int n, size_t max_bytes) {
    if (!ctx || (n > 0 && !table) || n < 0 || n > 65535 || max_bytes % 8 != 0) return GB_EARG;
    if (n == 0 || max_bytes == 0) return GB_OK;
    const unsigned long long elems = max_bytes / 8;
    const unsigned gx = (unsigned)((elems + 255) / 256 < 1024 ? (elems + 255) / 256 : 1024);
    k_copy_many<<<dim3(gx, (unsigned)n), 256, 0, ctx->stream>>>(reinterpret_cast<const unsigned long long *>(table));
    return gb_after_launch(ctx, "copy_many");
}

// the GPU's global nanosecond timer when the stream reaches this point
__global__ void k_stamp(unsigned long long *buf, int slot) {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    buf[slot] = t;
}

extern "C" int gb_stamp(gb_ctx *ctx, uint64_t *buf, int slot) {
    if (!ctx || !buf || slot < 0) return GB_EARG;
    k_stamp<<<1, 1, 0, ctx->stream>>>(reinterpret_cast<unsigned long long *>(buf), slot);
    return gb_after_launch(ctx, "stamp");
}

extern "C" int gb_interp(gb_ctx *ctx, const gb_view *dst, const gb_view *a, const gb_view *b, const double *w) {
    if (!dst || !a || !b || !w) return GB_EARG;
    DV d = dv(dst);
    int64_t total = d.n0 * d.n1 * d.n2 * d.n3;
    if (total <= 0) return GB_OK;
    k_interp<<<launch_grid(total), 256, 0, ctx->stream>>>(d, dv(a), dv(b), w, total);
    return gb_after_launch(ctx, "interp");
}

// dst[...] = seqsum over `axis` of src (accumulated in index order), times post_mul if != 1
__global__ void k_seqsum(DV d, DV s, int axis, int64_t len, double post_mul, int use_mul, int64_t total) {
    int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    int64_t sstep = axis == 0 ? s.s0 : axis == 1 ? s.s1 : axis == 2 ? s.s2 : s.s3;
    for (; k < total; k += stride) {
        int64_t r = k;
        int64_t i3 = r % d.n3; r /= d.n3;
        int64_t i2 = r % d.n2; r /= d.n2;
        int64_t i1 = r % d.n1; r /= d.n1;
        int64_t i0 = r;
        const double *q = s.p + off4(s, i0, i1, i2, i3);
        double acc = q[0];
        for (int64_t t = 1; t < len; ++t) acc = acc + q[t * sstep];
        if (use_mul) acc = acc * post_mul;
        d.p[off4(d, i0, i1, i2, i3)] = acc;
    }
}

extern "C" int gb_seqsum(gb_ctx *ctx, const gb_view *dst, const gb_view *src, int axis, double post_mul) {
    if (!dst || !src || axis < 0 || axis > 3) return GB_EARG;
    DV d = dv(dst), s = dv(src);
    int64_t len = src->n[axis];
    // the destination iterates src's other axes; the summed axis has extent 1 there
    int64_t total = d.n0 * d.n1 * d.n2 * d.n3;
    if (total <= 0) return GB_OK;
    k_seqsum<<<launch_grid(total), 256, 0, ctx->stream>>>(d, s, axis, len, post_mul, post_mul != 1.0, total);
    return gb_after_launch(ctx, "seqsum");
}
