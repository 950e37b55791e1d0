// Context, scratch memory, error plumbing, CSR layout and the FP64 peak probe.
#include "common.cuh"
#include "mie_device.cuh"

#include <stdlib.h>
#include <string.h>

int ctx_fail(gbmie_ctx *ctx, int status, const char *fmt, ...)
{
    if (ctx) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(ctx->err, sizeof(ctx->err), fmt, ap);
        va_end(ap);
    }
    return status;
}

int ctx_cuda(gbmie_ctx *ctx, cudaError_t e, const char *what)
{
    if (e == cudaSuccess) return GBMIE_OK;
    int st = (e == cudaErrorMemoryAllocation) ? GBMIE_ERR_NOMEM : GBMIE_ERR_CUDA;
    return ctx_fail(ctx, st, "%s: %s", what, cudaGetErrorString(e));
}

void ctx_pre_launch(gbmie_ctx *ctx)
{
    if (!ctx->timing || ctx->ntimer >= GBMIE_TIMER_CAP) return;
    gbmie_timer_rec &r = ctx->timers[ctx->ntimer];
    if (!r.start) {
        cudaEventCreate(&r.start);
        cudaEventCreate(&r.stop);
    }
    cudaEventRecord(r.start, ctx->stream);
    ctx->timer_open = 1;
}

int ctx_check_launch(gbmie_ctx *ctx, const char *what)
{
    ctx->launches++;
    if (ctx->timer_open) {
        gbmie_timer_rec &r = ctx->timers[ctx->ntimer];
        cudaEventRecord(r.stop, ctx->stream);
        r.name = what;
        ctx->ntimer++;
        ctx->timer_open = 0;
    }
    return ctx_cuda(ctx, cudaGetLastError(), what);
}

int ctx_scratch(gbmie_ctx *ctx, size_t bytes, void **ptr)
{
    if (bytes == 0) bytes = 256;
    if (bytes > ctx->scratch_bytes) {
        // the scratch block may be in use on any stream the context was bound to
        GBMIE_TRY(ctx_cuda(ctx, cudaDeviceSynchronize(), "scratch sync"));
        if (ctx->scratch) cudaFree(ctx->scratch);
        ctx->scratch = NULL;
        ctx->scratch_bytes = 0;
        size_t want = align_up(bytes + bytes / 4, 1 << 20);
        cudaError_t e = cudaMalloc(&ctx->scratch, want);
        if (e != cudaSuccess) {
            e = cudaMalloc(&ctx->scratch, bytes);
            want = bytes;
        }
        GBMIE_TRY(ctx_cuda(ctx, e, "scratch allocation"));
        ctx->scratch_bytes = want;
    }
    *ptr = ctx->scratch;
    return GBMIE_OK;
}

int ctx_angle_op_get(gbmie_ctx *ctx, const double *hcos, int n_ang, int n_pad, int k_pad, int nmax, size_t bytes,
                     void **bt, int *entry, int *fresh)
{
    *bt = nullptr;
    *entry = -1;
    *fresh = 0;
    const int cap = (int)(sizeof(ctx->angle_ops) / sizeof(ctx->angle_ops[0]));
    for (int i = 0; i < cap; ++i) {
        gbmie_ctx::AngleOp &e = ctx->angle_ops[i];
        if (e.bt && e.n_ang == n_ang && e.n_pad == n_pad && e.k_pad == k_pad && e.nmax == nmax &&
            memcmp(e.hcos, hcos, sizeof(double) * n_ang) == 0) {
            ++e.refs;
            *bt = e.bt;
            *entry = i;
            return GBMIE_OK;
        }
    }
    // a free slot, else an unused entry is evicted
    int slot = -1;
    for (int i = 0; i < cap && slot < 0; ++i)
        if (!ctx->angle_ops[i].bt) slot = i;
    for (int i = 0; i < cap && slot < 0; ++i)
        if (ctx->angle_ops[i].refs == 0) {
            cudaFree(ctx->angle_ops[i].bt);
            free(ctx->angle_ops[i].hcos);
            ctx->angle_ops[i].bt = nullptr;
            slot = i;
        }
    void *mem = nullptr;
    GBMIE_TRY(ctx_cuda(ctx, cudaMalloc(&mem, bytes), "angle-function operand"));
    if (slot < 0) {   // every entry in use: a plan-owned operand outside the cache
        *bt = mem;
        *fresh = 1;
        return GBMIE_OK;
    }
    gbmie_ctx::AngleOp &e = ctx->angle_ops[slot];
    e.hcos = (double *)malloc(sizeof(double) * n_ang);
    if (!e.hcos) {
        cudaFree(mem);
        return GBMIE_ERR_NOMEM;
    }
    memcpy(e.hcos, hcos, sizeof(double) * n_ang);
    e.bt = mem;
    e.n_ang = n_ang;
    e.n_pad = n_pad;
    e.k_pad = k_pad;
    e.nmax = nmax;
    e.refs = 1;
    *bt = mem;
    *entry = slot;
    *fresh = 1;
    return GBMIE_OK;
}

void ctx_angle_op_release(gbmie_ctx *ctx, int entry)
{
    if (entry >= 0 && ctx->angle_ops[entry].refs > 0) --ctx->angle_ops[entry].refs;
}

extern "C" {

const char *gbmie_status_string(int status)
{
    switch (status) {
    case GBMIE_OK: return "ok";
    case GBMIE_ERR_INVALID: return "invalid argument";
    case GBMIE_ERR_NMAX: return "nmax above GBMIE_MAX_NMAX";
    case GBMIE_ERR_CUDA: return "CUDA error";
    case GBMIE_ERR_TIMEOUT: return "device wait timed out";
    case GBMIE_ERR_NOMEM: return "out of device memory";
    case GBMIE_ERR_UNSUPPORTED: return "unsupported option";
    case GBMIE_ERR_CAPACITY: return "request exceeds the fixed device array of gbmie_s12_noalloc";
    default: return "unknown status";
    }
}

const char *gbmie_last_error(const gbmie_ctx *ctx) { return ctx ? ctx->err : "no context"; }

int64_t gbmie_launch_count(const gbmie_ctx *ctx) { return ctx ? ctx->launches : 0; }

int gbmie_ctx_create(int device, gbmie_ctx **out)
{
    if (!out) return GBMIE_ERR_INVALID;
    *out = NULL;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return GBMIE_ERR_CUDA;
    if (cudaSetDevice(device) != cudaSuccess) return GBMIE_ERR_CUDA;
    gbmie_ctx *ctx = (gbmie_ctx *)calloc(1, sizeof(gbmie_ctx));
    if (!ctx) return GBMIE_ERR_NOMEM;
    ctx->device = device;
    ctx->stream = 0;
    if (cudaMalloc(&ctx->d_flags, 64) != cudaSuccess ||
        cudaMallocHost(&ctx->h_flags, 64) != cudaSuccess ||
        cudaMallocHost(&ctx->h_pinned, 4096) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming) != cudaSuccess) {
        gbmie_ctx_destroy(ctx);
        return GBMIE_ERR_NOMEM;
    }
    cudaMemset(ctx->d_flags, 0, 64);
    // plan arrays are stream-ordered allocations from the device's default
    // pool: keep freed blocks in the pool (the default threshold returns them
    // to the CUDA driver at every synchronisation) so that plan creation reuses
    // them; a process-level attribute of the pool, no device setting
    {
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
            uint64_t keep = UINT64_MAX;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
    }
    cudaDeviceSynchronize();
    *out = ctx;
    return GBMIE_OK;
}

int gbmie_ctx_destroy(gbmie_ctx *ctx)
{
    if (!ctx) return GBMIE_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    else cudaDeviceSynchronize();
    if (ctx->scratch) cudaFree(ctx->scratch);
    table_cache_release(ctx);
    for (auto &e : ctx->angle_ops) {
        if (e.bt) cudaFree(e.bt);
        free(e.hcos);
    }
    if (ctx->timers) {
        for (int i = 0; i < GBMIE_TIMER_CAP; ++i)
            if (ctx->timers[i].start) {
                cudaEventDestroy(ctx->timers[i].start);
                cudaEventDestroy(ctx->timers[i].stop);
            }
        free(ctx->timers);
    }
    if (ctx->side) {
        cudaStreamSynchronize(ctx->side);
        cudaStreamDestroy(ctx->side);
    }
    if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
    if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
    if (ctx->d_flags) cudaFree(ctx->d_flags);
    if (ctx->h_flags) cudaFreeHost(ctx->h_flags);
    if (ctx->h_pinned) cudaFreeHost(ctx->h_pinned);
    free(ctx);
    return GBMIE_OK;
}

int gbmie_ctx_set_timing(gbmie_ctx *ctx, int enable)
{
    if (!ctx) return GBMIE_ERR_INVALID;
    if (enable && !ctx->timers) {
        ctx->timers = (gbmie_timer_rec *)calloc(GBMIE_TIMER_CAP, sizeof(gbmie_timer_rec));
        if (!ctx->timers) return GBMIE_ERR_NOMEM;
    }
    ctx->timing = enable ? 1 : 0;
    ctx->ntimer = 0;
    ctx->timer_open = 0;
    return GBMIE_OK;
}

int gbmie_ctx_kernel_times(gbmie_ctx *ctx, int32_t cap, const char **names, int64_t *launches, double *total_ms,
                           int32_t *n)
{
    if (!ctx || !n || cap < 0 || (cap > 0 && (!names || !launches || !total_ms))) return GBMIE_ERR_INVALID;
    *n = 0;
    if (!ctx->timers) return GBMIE_OK;
    GBMIE_TRY(ctx_cuda(ctx, cudaStreamSynchronize(ctx->stream), "timing sync"));
    int nk = 0;
    for (int i = 0; i < ctx->ntimer; ++i) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ctx->timers[i].start, ctx->timers[i].stop);
        int k = 0;
        while (k < nk && strcmp(names[k], ctx->timers[i].name) != 0) ++k;
        if (k == nk) {
            if (nk >= cap) continue;
            names[k] = ctx->timers[i].name;
            launches[k] = 0;
            total_ms[k] = 0.0;
            ++nk;
        }
        launches[k] += 1;
        total_ms[k] += ms;
    }
    *n = nk;
    return GBMIE_OK;
}

int gbmie_ctx_set_stream(gbmie_ctx *ctx, void *stream)
{
    if (!ctx) return GBMIE_ERR_INVALID;
    ctx->stream = (cudaStream_t)stream;
    return GBMIE_OK;
}

// Synchronise and turn device-side flags into a status.
int gbmie_ctx_synchronize(gbmie_ctx *ctx)
{
    if (!ctx) return GBMIE_ERR_INVALID;
    GBMIE_TRY(ctx_cuda(ctx, cudaMemcpyAsync(ctx->h_flags, ctx->d_flags, sizeof(int), cudaMemcpyDeviceToHost,
                                            ctx->stream), "flag readback"));
    GBMIE_TRY(ctx_cuda(ctx, cudaStreamSynchronize(ctx->stream), "stream synchronize"));
    int f = ctx->h_flags[0];
    if (f) {
        cudaMemsetAsync(ctx->d_flags, 0, sizeof(int), ctx->stream);
        cudaStreamSynchronize(ctx->stream);
        if (f & GBMIE_FLAG_TIMEOUT) return ctx_fail(ctx, GBMIE_ERR_TIMEOUT, "device wait hit its iteration limit");
        if (f & GBMIE_FLAG_NMAX)
            return ctx_fail(ctx, GBMIE_ERR_NMAX, "an instance needs more partial waves than the call allows "
                                                 "(GBMIE_MAX_NMAX = %d, or the given row length)", GBMIE_MAX_NMAX);
        return ctx_fail(ctx, GBMIE_ERR_INVALID, "invalid instance parameters (x < 0, y < x, NaN, "
                                               "or coated with mu != 1)");
    }
    return GBMIE_OK;
}

} // extern "C"

// ---------------------------------------------------------------------------
// CSR layout: offsets[i+1] - offsets[i] = nmax(size[i]) + add_per_row.
// Three passes: per-block scan, scan of block totals, add block bases.
// ---------------------------------------------------------------------------
// one row per thread in 256-thread blocks: the rows' nmax (an FP64 pow each)
// spread over every SM (120,000 rows: 469 blocks rather than 30)
#define SCAN_THREADS 256
#define SCAN_ITEMS 1

__device__ __forceinline__ int64_t block_exclusive_scan(int64_t v, int64_t *total)
{
    __shared__ int64_t warp_tot[32];
    __shared__ int64_t block_tot;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int64_t inc = v;
    for (int o = 1; o < 32; o <<= 1) {
        int64_t t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) warp_tot[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        int64_t w = lane < nw ? warp_tot[lane] : 0;
        int64_t wi = w;
        for (int o = 1; o < 32; o <<= 1) {
            int64_t t = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += t;
        }
        if (lane < nw) warp_tot[lane] = wi - w;
        if (lane == 31) block_tot = wi;
    }
    __syncthreads();
    const int64_t excl = warp_tot[wid] + inc - v;
    *total = block_tot;
    __syncthreads();
    return excl;
}

__global__ void k_layout_blocks(int64_t n, const double *__restrict__ size, int64_t add, int64_t *__restrict__ off,
                                int64_t *__restrict__ bsum, int *__restrict__ flags)
{
    const int64_t base = (int64_t)blockIdx.x * SCAN_THREADS * SCAN_ITEMS + (int64_t)threadIdx.x * SCAN_ITEMS;
    int64_t c[SCAN_ITEMS];
    int64_t s = 0;
    int bad = 0;
    for (int j = 0; j < SCAN_ITEMS; ++j) {
        const int64_t i = base + j;
        c[j] = 0;
        if (i < n) {
            const double x = size[i];
            if (!(x >= 0.0) || !isfinite(x)) {
                bad |= GBMIE_FLAG_INVALID;
                c[j] = 2 + add;
            } else {
                int nm = mie_nmax(x);
                if (nm > GBMIE_MAX_NMAX) {
                    bad |= GBMIE_FLAG_NMAX;
                    nm = GBMIE_MAX_NMAX;
                }
                c[j] = nm + add;
            }
        }
        s += c[j];
    }
    if (bad) atomicOr(flags, bad);
    int64_t tot;
    int64_t e = block_exclusive_scan(s, &tot);
    for (int j = 0; j < SCAN_ITEMS; ++j) {
        const int64_t i = base + j;
        e += c[j];
        if (i < n) off[i + 1] = e;
    }
    if (threadIdx.x == 0) {
        bsum[blockIdx.x] = tot;
        if (blockIdx.x == 0) off[0] = 0;
    }
}

__global__ void k_layout_bsum(int64_t nb, int64_t *__restrict__ bsum, int64_t *__restrict__ total)
{
    int64_t carry = 0;
    for (int64_t b0 = 0; b0 < nb; b0 += SCAN_THREADS) {
        const int64_t b = b0 + threadIdx.x;
        const int64_t v = b < nb ? bsum[b] : 0;
        int64_t tot;
        const int64_t e = block_exclusive_scan(v, &tot);
        if (b < nb) bsum[b] = carry + e;
        carry += tot;
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void k_layout_add(int64_t n, const int64_t *__restrict__ bsum, int64_t *__restrict__ off)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) off[i + 1] += bsum[i / (SCAN_THREADS * SCAN_ITEMS)];
}

// total_host may be NULL (no synchronisation); bsum scratch is carved from the
// end of the offsets' neighbour: callers pass a buffer of nb+1 int64 in `aux`.
static int layout_impl(gbmie_ctx *ctx, int64_t n, const double *size, int64_t add, int64_t *off, int64_t *aux,
                       int64_t *total_dev)
{
    const int64_t per = SCAN_THREADS * SCAN_ITEMS;
    const int64_t nb = ceil_div64(n, per);
    ctx_pre_launch(ctx);
    k_layout_blocks<<<(unsigned)nb, SCAN_THREADS, 0, ctx->stream>>>(n, size, add, off, aux, ctx->d_flags);
    GBMIE_TRY(ctx_check_launch(ctx, "k_layout_blocks"));
    ctx_pre_launch(ctx);
    k_layout_bsum<<<1, SCAN_THREADS, 0, ctx->stream>>>(nb, aux, total_dev);
    GBMIE_TRY(ctx_check_launch(ctx, "k_layout_bsum"));
    ctx_pre_launch(ctx);
    k_layout_add<<<(unsigned)ceil_div64(n, 256), 256, 0, ctx->stream>>>(n, aux, off);
    return ctx_check_launch(ctx, "k_layout_add");
}

// Internal: layout into `offsets` with a private block-sum buffer; optional
// synchronous total.
int launch_layout(gbmie_ctx *ctx, int64_t n, const double *size, int64_t add_per_row, int64_t *offsets,
                  int64_t *total_host)
{
    const int64_t nb = ceil_div64(n, SCAN_THREADS * SCAN_ITEMS);
    int64_t *aux = NULL;
    GBMIE_TRY(ctx_cuda(ctx, cudaMallocAsync((void **)&aux, (size_t)(nb + 2) * sizeof(int64_t), ctx->stream),
                       "layout aux"));
    int st = layout_impl(ctx, n, size, add_per_row, offsets, aux, aux + nb + 1);
    if (st == GBMIE_OK && total_host) {
        st = ctx_cuda(ctx, cudaMemcpyAsync(ctx->h_pinned, aux + nb + 1, sizeof(int64_t), cudaMemcpyDeviceToHost,
                                           ctx->stream), "layout total");
    }
    cudaFreeAsync(aux, ctx->stream);
    if (st != GBMIE_OK) return st;
    if (total_host) {
        GBMIE_TRY(gbmie_ctx_synchronize(ctx));
        *total_host = ctx->h_pinned[0];
    }
    return GBMIE_OK;
}

extern "C" int gbmie_layout(gbmie_ctx *ctx, int64_t n, const double *size, int64_t *offsets, int64_t *total)
{
    if (!ctx || n < 0 || (n > 0 && (!size || !offsets))) return ctx_fail(ctx, GBMIE_ERR_INVALID, "gbmie_layout: bad arguments");
    cudaSetDevice(ctx->device);
    if (n == 0) {
        GBMIE_TRY(ctx_cuda(ctx, cudaMemsetAsync(offsets, 0, sizeof(int64_t), ctx->stream), "layout"));
        if (total) *total = 0;
        return gbmie_ctx_synchronize(ctx);
    }
    int64_t t = 0;
    GBMIE_TRY(launch_layout(ctx, n, size, 0, offsets, &t));
    if (total) *total = t;
    return GBMIE_OK;
}

__global__ void k_nmax_one(double x, int *out) { *out = mie_nmax(x); }

extern "C" int gbmie_nmax(gbmie_ctx *ctx, double x, int32_t *nmax)
{
    if (!ctx || !nmax || !(x >= 0.0) || !isfinite(x)) return ctx_fail(ctx, GBMIE_ERR_INVALID, "gbmie_nmax: bad x");
    cudaSetDevice(ctx->device);
    int *d = NULL;
    GBMIE_TRY(ctx_cuda(ctx, cudaMallocAsync((void **)&d, sizeof(int), ctx->stream), "nmax alloc"));
    ctx_pre_launch(ctx);
    k_nmax_one<<<1, 1, 0, ctx->stream>>>(x, d);
    int st = ctx_check_launch(ctx, "k_nmax_one");
    if (st == GBMIE_OK)
        st = ctx_cuda(ctx, cudaMemcpyAsync(ctx->h_pinned, d, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream),
                      "nmax copy");
    cudaFreeAsync(d, ctx->stream);
    GBMIE_TRY(st);
    GBMIE_TRY(ctx_cuda(ctx, cudaStreamSynchronize(ctx->stream), "nmax sync"));
    *nmax = ((int *)ctx->h_pinned)[0];
    return GBMIE_OK;
}

// ---------------------------------------------------------------------------
// FP64 peak probe: 8 independent DFMA chains per thread, a multiple of the
// SM count in blocks.  2 flop per DFMA.
// ---------------------------------------------------------------------------
__global__ void k_fp64_peak(int iters, double seed, double *sink)
{
    double a0 = seed + threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3;
    double a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
    const double b = 0.999999, c = 1e-7;
#pragma unroll 1
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            a0 = fma(a0, b, c); a1 = fma(a1, b, c); a2 = fma(a2, b, c); a3 = fma(a3, b, c);
            a4 = fma(a4, b, c); a5 = fma(a5, b, c); a6 = fma(a6, b, c); a7 = fma(a7, b, c);
        }
    }
    double s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (s == 42.0) sink[0] = s;
}

extern "C" int gbmie_measure_fp64_peak(gbmie_ctx *ctx, double *gflops)
{
    if (!ctx || !gflops) return GBMIE_ERR_INVALID;
    cudaSetDevice(ctx->device);
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device);
    double *sink = NULL;
    GBMIE_TRY(ctx_cuda(ctx, cudaMallocAsync((void **)&sink, sizeof(double), ctx->stream), "peak alloc"));
    const int threads = 256, blocks = nsm * 8, iters = 4096;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_fp64_peak<<<blocks, threads, 0, ctx->stream>>>(64, 1.0, sink);  // warm-up
    cudaEventRecord(e0, ctx->stream);
    k_fp64_peak<<<blocks, threads, 0, ctx->stream>>>(iters, 1.0, sink);
    cudaEventRecord(e1, ctx->stream);
    ctx->launches += 2;
    cudaError_t e = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFreeAsync(sink, ctx->stream);
    GBMIE_TRY(ctx_cuda(ctx, e, "peak run"));
    const double flop = 2.0 * 8.0 * 8.0 * (double)iters * threads * blocks;
    *gflops = flop / (ms * 1e-3) / 1e9;
    return GBMIE_OK;
}
