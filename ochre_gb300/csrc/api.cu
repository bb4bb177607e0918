// C ABI (include/ochre_gpu.h): contexts, orchestration of the kernel chain,
// the host-buffer entry point and the single-rasterizer mirror of ochre's
// Rust API (src/rasterizer.rs).
#include <cuda_runtime.h>

#include <cmath>
#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "common.cuh"
#include "flatten.cuh"
#include "scan.cuh"
#include "internal.h"

namespace ochre {

cudaError_t DevBuf::ensure(size_t bytes) {
    if (bytes <= cap && p != nullptr) return cudaSuccess;
    if (fixed) {
        if (arena != nullptr) arena->overflow = true;
        return cudaErrorMemoryAllocation;
    }
    if (arena != nullptr) {
        const size_t need = (bytes + 255) & ~(size_t)255;
        if (arena->used + need > arena->size) {
            arena->overflow = true;
            return cudaErrorMemoryAllocation;
        }
        p = arena->base + arena->used;
        cap = need;
        arena->used += need;
        return cudaSuccess;
    }
    if (bytes == 0) bytes = 16;
    size_t want = cap ? cap : 256;
    while (want < bytes) want *= 2;
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, want);
    if (e != cudaSuccess) {
        // retry at the exact size before giving up
        cudaGetLastError();
        e = cudaMalloc(&q, bytes);
        if (e != cudaSuccess) return e;
        want = bytes;
    }
    if (p) cudaFree(p);
    p = q;
    cap = want;
    return cudaSuccess;
}
void DevBuf::release() {
    if (p && arena == nullptr && !fixed) cudaFree(p);
    p = nullptr;
    cap = 0;
}
cudaError_t HostBuf::ensure(size_t bytes) {
    if (bytes <= cap && p != nullptr) return cudaSuccess;
    if (bytes == 0) bytes = 16;
    size_t want = cap ? cap : 256;
    while (want < bytes) want *= 2;
    void* q = nullptr;
    cudaError_t e = cudaMallocHost(&q, want);
    if (e != cudaSuccess) return e;
    if (p) cudaFreeHost(p);
    p = q;
    dev = nullptr;
    cap = want;
    return cudaSuccess;
}
cudaError_t HostBuf::ensure_mapped(size_t bytes) {
    if (bytes <= cap && p != nullptr && dev != nullptr) return cudaSuccess;
    if (bytes == 0) bytes = 16;
    size_t want = cap ? cap : 256;
    while (want < bytes) want *= 2;
    void* q = nullptr;
    void* d = nullptr;
    cudaError_t e = cudaHostAlloc(&q, want, cudaHostAllocMapped);
    if (e != cudaSuccess) return e;
    e = cudaHostGetDevicePointer(&d, q, 0);
    if (e != cudaSuccess) {
        cudaFreeHost(q);
        return e;
    }
    if (p) cudaFreeHost(p);
    p = q;
    dev = d;
    cap = want;
    return cudaSuccess;
}
void HostBuf::release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    dev = nullptr;
    cap = 0;
}

__global__ void k_copy_words(const uint32_t* __restrict__ src, uint32_t n, uint32_t* dst) {
    const uint32_t i = threadIdx.x;
    if (i < n) dst[i] = src[i];
}

__global__ void k_plan_cap(uint32_t* count, uint32_t cap, uint32_t* err) {
    if (*count > cap) {
        *count = 0u;
        atomicOr(err, ERR_CAPACITY);
    }
}

__global__ void k_plan_entries(DevScalars* ds, uint32_t cap, uint32_t key_bits, uint32_t inc_cap) {
    const uint64_t e = (uint64_t)ds->line_ent_total + ds->n_empty;
    const uint64_t k = ds->keyspace;
    const bool keys_fit = key_bits >= 64 || k == 0 || ((k - 1) >> key_bits) == 0;
    if (e > cap || !keys_fit || ds->inc_total > inc_cap) {
        ds->n_entries = 0u;
        ds->n_lines = 0u;   // no line emits an entry
        atomicOr(&ds->err, ERR_CAPACITY);
    } else {
        ds->n_entries = (uint32_t)e;
    }
}

cudaError_t launch_plan_cap(ochre_gpu_ctx* ctx, uint32_t* count, uint32_t cap, cudaStream_t s) {
    k_plan_cap<<<1, 1, 0, s>>>(count, cap, &dev_scalars(ctx)->err);
    return cudaGetLastError();
}

cudaError_t launch_plan_entries(ochre_gpu_ctx* ctx, uint32_t cap, uint32_t key_bits, uint32_t inc_cap,
                                cudaStream_t s) {
    k_plan_entries<<<1, 1, 0, s>>>(dev_scalars(ctx), cap, key_bits, inc_cap);
    return cudaGetLastError();
}

void wait_inputs(ochre_gpu_ctx* ctx, cudaStream_t s) {
    if (!ctx->pts_pending) return;
    cudaStreamWaitEvent(s, ctx->ev_pts, 0);
    ctx->pts_pending = false;
}

int copy_scalars_async(ochre_gpu_ctx* ctx, cudaStream_t s) {
    static_assert(sizeof(DevScalars) / 4 <= 64, "one word per thread of k_copy_words");
    if (ctx->h_scalars_dev) {
        k_copy_words<<<1, 64, 0, s>>>(ctx->scalars.as<uint32_t>(), (uint32_t)(sizeof(DevScalars) / 4),
                                       static_cast<uint32_t*>(ctx->h_scalars_dev));
        OCHRE_CUDA_TRY(cudaGetLastError());
    } else {
        OCHRE_CUDA_TRY(cudaMemcpyAsync(ctx->h_scalars.p, ctx->scalars.p, sizeof(DevScalars), cudaMemcpyDeviceToHost,
                                       s));
    }
    return OCHRE_OK;
}

cudaError_t reset_scalars(ochre_gpu_ctx* ctx, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(ctx->scalars.p, 0, sizeof(DevScalars), s);
    if (e == cudaSuccess && ctx->test_spin_log2 != 0u)
        e = cudaMemcpyAsync(&dev_scalars(ctx)->spin_log2, &ctx->test_spin_log2, sizeof(uint32_t),
                            cudaMemcpyHostToDevice, s);
    return e;
}

int read_scalars(ochre_gpu_ctx* ctx, cudaStream_t s) {
    const int st = copy_scalars_async(ctx, s);
    if (st != OCHRE_OK) return st;
    OCHRE_CUDA_TRY(cudaStreamSynchronize(s));
    return OCHRE_OK;
}

void prof_begin(ochre_gpu_ctx* ctx, const char* name, cudaStream_t s) {
    ctx->launches++;
    if (!(ctx->flags & OCHRE_CTX_PROFILE)) return;
    if (ctx->prof_used == ctx->prof.size()) {
        ochre_gpu_ctx::Prof p{name, nullptr, nullptr};
        if (cudaEventCreate(&p.a) != cudaSuccess || cudaEventCreate(&p.b) != cudaSuccess) {
            cudaGetLastError();
            return;
        }
        ctx->prof.push_back(p);
    }
    ochre_gpu_ctx::Prof& p = ctx->prof[ctx->prof_used];
    p.name = name;
    cudaEventRecord(p.a, s);
}

void prof_end(ochre_gpu_ctx* ctx, cudaStream_t s) {
    if (!(ctx->flags & OCHRE_CTX_PROFILE) || ctx->prof_used >= ctx->prof.size()) return;
    cudaEventRecord(ctx->prof[ctx->prof_used].b, s);
    ctx->prof_used++;
}

// Converts the recorded event pairs of the finished run into timings.
void collect_timings(ochre_gpu_ctx* ctx, cudaStream_t s) {
    ctx->timings.clear();
    if (!(ctx->flags & OCHRE_CTX_PROFILE) || ctx->prof_used == 0) return;
    cudaStreamSynchronize(s);
    for (uint32_t i = 0; i < ctx->prof_used; i++) {
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, ctx->prof[i].a, ctx->prof[i].b) != cudaSuccess) {
            cudaGetLastError();
            ms = -1.0f;
        }
        ctx->timings.push_back(ochre_kernel_time{ctx->prof[i].name, ms});
    }
}

int check_device_error(ochre_gpu_ctx* ctx) {
    const uint32_t e = host_scalars(ctx)->err;
    if (e & ERR_INVALID) return OCHRE_E_INVALID;
    if (e & ERR_LIMIT) return OCHRE_E_LIMIT;
    if (e & ERR_TIMEOUT) return OCHRE_E_TIMEOUT;
    if (e & ERR_CAPACITY) return OCHRE_E_CAPACITY;
    return OCHRE_OK;
}

// 1 when a[0..n] is non-decreasing.  No early exit: the loop vectorises,
// and reading the array (host memory) is what it costs.
static bool non_decreasing(const uint32_t* a, uint64_t n) {
    uint32_t bad = 0;
    for (uint64_t i = 0; i < n; i++) bad |= (uint32_t)(a[i + 1] < a[i]);
    return bad == 0;
}

int run_device(ochre_gpu_ctx* ctx, const ochre_batch* in_orig, ochre_result* out, cudaStream_t s, bool remember_miss) {
    // the test hooks apply to this run only
    struct HookReset {
        ochre_gpu_ctx* c;
        ~HookReset() {
            c->test_spin_log2 = 0;
            c->test_skip_first_ticket = 0;
        }
    } hook_reset{ctx};
    std::memset(out, 0, sizeof *out);
    ctx->epoch++;
    ctx->stats = ochre_stats{};
    ctx->prof_used = 0;
    ctx->launches = 0;
    ctx->timings.clear();
    // stroked fills become plain fills first (Rasterizer::stroke, rasterizer.rs:169-171)
    ochre_batch expanded;
    {
        const int sst = stage_stroke(ctx, in_orig, s, &expanded);
        if (sst != OCHRE_OK) return sst;
    }
    const ochre_batch* in = &expanded;
    OCHRE_CUDA_TRY(reset_scalars(ctx, s));
    const uint32_t R = in->n_rasters;
    OCHRE_CUDA_TRY(ctx->out_raster_tile_off.ensure((size_t)(R + 1) * 4));
    OCHRE_CUDA_TRY(ctx->out_raster_span_off.ensure((size_t)(R + 1) * 4));
    if (R == 0) {
        OCHRE_CUDA_TRY(cudaMemsetAsync(ctx->out_raster_tile_off.p, 0, 4, s));
        OCHRE_CUDA_TRY(cudaMemsetAsync(ctx->out_raster_span_off.p, 0, 4, s));
        out->raster_tile_off = ctx->out_raster_tile_off.as<uint32_t>();
        out->raster_span_off = ctx->out_raster_span_off.as<uint32_t>();
        return OCHRE_OK;
    }
    uint32_t T = 0, N = 0;
    bool handled = false;
    int st = OCHRE_OK;
    // a batch that did not fit the fused kernel last time (same arrays and
    // counts) goes to the chain directly; the results are the same either way
    const bool known_miss = remember_miss && ctx->fused_miss_valid && same_batch(ctx->fused_miss, *in_orig);
    if (!(ctx->flags & OCHRE_CTX_CHAIN_ONLY) && !known_miss) {
        st = stage_fused(ctx, in, s, &handled, &T, &N);
        if (st != OCHRE_OK) return st;
        if (remember_miss) {
            ctx->fused_miss_valid = !handled;
            if (!handled) ctx->fused_miss = *in_orig;
        }
    }
    if (handled) {
        ctx->stats.fused = 1;
    } else {
        OCHRE_CUDA_TRY(reset_scalars(ctx, s));
        uint32_t L = 0;
        st = stage_flatten(ctx, in, s, &L);
        if (st != OCHRE_OK) return st;
        uint64_t E = 0;
        uint32_t bits = 0;
        st = stage_bin(ctx, in, L, s, &E, &bits);
        if (st != OCHRE_OK) return st;
        uint32_t passes = 0;
        st = stage_sort(ctx, E, bits, s, &passes);
        if (st != OCHRE_OK) return st;
        st = stage_tiles(ctx, in, E, s, &T, &N);
        if (st != OCHRE_OK) return st;
        ctx->stats.n_lines = L;
        ctx->stats.n_entries = E;
        ctx->stats.key_bits = bits;
        ctx->stats.sort_passes = passes;
    }
    ctx->stats.n_tiles = T;
    ctx->stats.n_spans = N;
    ctx->stats.n_launches = ctx->launches;
    collect_timings(ctx, s);
    out->n_tiles = T;
    out->n_spans = N;
    out->tile_xy = ctx->out_tile_xy.as<int16_t>();
    out->tile_alpha = ctx->out_tile_alpha.as<uint8_t>();
    out->tile_cov = (ctx->flags & OCHRE_CTX_WANT_COV) ? ctx->out_tile_cov.as<float>() : nullptr;
    out->span_xy = ctx->out_span_xy.as<int16_t>();
    out->span_width = ctx->out_span_w.as<uint16_t>();
    out->span_tile = ctx->out_span_tile.as<uint32_t>();
    out->raster_tile_off = ctx->out_raster_tile_off.as<uint32_t>();
    out->raster_span_off = ctx->out_raster_span_off.as<uint32_t>();
    return OCHRE_OK;
}

}  // namespace ochre

using namespace ochre;

extern "C" {

const char* ochre_gpu_status_string(int status) {
    switch (status) {
    case OCHRE_OK: return "ok";
    case OCHRE_E_INVALID: return "invalid input";
    case OCHRE_E_CAPACITY: return "size limit exceeded";
    case OCHRE_E_CUDA: return "CUDA error";
    case OCHRE_E_TIMEOUT: return "bounded device wait timed out";
    case OCHRE_E_NOMEM: return "out of memory";
    case OCHRE_E_LIMIT: return "iteration cap hit (input would not terminate in the reference)";
    default: return "unknown status";
    }
}

int ochre_gpu_create(ochre_gpu_ctx** out, int device, uint32_t flags) {
    if (!out) return OCHRE_E_INVALID;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) return OCHRE_E_CUDA;
    ochre_gpu_ctx* ctx = new (std::nothrow) ochre_gpu_ctx();
    if (!ctx) return OCHRE_E_NOMEM;
    ctx->device = device;
    ctx->flags = flags;
    if (cudaSetDevice(device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
        ctx->scalars.ensure(sizeof(DevScalars)) != cudaSuccess) {
        ochre_gpu_destroy(ctx);
        return OCHRE_E_CUDA;
    }
    // scalars read back through mapped pinned host memory
    {
        void* hp = nullptr;
        void* dp = nullptr;
        if (cudaHostAlloc(&hp, sizeof(DevScalars), cudaHostAllocMapped) == cudaSuccess &&
            cudaHostGetDevicePointer(&dp, hp, 0) == cudaSuccess) {
            std::memset(hp, 0, sizeof(DevScalars));
            ctx->h_scalars.p = hp;
            ctx->h_scalars.cap = sizeof(DevScalars);
            ctx->h_scalars_dev = dp;
        } else {
            cudaGetLastError();
            if (hp) cudaFreeHost(hp);
            if (ctx->h_scalars.ensure(sizeof(DevScalars)) != cudaSuccess) {
                ochre_gpu_destroy(ctx);
                return OCHRE_E_CUDA;
            }
        }
    }
    *out = ctx;
    return OCHRE_OK;
}

void ochre_gpu_destroy(ochre_gpu_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->own_stream) cudaStreamSynchronize(ctx->own_stream);
    for (DevBuf* b : device_buffers(ctx)) b->release();
    HostBuf* host[] = {&ctx->h_scalars, &ctx->h_tile_xy, &ctx->h_tile_alpha, &ctx->h_tile_cov, &ctx->h_span_xy,
                       &ctx->h_span_w, &ctx->h_span_tile, &ctx->h_raster_tile_off, &ctx->h_raster_span_off};
    for (HostBuf* b : host) b->release();
    for (auto& p : ctx->prof) {
        cudaEventDestroy(p.a);
        cudaEventDestroy(p.b);
    }
    if (ctx->copy_stream) {
        cudaStreamSynchronize(ctx->copy_stream);
        cudaStreamDestroy(ctx->copy_stream);
    }
    if (ctx->walk_stream) {
        cudaStreamSynchronize(ctx->walk_stream);
        cudaStreamDestroy(ctx->walk_stream);
    }
    if (ctx->ev_walk_fork) cudaEventDestroy(ctx->ev_walk_fork);
    if (ctx->ev_walk_join) cudaEventDestroy(ctx->ev_walk_join);
    if (ctx->ev_prior) cudaEventDestroy(ctx->ev_prior);
    if (ctx->ev_pts) cudaEventDestroy(ctx->ev_pts);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    delete ctx;
}

}  // extern "C"

namespace ochre {

std::vector<DevBuf*> device_buffers(ochre_gpu_ctx* ctx) {
    return {&ctx->in_verbs, &ctx->in_pts, &ctx->in_fill_off, &ctx->in_fill_xf, &ctx->in_fill_flags,
                     &ctx->in_raster_off, &ctx->cmd_foff, &ctx->cmd_mv, &ctx->cmd_ep, &ctx->cmd_line_off,
                     &ctx->lines, &ctx->line_raster, &ctx->line_ent_off, &ctx->line_inc_off, &ctx->long_lines, &ctx->incs, &ctx->raster_bbox, &ctx->raster_keybase,
                     &ctx->raster_empty, &ctx->raster_wsum, &ctx->raster_wbase, &ctx->tile_head_bins,
                     &ctx->tile_head_wind, &ctx->keys, &ctx->vals, &ctx->keys_alt, &ctx->vals_alt, &ctx->bins,
                     &ctx->sort_hist, &ctx->sort_lookback, &ctx->tile_head, &ctx->tile_info, &ctx->tile_row_start, &ctx->tile_state,
                     &ctx->span_flag, &ctx->span_val, &ctx->scan_status, &ctx->scalars, &ctx->fused_chain, &ctx->fused_stage,
                     &ctx->grad_g, &ctx->grad_gs, &ctx->grad_left, &ctx->grad_line, &ctx->grad_pts,
                     &ctx->sk_cmd_foff, &ctx->sk_cmd_mv, &ctx->sk_cmd_ep, &ctx->sk_poly_off, &ctx->sk_poly_foff,
                     &ctx->sk_pverbs, &ctx->sk_ppts, &ctx->sk_pfoff, &ctx->sk_pfill_off, &ctx->sk_first_close,
                     &ctx->sk_unit_start, &ctx->sk_out_off, &ctx->sk_out_foff, &ctx->sk_unit_fill, &ctx->sk_overbs,
                     &ctx->sk_opts, &ctx->sk_ofill_off, &ctx->sk_oflags, &ctx->in_fill_width,
                     &ctx->out_tile_xy,
                     &ctx->out_tile_alpha, &ctx->out_tile_cov, &ctx->out_span_xy, &ctx->out_span_w,
                     &ctx->out_span_tile, &ctx->out_raster_tile_off, &ctx->out_raster_span_off};
}

}  // namespace ochre

extern "C" {

int ochre_gpu_set_flags(ochre_gpu_ctx* ctx, uint32_t flags) {
    if (!ctx) return OCHRE_E_INVALID;
    ctx->flags = flags;
    return OCHRE_OK;
}

int ochre_gpu_rasterize_device(ochre_gpu_ctx* ctx, const ochre_batch* in, ochre_result* out, void* stream) {
    if (!ctx || !in || !out) return OCHRE_E_INVALID;
    if (in->n_rasters > MAX_RASTERS || in->n_cmds > MAX_COUNT) return OCHRE_E_CAPACITY;
    if (in->raster_fill_off == nullptr && in->n_rasters != in->n_fills) return OCHRE_E_INVALID;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return OCHRE_E_CUDA;
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->own_stream;
    return run_device(ctx, in, out, s, true);
}

int ochre_validate_batch(const ochre_batch* in) {
    if (!in) return OCHRE_E_INVALID;
    if (in->n_fills > 0 && (in->fill_cmd_off == nullptr || in->fill_xf == nullptr)) return OCHRE_E_INVALID;
    if (in->n_cmds > 0 && (in->verbs == nullptr)) return OCHRE_E_INVALID;
    if (in->n_floats > 0 && in->pts == nullptr) return OCHRE_E_INVALID;
    if (in->n_cmds > MAX_COUNT || in->n_floats > 0xffffffffull) return OCHRE_E_CAPACITY;
    if (in->n_rasters > MAX_RASTERS) return OCHRE_E_CAPACITY;
    if (in->raster_fill_off == nullptr && in->n_rasters != in->n_fills) return OCHRE_E_INVALID;
    if (in->n_fills == 0 && in->n_cmds != 0) return OCHRE_E_INVALID;
    if (in->fill_cmd_off && (in->fill_cmd_off[0] != 0 || in->fill_cmd_off[in->n_fills] != in->n_cmds ||
                             !non_decreasing(in->fill_cmd_off, in->n_fills)))
        return OCHRE_E_INVALID;
    if (in->raster_fill_off && (in->raster_fill_off[0] != 0 || in->raster_fill_off[in->n_rasters] != in->n_fills ||
                                !non_decreasing(in->raster_fill_off, in->n_rasters)))
        return OCHRE_E_INVALID;
    return OCHRE_OK;
}

int ochre_gpu_rasterize(ochre_gpu_ctx* ctx, const ochre_batch* in, ochre_result* out) {
    if (!ctx || !in || !out) return OCHRE_E_INVALID;
    int st = ochre_validate_batch(in);
    if (st != OCHRE_OK) return st;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return OCHRE_E_CUDA;
    cudaStream_t s = ctx->own_stream;
    // host -> device (one copy per array)
    ochre_batch d = *in;
    OCHRE_CUDA_TRY(ctx->in_verbs.ensure(in->n_cmds));
    OCHRE_CUDA_TRY(ctx->in_pts.ensure(in->n_floats * 4));
    OCHRE_CUDA_TRY(ctx->in_fill_off.ensure(((size_t)in->n_fills + 1) * 4));
    OCHRE_CUDA_TRY(ctx->in_fill_xf.ensure((size_t)in->n_fills * 24));
    // Whatever leaves this call, the point copy has finished and the run's
    // stream is past it (the caller may free or reuse its arrays).
    struct JoinInputs {
        ochre_gpu_ctx* ctx;
        cudaStream_t s;
        ~JoinInputs() {
            if (ctx->pts_pending) {
                wait_inputs(ctx, s);
                cudaStreamSynchronize(s);
            }
        }
    } join{ctx, s};
    // A large point array already in pinned host memory is read by the
    // kernels in place (over the C2C link, overlapped with their work);
    // otherwise it goes on a copy stream, so that the other copies and the
    // stages before the first read of points (command and float-offset scans,
    // clears) overlap it.
    const size_t pts_bytes = (size_t)in->n_floats * 4;
    const float* pts_in_place = nullptr;
    if (pts_bytes >= ((size_t)4 << 20)) {
        cudaPointerAttributes pa;
        if (cudaPointerGetAttributes(&pa, in->pts) == cudaSuccess && pa.type == cudaMemoryTypeHost &&
            pa.devicePointer != nullptr)
            pts_in_place = static_cast<const float*>(pa.devicePointer);
        cudaGetLastError();
    }
    bool pts_async = pts_in_place == nullptr && pts_bytes >= ((size_t)4 << 20);
    if (pts_async && !ctx->copy_stream) {
        if (cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&ctx->ev_prior, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&ctx->ev_pts, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            pts_async = false;
        }
    }
    if (pts_async) {
        // after everything already queued on the run's stream (earlier runs read in_pts)
        OCHRE_CUDA_TRY(cudaEventRecord(ctx->ev_prior, s));
        OCHRE_CUDA_TRY(cudaStreamWaitEvent(ctx->copy_stream, ctx->ev_prior, 0));
        OCHRE_CUDA_TRY(cudaMemcpyAsync(ctx->in_pts.p, in->pts, pts_bytes, cudaMemcpyHostToDevice, ctx->copy_stream));
        OCHRE_CUDA_TRY(cudaEventRecord(ctx->ev_pts, ctx->copy_stream));
        ctx->pts_pending = true;
    } else if (in->n_floats && !pts_in_place) {
        OCHRE_CUDA_TRY(cudaMemcpyAsync(ctx->in_pts.p, in->pts, pts_bytes, cudaMemcpyHostToDevice, s));
    }
    if (in->n_cmds) OCHRE_CUDA_TRY(cudaMemcpyAsync(ctx->in_verbs.p, in->verbs, in->n_cmds, cudaMemcpyHostToDevice, s));
    if (in->fill_cmd_off)
        OCHRE_CUDA_TRY(cudaMemcpyAsync(ctx->in_fill_off.p, in->fill_cmd_off, ((size_t)in->n_fills + 1) * 4,
                                       cudaMemcpyHostToDevice, s));
    else
        OCHRE_CUDA_TRY(cudaMemsetAsync(ctx->in_fill_off.p, 0, 4, s));
    if (in->n_fills)
        OCHRE_CUDA_TRY(cudaMemcpyAsync(ctx->in_fill_xf.p, in->fill_xf, (size_t)in->n_fills * 24, cudaMemcpyHostToDevice, s));
    d.verbs = ctx->in_verbs.as<uint8_t>();
    d.pts = pts_in_place ? pts_in_place : ctx->in_pts.as<float>();
    d.fill_cmd_off = ctx->in_fill_off.as<uint32_t>();
    d.fill_xf = ctx->in_fill_xf.as<float>();
    if (in->fill_flags) {
        OCHRE_CUDA_TRY(ctx->in_fill_flags.ensure(in->n_fills));
        OCHRE_CUDA_TRY(cudaMemcpyAsync(ctx->in_fill_flags.p, in->fill_flags, in->n_fills, cudaMemcpyHostToDevice, s));
        d.fill_flags = ctx->in_fill_flags.as<uint8_t>();
    }
    if (in->fill_width && in->n_fills) {
        OCHRE_CUDA_TRY(ctx->in_fill_width.ensure((size_t)in->n_fills * 4));
        OCHRE_CUDA_TRY(cudaMemcpyAsync(ctx->in_fill_width.p, in->fill_width, (size_t)in->n_fills * 4,
                                       cudaMemcpyHostToDevice, s));
        d.fill_width = ctx->in_fill_width.as<float>();
    }
    if (in->raster_fill_off) {
        OCHRE_CUDA_TRY(ctx->in_raster_off.ensure(((size_t)in->n_rasters + 1) * 4));
        OCHRE_CUDA_TRY(cudaMemcpyAsync(ctx->in_raster_off.p, in->raster_fill_off, ((size_t)in->n_rasters + 1) * 4,
                                       cudaMemcpyHostToDevice, s));
        d.raster_fill_off = ctx->in_raster_off.as<uint32_t>();
    }
    // Outputs: when the previous call sized them, the kernels write straight
    // into mapped pinned host memory (no device->host copy after the run);
    // otherwise, or when this batch outgrows them, into device memory, then
    // copied, and the host buffers are resized for the next call.
    const size_t R = in->n_rasters;
    const bool want_cov = (ctx->flags & OCHRE_CTX_WANT_COV) != 0;
    HostBuf* hb[] = {&ctx->h_tile_xy, &ctx->h_tile_alpha, &ctx->h_span_xy, &ctx->h_span_w, &ctx->h_span_tile,
                     &ctx->h_raster_tile_off, &ctx->h_raster_span_off, &ctx->h_tile_cov};
    DevBuf* ob[] = {&ctx->out_tile_xy, &ctx->out_tile_alpha, &ctx->out_span_xy, &ctx->out_span_w, &ctx->out_span_tile,
                    &ctx->out_raster_tile_off, &ctx->out_raster_span_off, &ctx->out_tile_cov};
    const int nb = want_cov ? 8 : 7;
    bool zero_copy = ctx->h_raster_tile_off.dev != nullptr && ctx->h_raster_tile_off.cap >= (R + 1) * 4 &&
                     ctx->h_raster_span_off.cap >= (R + 1) * 4;
    for (int i = 0; i < nb && zero_copy; i++) zero_copy = hb[i]->dev != nullptr;
    ochre_result dr;
    if (zero_copy) {
        Arena flag;   // records an overflow of the fixed outputs
        DevBuf saved[8];
        for (int i = 0; i < nb; i++) {
            saved[i] = *ob[i];
            DevBuf v;
            v.p = hb[i]->dev;
            v.cap = hb[i]->cap;
            v.fixed = true;
            v.arena = &flag;
            *ob[i] = v;
        }
        st = run_device(ctx, &d, &dr, s);
        for (int i = 0; i < nb; i++) *ob[i] = saved[i];
        if (st == OCHRE_OK) {
            OCHRE_CUDA_TRY(cudaStreamSynchronize(s));
            out->n_tiles = dr.n_tiles;
            out->n_spans = dr.n_spans;
            out->tile_xy = ctx->h_tile_xy.as<int16_t>();
            out->tile_alpha = ctx->h_tile_alpha.as<uint8_t>();
            out->tile_cov = (dr.tile_cov && dr.n_tiles) ? ctx->h_tile_cov.as<float>() : nullptr;
            out->span_xy = ctx->h_span_xy.as<int16_t>();
            out->span_width = ctx->h_span_w.as<uint16_t>();
            out->span_tile = ctx->h_span_tile.as<uint32_t>();
            out->raster_tile_off = ctx->h_raster_tile_off.as<uint32_t>();
            out->raster_span_off = ctx->h_raster_span_off.as<uint32_t>();
            return OCHRE_OK;
        }
        if (!flag.overflow && st != OCHRE_E_CAPACITY) return st;   // a real error, not a capacity one
    }
    st = run_device(ctx, &d, &dr, s);
    if (st != OCHRE_OK) return st;
    // device -> pinned host, and host buffers mapped and sized (x1.25) for the next call
    const size_t T = dr.n_tiles, N = dr.n_spans;
    // spans: the general chain reserves one span slot per tile
    const size_t Tc = T + T / 4 + 64, Nc = Tc;
    OCHRE_CUDA_TRY(cudaStreamSynchronize(s));
    OCHRE_CUDA_TRY(ctx->h_tile_xy.ensure_mapped(Tc * 4));
    OCHRE_CUDA_TRY(ctx->h_tile_alpha.ensure_mapped(Tc * 64));
    OCHRE_CUDA_TRY(ctx->h_span_xy.ensure_mapped(Nc * 4));
    OCHRE_CUDA_TRY(ctx->h_span_w.ensure_mapped(Nc * 2));
    OCHRE_CUDA_TRY(ctx->h_span_tile.ensure_mapped(Nc * 4));
    OCHRE_CUDA_TRY(ctx->h_raster_tile_off.ensure_mapped((R + 1) * 4));
    OCHRE_CUDA_TRY(ctx->h_raster_span_off.ensure_mapped((R + 1) * 4));
    if (T) {
        OCHRE_CUDA_TRY(cudaMemcpyAsync(ctx->h_tile_xy.p, dr.tile_xy, T * 4, cudaMemcpyDeviceToHost, s));
        OCHRE_CUDA_TRY(cudaMemcpyAsync(ctx->h_tile_alpha.p, dr.tile_alpha, T * 64, cudaMemcpyDeviceToHost, s));
    }
    if (N) {
        OCHRE_CUDA_TRY(cudaMemcpyAsync(ctx->h_span_xy.p, dr.span_xy, N * 4, cudaMemcpyDeviceToHost, s));
        OCHRE_CUDA_TRY(cudaMemcpyAsync(ctx->h_span_w.p, dr.span_width, N * 2, cudaMemcpyDeviceToHost, s));
        OCHRE_CUDA_TRY(cudaMemcpyAsync(ctx->h_span_tile.p, dr.span_tile, N * 4, cudaMemcpyDeviceToHost, s));
    }
    OCHRE_CUDA_TRY(cudaMemcpyAsync(ctx->h_raster_tile_off.p, dr.raster_tile_off, (R + 1) * 4, cudaMemcpyDeviceToHost, s));
    OCHRE_CUDA_TRY(cudaMemcpyAsync(ctx->h_raster_span_off.p, dr.raster_span_off, (R + 1) * 4, cudaMemcpyDeviceToHost, s));
    if (want_cov) OCHRE_CUDA_TRY(ctx->h_tile_cov.ensure_mapped(Tc * 256));
    if (dr.tile_cov && T)
        OCHRE_CUDA_TRY(cudaMemcpyAsync(ctx->h_tile_cov.p, dr.tile_cov, T * 256, cudaMemcpyDeviceToHost, s));
    OCHRE_CUDA_TRY(cudaStreamSynchronize(s));
    out->n_tiles = dr.n_tiles;
    out->n_spans = dr.n_spans;
    out->tile_xy = ctx->h_tile_xy.as<int16_t>();
    out->tile_alpha = ctx->h_tile_alpha.as<uint8_t>();
    out->tile_cov = (dr.tile_cov && T) ? ctx->h_tile_cov.as<float>() : nullptr;
    out->span_xy = ctx->h_span_xy.as<int16_t>();
    out->span_width = ctx->h_span_w.as<uint16_t>();
    out->span_tile = ctx->h_span_tile.as<uint32_t>();
    out->raster_tile_off = ctx->h_raster_tile_off.as<uint32_t>();
    out->raster_span_off = ctx->h_raster_span_off.as<uint32_t>();
    return OCHRE_OK;
}

int ochre_gpu_last_timings(const ochre_gpu_ctx* ctx, ochre_kernel_time* out, uint32_t cap, uint32_t* n) {
    if (!ctx || !n || (cap && !out)) return OCHRE_E_INVALID;
    const uint32_t m = (uint32_t)ctx->timings.size();
    for (uint32_t i = 0; i < m && i < cap; i++) out[i] = ctx->timings[i];
    *n = m;
    return OCHRE_OK;
}

int ochre_gpu_set_tunable(ochre_gpu_ctx* ctx, const char* name, int value) {
    if (!ctx || !name) return OCHRE_E_INVALID;
    if (!std::strcmp(name, "fused_threads")) {
        if (value != 64 && value != 96 && value != 128) return OCHRE_E_INVALID;
        ctx->tune_fused_threads = value;
    } else if (!std::strcmp(name, "fused_chunk")) {
        if (value != 8 && value != 16 && value != 32) return OCHRE_E_INVALID;
        ctx->tune_fused_chunk = value;
    } else if (!std::strcmp(name, "chain_tiles_per_warp")) {
        if (value != 4 && value != 8 && value != 16) return OCHRE_E_INVALID;
        ctx->tune_chain_tiles_per_warp = value;
    } else if (!std::strcmp(name, "chain_coverage_form")) {
        if (value < 0 || value > 2) return OCHRE_E_INVALID;
        ctx->tune_chain_coverage_form = value;
    } else if (!std::strcmp(name, "sort_digit_bits")) {
        if (value != 8 && value != 11) return OCHRE_E_INVALID;
        ctx->tune_sort_digit_bits = value;
    } else if (!std::strcmp(name, "chain_long_cells")) {
        if (value != 0 && (value < 16 || value > 65535)) return OCHRE_E_INVALID;
        ctx->tune_chain_long_cells = value;
    } else if (!std::strcmp(name, "chain_walk_refill")) {
        if (value < 1 || value > 32) return OCHRE_E_INVALID;
        ctx->tune_chain_walk_refill = value;
    } else if (!std::strcmp(name, "test_spin_log2")) {
        if (value < 0 || value > 40) return OCHRE_E_INVALID;
        ctx->test_spin_log2 = (uint32_t)value;
    } else if (!std::strcmp(name, "test_skip_first_ticket")) {
        if (value < 0 || value > 1) return OCHRE_E_INVALID;
        ctx->test_skip_first_ticket = (uint32_t)value;
    } else {
        return OCHRE_E_INVALID;
    }
    return OCHRE_OK;
}

int ochre_gpu_get_tunable(const ochre_gpu_ctx* ctx, const char* name, int* value) {
    if (!ctx || !name || !value) return OCHRE_E_INVALID;
    if (!std::strcmp(name, "fused_threads")) *value = ctx->tune_fused_threads;
    else if (!std::strcmp(name, "fused_chunk")) *value = ctx->tune_fused_chunk;
    else if (!std::strcmp(name, "chain_tiles_per_warp")) *value = ctx->tune_chain_tiles_per_warp;
    else if (!std::strcmp(name, "chain_coverage_form")) *value = ctx->tune_chain_coverage_form;
    else if (!std::strcmp(name, "chain_long_cells")) *value = ctx->tune_chain_long_cells;
    else if (!std::strcmp(name, "sort_digit_bits")) *value = ctx->tune_sort_digit_bits;
    else if (!std::strcmp(name, "chain_walk_refill")) *value = ctx->tune_chain_walk_refill;
    else return OCHRE_E_INVALID;
    return OCHRE_OK;
}

int ochre_gpu_last_stats(const ochre_gpu_ctx* ctx, ochre_stats* out) {
    if (!ctx || !out) return OCHRE_E_INVALID;
    *out = ctx->stats;
    return OCHRE_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Single-rasterizer mirror: buffers commands on the host like the Rust
// Rasterizer buffers increments, then rasterizes on finish.
// ---------------------------------------------------------------------------
struct ochre_rasterizer {
    ochre_gpu_ctx* ctx;
    std::vector<uint8_t> verbs;
    std::vector<float> pts;
    std::vector<uint32_t> fill_off{0};
    std::vector<float> xf;
    std::vector<uint8_t> flags;
    std::vector<float> width;
    // A run of raw commands (move_to/line_to/command) is one untransformed fill.
    bool open_raw = false;
};

static const float kIdentity[6] = {1.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f};

static void raw_cmd(ochre_rasterizer* r, uint8_t verb, const float* f, int nf) {
    if (!r->open_raw) {
        r->xf.insert(r->xf.end(), kIdentity, kIdentity + 6);
        r->flags.push_back(OCHRE_FILL_RAW);
        r->width.push_back(0.0f);
        r->fill_off.push_back((uint32_t)r->verbs.size());
        r->open_raw = true;
    }
    r->verbs.push_back(verb);
    r->pts.insert(r->pts.end(), f, f + nf);
    r->fill_off.back() = (uint32_t)r->verbs.size();
}

extern "C" {

int ochre_rasterizer_new(ochre_gpu_ctx* ctx, ochre_rasterizer** out) {
    if (!ctx || !out) return OCHRE_E_INVALID;
    *out = new (std::nothrow) ochre_rasterizer();
    if (!*out) return OCHRE_E_NOMEM;
    (*out)->ctx = ctx;
    return OCHRE_OK;
}

int ochre_rasterizer_move_to(ochre_rasterizer* r, float x, float y) {
    if (!r) return OCHRE_E_INVALID;
    const float f[2] = {x, y};
    raw_cmd(r, OCHRE_MOVE, f, 2);
    return OCHRE_OK;
}

int ochre_rasterizer_line_to(ochre_rasterizer* r, float x, float y) {
    if (!r) return OCHRE_E_INVALID;
    const float f[2] = {x, y};
    raw_cmd(r, OCHRE_LINE, f, 2);
    return OCHRE_OK;
}

int ochre_rasterizer_command(ochre_rasterizer* r, uint8_t verb, const float* floats) {
    if (!r || verb > OCHRE_CLOSE) return OCHRE_E_INVALID;
    const int nf = (int)floats_per_verb(verb);
    if (nf && !floats) return OCHRE_E_INVALID;
    raw_cmd(r, verb, floats, nf);
    return OCHRE_OK;
}

int ochre_rasterizer_fill(ochre_rasterizer* r, const uint8_t* verbs, size_t n_verbs, const float* pts,
                          size_t n_floats, const float xf[6]) {
    if (!r || (n_verbs && !verbs) || (n_floats && !pts) || !xf) return OCHRE_E_INVALID;
    size_t need = 0;
    for (size_t i = 0; i < n_verbs; i++) {
        if (verbs[i] > OCHRE_CLOSE) return OCHRE_E_INVALID;
        need += floats_per_verb(verbs[i]);
    }
    if (need > n_floats) return OCHRE_E_INVALID;
    r->open_raw = false;
    r->verbs.insert(r->verbs.end(), verbs, verbs + n_verbs);
    r->pts.insert(r->pts.end(), pts, pts + need);
    r->xf.insert(r->xf.end(), xf, xf + 6);
    r->flags.push_back(0);
    r->width.push_back(0.0f);
    r->fill_off.push_back((uint32_t)r->verbs.size());
    return OCHRE_OK;
}

int ochre_rasterizer_stroke(ochre_rasterizer* r, const uint8_t* verbs, size_t n_verbs, const float* pts,
                            size_t n_floats, float width, const float xf[6]) {
    const int st = ochre_rasterizer_fill(r, verbs, n_verbs, pts, n_floats, xf);
    if (st != OCHRE_OK) return st;
    r->flags.back() = OCHRE_FILL_STROKE;
    r->width.back() = width;
    return OCHRE_OK;
}

void ochre_rasterizer_free(ochre_rasterizer* r) { delete r; }

int ochre_rasterizer_finish(ochre_rasterizer* r, ochre_tile_fn tile, ochre_span_fn span, void* user) {
    if (!r) return OCHRE_E_INVALID;
    ochre_batch b{};
    b.verbs = r->verbs.data();
    b.n_cmds = r->verbs.size();
    b.pts = r->pts.data();
    b.n_floats = r->pts.size();
    b.fill_cmd_off = r->fill_off.data();
    b.fill_xf = r->xf.data();
    b.fill_flags = r->flags.data();
    b.fill_width = r->width.data();
    b.n_fills = (uint32_t)(r->fill_off.size() - 1);
    const uint32_t raster_off[2] = {0, b.n_fills};
    b.raster_fill_off = raster_off;
    b.n_rasters = 1;
    ochre_result res;
    int st = ochre_gpu_rasterize(r->ctx, &b, &res);
    if (st == OCHRE_OK) {
        uint32_t s = 0;
        for (uint32_t t = 0; t < res.n_tiles; t++) {
            if (tile) tile(user, res.tile_xy[2 * t], res.tile_xy[2 * t + 1], res.tile_alpha + 64 * (size_t)t);
            while (s < res.n_spans && res.span_tile[s] == t) {
                if (span) span(user, res.span_xy[2 * s], res.span_xy[2 * s + 1], res.span_width[s]);
                s++;
            }
        }
    }
    delete r;
    return st;
}

}  // extern "C"
