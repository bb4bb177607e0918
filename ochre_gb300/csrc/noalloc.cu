// Rasterization for callers that must not allocate device memory.
//
// Some hosts budget all GPU memory up front and forbid driver allocations
// afterwards: renderers that reserve their memory at start-up because
// cudaMalloc/cudaFree synchronise the device and can stall a frame, and
// applications where another framework's allocator owns the device memory.
// ochre_gpu_rasterize_noalloc runs the same chain as
// ochre_gpu_rasterize_device but takes every intermediate buffer from one
// file-scope device array (OCHRE_NOALLOC_SCRATCH_BYTES) and writes results
// into buffers the caller provides.  It calls no cudaMalloc, cudaFree or
// other allocating routine.
//
// The array is shared by every call and keeps the previous call's contents;
// each stage clears what must start at zero (scan and sort look-back state,
// tickets, device scalars) before it runs.  Calls that overlap on the GPU
// (for example on two streams) race on the array; calls from several host
// threads are serialised by a mutex, and a call that fails waits for the
// work it already queued before it releases the array, so the next call
// (on any stream) never meets kernels of a failed one still writing into it.
#include <mutex>

#include "common.cuh"
#include "internal.h"

namespace {

constexpr size_t kScratchBytes = OCHRE_NOALLOC_SCRATCH_BYTES;

// The scratch itself.  Host code must not pass `g_scratch` to a kernel: in
// host code the name is a host-side stand-in, so every call looks the device
// address up with cudaGetSymbolAddress, with the calling device current.  The
// lookup allocates nothing; doing it per call (not once per device) keeps the
// address right when a context is torn down and created again, which reloads
// the module and may place the array elsewhere.
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

ochre::DevScalars g_host_scalars;  // host copy of the run's device scalars
std::mutex g_mutex;

void use_arena(ochre::DevBuf& b, ochre::Arena* a) {
    b.p = nullptr;
    b.cap = 0;
    b.arena = a;
    b.fixed = false;
}

void use_caller(ochre::DevBuf& b, void* p, size_t bytes, ochre::Arena* a) {
    b.p = p;
    b.cap = p ? bytes : 0;
    b.arena = a;   // only to report overflow
    b.fixed = true;
}

}  // namespace

extern "C" int ochre_gpu_rasterize_noalloc(const ochre_batch* in, ochre_output_buffers* out, void* stream) {
    if (in == nullptr || out == nullptr) return OCHRE_E_INVALID;
    if (out->tile_xy == nullptr || out->tile_alpha == nullptr || out->span_xy == nullptr ||
        out->span_width == nullptr || out->span_tile == nullptr || out->raster_tile_off == nullptr ||
        out->raster_span_off == nullptr)
        return OCHRE_E_INVALID;
    // the kernels store tile rows 8 bytes at a time and positions as 32-bit words
    auto misaligned = [](const void* p, uintptr_t a) { return (reinterpret_cast<uintptr_t>(p) & (a - 1)) != 0; };
    if (misaligned(out->tile_xy, 4) || misaligned(out->tile_alpha, 8) || misaligned(out->span_xy, 4) ||
        misaligned(out->span_width, 2) || misaligned(out->span_tile, 4) || misaligned(out->raster_tile_off, 4) ||
        misaligned(out->raster_span_off, 4))
        return OCHRE_E_INVALID;
    out->n_tiles = 0;
    out->n_spans = 0;
    std::lock_guard<std::mutex> lock(g_mutex);
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return OCHRE_E_CUDA;
    // The array's device address on the current device.  The first call on a
    // device loads the library's device code there (placing the array).
    void* scratch = nullptr;
    {
        const cudaError_t e = cudaGetSymbolAddress(&scratch, g_scratch);
        if (e != cudaSuccess || scratch == nullptr) {
            cudaGetLastError();
            return OCHRE_E_CUDA;
        }
    }

    ochre::Arena arena;
    arena.base = static_cast<char*>(scratch);
    arena.size = kScratchBytes;

    ochre_gpu_ctx ctx;
    ctx.device = dev;
    ctx.flags = 0;
    // the fused path's per-CTA staging comes from the array too: a smaller
    // persistent grid keeps it to a few MB
    ctx.fused_max_ctas = 256;
    ctx.no_side_stream = true;   // creates no stream: every kernel on the caller's
    ctx.own_stream = static_cast<cudaStream_t>(stream);
    ochre::DevBuf* internal[] = {&ctx.in_verbs, &ctx.in_pts, &ctx.in_fill_off, &ctx.in_fill_xf,
                                 &ctx.in_fill_flags, &ctx.in_raster_off, &ctx.cmd_foff, &ctx.cmd_mv, &ctx.cmd_ep,
                                 &ctx.cmd_line_off, &ctx.lines, &ctx.line_raster, &ctx.line_ent_off, &ctx.line_inc_off,
                                 &ctx.long_lines, &ctx.incs,
                                 &ctx.raster_bbox, &ctx.raster_keybase, &ctx.raster_empty,
                                 &ctx.raster_wsum, &ctx.raster_wbase, &ctx.tile_head_bins, &ctx.tile_head_wind, &ctx.keys, &ctx.vals,
                                 &ctx.keys_alt, &ctx.vals_alt, &ctx.bins, &ctx.sort_hist, &ctx.sort_lookback,
                                 &ctx.tile_head, &ctx.tile_info, &ctx.tile_row_start, &ctx.tile_state, &ctx.span_flag, &ctx.span_val,
                                 &ctx.scan_status, &ctx.scalars, &ctx.fused_chain, &ctx.fused_stage, &ctx.out_tile_cov,
                                 &ctx.grad_g, &ctx.grad_gs, &ctx.grad_left, &ctx.grad_line, &ctx.grad_pts,
                                 &ctx.sk_cmd_foff, &ctx.sk_cmd_mv, &ctx.sk_cmd_ep, &ctx.sk_poly_off,
                                 &ctx.sk_poly_foff, &ctx.sk_pverbs, &ctx.sk_ppts, &ctx.sk_pfoff, &ctx.sk_pfill_off,
                                 &ctx.sk_first_close, &ctx.sk_unit_start, &ctx.sk_out_off, &ctx.sk_out_foff,
                                 &ctx.sk_unit_fill, &ctx.sk_overbs, &ctx.sk_opts, &ctx.sk_ofill_off, &ctx.sk_oflags,
                                 &ctx.in_fill_width};
    for (ochre::DevBuf* b : internal) use_arena(*b, &arena);
    const size_t R1 = (size_t)in->n_rasters + 1;
    use_caller(ctx.out_tile_xy, out->tile_xy, (size_t)out->tile_capacity * 4, &arena);
    use_caller(ctx.out_tile_alpha, out->tile_alpha, (size_t)out->tile_capacity * 64, &arena);
    use_caller(ctx.out_span_xy, out->span_xy, (size_t)out->span_capacity * 4, &arena);
    use_caller(ctx.out_span_w, out->span_width, (size_t)out->span_capacity * 2, &arena);
    use_caller(ctx.out_span_tile, out->span_tile, (size_t)out->span_capacity * 4, &arena);
    use_caller(ctx.out_raster_tile_off, out->raster_tile_off, R1 * 4, &arena);
    use_caller(ctx.out_raster_span_off, out->raster_span_off, R1 * 4, &arena);
    if (ctx.scalars.ensure(sizeof(ochre::DevScalars)) != cudaSuccess) return OCHRE_E_CAPACITY;
    ctx.h_scalars.p = &g_host_scalars;
    ctx.h_scalars.cap = sizeof(g_host_scalars);

    if (in->n_rasters > ochre::MAX_RASTERS || in->n_cmds > ochre::MAX_COUNT) return OCHRE_E_CAPACITY;
    if (in->raster_fill_off == nullptr && in->n_rasters != in->n_fills) return OCHRE_E_INVALID;
    ochre_result res;
    int st = ochre::run_device(&ctx, in, &res, ctx.own_stream);
    if (st != OCHRE_OK) {
        // A stage can fail after launching kernels (an intermediate that no
        // longer fits the array is only found when the next stage sizes its
        // buffers).  Wait for them while the array is still held.
        cudaStreamSynchronize(ctx.own_stream);
        cudaGetLastError();
        if (arena.overflow) st = OCHRE_E_CAPACITY;
    }
    if (st == OCHRE_OK) {
        out->n_tiles = res.n_tiles;
        out->n_spans = res.n_spans;
    }
    // ctx's buffers point into the arena or at the caller's memory: nothing
    // to release.
    ctx.h_scalars.p = nullptr;
    return st;
}
