// Headless compositing of rasterization results into an RGBA8 canvas: the
// reference example's GL path (examples/svg.rs) restated on the device.
//   * every tile is an 8x8 quad textured with its alpha mask, every span an
//     n x 8 quad with mask 1 (atlas texel (0,0) = 255, :33-38, 85-87);
//   * fragment = raster colour * (1, 1, 1, mask) (:341-353);
//   * blend SRC_ALPHA, ONE_MINUS_SRC_ALPHA on all four channels (:173-174)
//     into an RGBA8 target, quantised after every quad: f -> floor(f*255 + 0.5);
//   * rasters are drawn in order (:139-165); within one raster no two quads
//     overlap, so only the raster order matters per pixel.
// The GL pipeline itself is unavailable on this machine; this kernel and the
// oracle restate its arithmetic.
//
// Device form: every quad is cut into the 8x8 screen tiles it covers (tile
// and span positions are multiples of 8), each piece keyed by (screen tile,
// raster) and radix-sorted; one warp per screen tile then blends its pieces
// in raster order, two pixels per lane, with the canvas in registers.
#include "common.cuh"
#include "internal.h"
#include "scan.cuh"

namespace ochre {

struct PieceCount {
    const int16_t* tile_xy;
    const int16_t* span_xy;
    const uint16_t* span_w;
    uint32_t T;
    int w, h, w8;
    __device__ __forceinline__ uint32_t operator()(uint64_t i) const {
        if (i < T) {
            const int x = tile_xy[2 * i], y = tile_xy[2 * i + 1];
            return (x >= 0 && y >= 0 && x < w && y < h) ? 1u : 0u;
        }
        const uint64_t s = i - T;
        const int x = span_xy[2 * s], y = span_xy[2 * s + 1];
        if (y < 0 || y >= h) return 0u;
        const int x0 = max(x, 0), x1 = min(x + (int)span_w[s], 8 * w8);
        return x1 > x0 ? (uint32_t)((x1 - x0) >> 3) : 0u;
    }
};
struct PieceOff {
    uint32_t* off;
    __device__ __forceinline__ void operator()(uint64_t i, uint32_t ex, uint32_t) const { off[i] = ex; }
};

__global__ void k_piece_emit(const int16_t* __restrict__ tile_xy, const int16_t* __restrict__ span_xy,
                             const uint16_t* __restrict__ span_w, const uint32_t* __restrict__ raster_tile_off,
                             const uint32_t* __restrict__ raster_span_off, uint32_t R, uint32_t T, uint32_t N, int w,
                             int h, int w8, uint32_t rbits, const uint32_t* __restrict__ off,
                             uint64_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= (uint64_t)T + N) return;
    uint32_t o = off[i];
    if (i < T) {
        const int x = tile_xy[2 * i], y = tile_xy[2 * i + 1];
        if (!(x >= 0 && y >= 0 && x < w && y < h)) return;
        const uint32_t r = upper_bound_u32(raster_tile_off, R + 1, (uint32_t)i) - 1u;
        const uint64_t st = (uint64_t)(y >> 3) * w8 + (x >> 3);
        keys[o] = (st << rbits) | r;
        vals[o] = (uint32_t)i;
        return;
    }
    const uint32_t s = (uint32_t)(i - T);
    const int x = span_xy[2 * s], y = span_xy[2 * s + 1];
    if (y < 0 || y >= h) return;
    const int x0 = max(x, 0), x1 = min(x + (int)span_w[s], 8 * w8);
    const uint32_t r = upper_bound_u32(raster_span_off, R + 1, s) - 1u;
    for (int xx = x0; xx < x1; xx += 8) {
        const uint64_t st = (uint64_t)(y >> 3) * w8 + (xx >> 3);
        keys[o] = (st << rbits) | r;
        vals[o] = T + s;
        o++;
    }
}

__device__ __forceinline__ uint32_t unorm8(float f) {
    float q = floorf(__fadd_rn(__fmul_rn(f, 255.0f), 0.5f));
    if (!(q >= 0.0f)) q = 0.0f;
    if (q > 255.0f) q = 255.0f;
    return (uint32_t)q;
}

// dst: RGBA8 packed little-endian (r in the low byte)
__device__ __forceinline__ uint32_t blend_px(uint32_t dst, uint32_t col, uint32_t mask) {
    const float a = __fmul_rn(__fdiv_rn((float)(col >> 24), 255.0f), __fdiv_rn((float)mask, 255.0f));
    const float ia = __fsub_rn(1.0f, a);
    uint32_t out = 0;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const float s = __fdiv_rn((float)((col >> (8 * c)) & 0xffu), 255.0f);
        const float d = __fdiv_rn((float)((dst >> (8 * c)) & 0xffu), 255.0f);
        out |= unorm8(__fadd_rn(__fmul_rn(s, a), __fmul_rn(d, ia))) << (8 * c);
    }
    const float d = __fdiv_rn((float)(dst >> 24), 255.0f);
    out |= unorm8(__fadd_rn(__fmul_rn(a, a), __fmul_rn(d, ia))) << 24;
    return out;
}

__device__ __forceinline__ uint64_t lower_bound_u64(const uint64_t* a, uint64_t n, uint64_t v) {
    uint64_t lo = 0, hi = n;
    while (lo < hi) {
        const uint64_t mid = (lo + hi) >> 1;
        if (a[mid] < v) lo = mid + 1; else hi = mid;
    }
    return lo;
}

__global__ void k_composite(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ vals, uint64_t E,
                            uint32_t rbits, uint32_t T, const uint8_t* __restrict__ tile_alpha,
                            const uint32_t* __restrict__ colors, uint32_t n_rasters, uint32_t w, uint32_t h,
                            uint32_t w8, uint32_t h8, uint32_t* __restrict__ canvas, const uint32_t* err) {
    const uint64_t st = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    // a wait of the sort gave up: the sorted pieces are not valid
    if (st >= (uint64_t)w8 * h8 || run_aborted(err)) return;
    const uint64_t lo = lower_bound_u64(keys, E, st << rbits);
    const uint64_t hi = lower_bound_u64(keys, E, (st + 1) << rbits);
    if (lo == hi) return;
    const uint32_t tx = (uint32_t)(st % w8), ty = (uint32_t)(st / w8);
    const uint32_t rmask = (1u << rbits) - 1u;
    uint32_t px[2];
    bool in[2];
    size_t idx[2];
#pragma unroll
    for (int k = 0; k < 2; k++) {
        const uint32_t p = 2 * lane + k;
        const uint32_t x = 8 * tx + (p & 7), y = 8 * ty + (p >> 3);
        in[k] = x < w && y < h;
        idx[k] = (size_t)y * w + x;
        px[k] = in[k] ? canvas[idx[k]] : 0u;
    }
    for (uint64_t e = lo; e < hi; e++) {
        const uint32_t r = (uint32_t)(keys[e] & rmask);
        const uint32_t v = vals[e];
        if (r >= n_rasters) continue;
        const uint32_t col = colors[r];
#pragma unroll
        for (int k = 0; k < 2; k++) {
            const uint32_t mask = v < T ? tile_alpha[(size_t)v * 64 + 2 * lane + k] : 255u;
            px[k] = blend_px(px[k], col, mask);
        }
    }
#pragma unroll
    for (int k = 0; k < 2; k++)
        if (in[k]) canvas[idx[k]] = px[k];
}

}  // namespace ochre

using namespace ochre;

extern "C" int ochre_gpu_composite(ochre_gpu_ctx* ctx, const ochre_result* res, uint32_t n_rasters,
                                   const uint8_t* colors, uint32_t w, uint32_t h, uint8_t* canvas, void* stream) {
    if (!ctx || !res || (n_rasters && !colors) || (w && h && !canvas)) return OCHRE_E_INVALID;
    if (w > 32768 || h > 32768 || n_rasters > MAX_RASTERS) return OCHRE_E_INVALID;
    if ((reinterpret_cast<uintptr_t>(canvas) & 3) || (reinterpret_cast<uintptr_t>(colors) & 3)) return OCHRE_E_INVALID;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return OCHRE_E_CUDA;
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->own_stream;
    ctx->epoch++;   // the sort below reuses the chain's buffers
    ctx->prof_used = 0;
    ctx->launches = 0;
    const uint32_t T = res->n_tiles, N = res->n_spans;
    if (w == 0 || h == 0 || n_rasters == 0 || (uint64_t)T + N == 0) return OCHRE_OK;
    const uint32_t w8 = (w + 7) / 8, h8 = (h + 7) / 8;
    uint32_t rbits = 1;
    while (rbits < 32 && ((n_rasters - 1) >> rbits)) rbits++;
    uint32_t sbits = 1;
    while (sbits < 40 && (((uint64_t)w8 * h8 - 1) >> sbits)) sbits++;
    DevScalars* ds = dev_scalars(ctx);
    const uint64_t S = (uint64_t)T + N;
    OCHRE_CUDA_TRY(ctx->line_ent_off.ensure(S * 4));
    OCHRE_CUDA_TRY(ctx->scan_status.ensure(scan_tiles(S) * sizeof(ScanStatus<uint32_t>)));
    OCHRE_CUDA_TRY(reset_scalars(ctx, s));
    OCHRE_LAUNCH(ctx, "composite_count", s, OCHRE_CUDA_TRY(launch_scan<uint32_t>(
        S, PieceCount{res->tile_xy, res->span_xy, res->span_width, T, (int)w, (int)h, (int)w8},
        PieceOff{ctx->line_ent_off.as<uint32_t>()}, OpSumU32{}, 0u, ctx->scan_status.p, &ds->ticket,
        &ds->n_line_ent, &ds->err, s)));
    int st = read_scalars(ctx, s);
    if (st != OCHRE_OK) return st;
    st = check_device_error(ctx);
    if (st != OCHRE_OK) return st;
    const uint64_t E = host_scalars(ctx)->n_line_ent;
    if (E == 0) return OCHRE_OK;
    if (E > MAX_COUNT) return OCHRE_E_CAPACITY;
    ctx->keys64 = true;
    OCHRE_CUDA_TRY(ctx->keys.ensure(E * 8));
    OCHRE_CUDA_TRY(ctx->vals.ensure(E * 4));
    OCHRE_CUDA_TRY(ctx->keys_alt.ensure(E * 8));
    OCHRE_CUDA_TRY(ctx->vals_alt.ensure(E * 4));
    OCHRE_LAUNCH(ctx, "composite_pieces", s, k_piece_emit<<<(unsigned)((S + 255) / 256), 256, 0, s>>>(
        res->tile_xy, res->span_xy, res->span_width, res->raster_tile_off, res->raster_span_off, n_rasters, T, N,
        (int)w, (int)h, (int)w8, rbits, ctx->line_ent_off.as<uint32_t>(), ctx->keys.as<uint64_t>(),
        ctx->vals.as<uint32_t>()));
    OCHRE_CUDA_TRY(cudaGetLastError());
    uint32_t passes = 0;
    st = stage_sort(ctx, E, sbits + rbits, s, &passes);
    if (st != OCHRE_OK) return st;
    const uint64_t threads = (uint64_t)w8 * h8 * 32;
    OCHRE_LAUNCH(ctx, "composite", s, k_composite<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(
        ctx->keys.as<uint64_t>(), ctx->vals.as<uint32_t>(), E, rbits, T, res->tile_alpha,
        reinterpret_cast<const uint32_t*>(colors), n_rasters, w, h, w8, h8, reinterpret_cast<uint32_t*>(canvas),
        &ds->err));
    OCHRE_CUDA_TRY(cudaGetLastError());
    ctx->stats.n_launches = ctx->launches;
    collect_timings(ctx, s);
    return check_device_error(ctx);
}
