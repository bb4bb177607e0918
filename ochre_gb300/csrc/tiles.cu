// Stage 4: sorted entries -> 8x8 alpha tiles and solid spans.
//
// Reference: the tile loop of finish (rasterizer.rs:213-267):
//   * scatter-add area/height of every increment of a tile (:223-228);
//   * alpha = min(|accum + area| * 256, 255) as u8 with accum the running
//     sum of heights along the pixel row, seeded by the carry `prev` from
//     the tiles to the left on the same tile row (:232-239, 243-250);
//   * a span between this tile and the next one on the row when there is a
//     gap and the running tile-row-crossing winding (never reset, so
//     effectively a prefix over the whole raster) is nonzero (:252-265).
//
// One warp per tile.  Tiles are numbered in sorted order, which is the
// reference's callback order.  The row carry (8 floats, segmented by
// (raster, tile_y)) and the winding (segmented by raster) are single-pass
// chained scans over tiles with decoupled look-back; warps take tiles by
// atomic ticket so a warp only waits on tiles owned by running warps, and
// every wait is bounded.
#include "common.cuh"
#include "internal.h"
#include "scan.cuh"

namespace ochre {

// Tile heads: the first bin entry of every run of equal keys.  The scan also
// counts bin entries (statistics only).
struct HeadScan {
    uint32_t heads;
    uint32_t bins;
};
struct OpHead {
    __device__ __forceinline__ HeadScan operator()(HeadScan a, HeadScan b) const {
        return HeadScan{a.heads + b.heads, a.bins + b.bins};
    }
};
template <class K>
struct HeadIn {
    const K* keys;
    const uint32_t* vals;
    __device__ __forceinline__ HeadScan operator()(uint64_t i) const {
        if (vals[i] & CROSS_TAG) return HeadScan{0u, 0u};
        return HeadScan{(i == 0 || keys[i] != keys[i - 1]) ? 1u : 0u, 1u};
    }
};
struct HeadOut {
    uint32_t* head;
    __device__ __forceinline__ void operator()(uint64_t i, HeadScan ex, HeadScan v) const {
        if (v.heads) head[ex.heads] = (uint32_t)i;
    }
};

template <class K>
__global__ void k_tile_info(const K* __restrict__ keys, const uint32_t* __restrict__ vals,
                            const BinRec* __restrict__ bins, const uint32_t* __restrict__ head, uint32_t n_tiles,
                            uint64_t n_entries, uint32_t n_rasters, TileInfo* __restrict__ info,
                            uint32_t* __restrict__ raster_tile_off) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_tiles) return;
    const uint32_t h = head[t];
    const K key = keys[h];
    const BinRec* rec = bins + vals[h];
    const int r = (int)rec->raster;
    TileInfo ti;
    ti.raster = r;
    ti.tx = div8((int)rec->x);
    ti.ty = div8((int)rec->y);
    ti.head = h;
    uint32_t nb = 1;
    while (h + nb < n_entries && keys[h + nb] == key) nb++;
    ti.nbins = nb;
    int w = 0;
    for (int64_t j = (int64_t)h - 1; j >= 0; j--) {
        const uint32_t v = vals[j];
        if (!(v & CROSS_TAG) || (int)((v >> 8) & 0x7fffffu) != r) break;
        w += (int)(int8_t)(v & 0xffu);
    }
    ti.lwind = w;
    info[t] = ti;
    bool first = t == 0;
    if (!first) first = (int)bins[vals[head[t - 1]]].raster != r;
    if (first) raster_tile_off[r] = t;
    if (t + 1 == n_tiles) raster_tile_off[n_rasters] = n_tiles;
}

constexpr int COV_WARPS = 8;

__global__ void __launch_bounds__(COV_WARPS * 32) k_tile_cov(
    const uint32_t* __restrict__ vals, const BinRec* __restrict__ bins, const float4* __restrict__ lines,
    const TileInfo* __restrict__ info, uint32_t n_tiles, TileState* state, uint32_t* ticket,
    uint32_t* __restrict__ out_xy, uint8_t* __restrict__ out_alpha, float* __restrict__ out_cov,
    uint32_t* __restrict__ span_flag, uint64_t* __restrict__ span_val, uint32_t* err) {
    __shared__ float s_area[COV_WARPS][64];
    __shared__ float s_height[COV_WARPS][64];
    __shared__ float s_carry[COV_WARPS][8];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t t = 0;
    if (lane == 0) t = atomicAdd(ticket, 1u);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= n_tiles) return;
    const TileInfo ti = info[t];
    float* sa = s_area[wid];
    float* sh = s_height[wid];
    sa[lane] = 0.0f; sa[lane + 32] = 0.0f;
    sh[lane] = 0.0f; sh[lane + 32] = 0.0f;
    __syncwarp();

    // Replay every bin of the tile (rasterizer.rs:97-106, 223-228).
    for (uint32_t b = lane; b < ti.nbins; b += 32) {
        const BinRec rec = bins[vals[ti.head + b]];
        if (rec.n == 0) continue;
        const float4 l = lines[rec.line];
        Walk w;
        WalkState s;
        walk_setup(v2(l.x, l.y), v2(l.z, l.w), w, s);
        s.x = rec.x;
        s.y = rec.y;
        s.row_t0 = rec.row_t0;
        s.row_t1 = rec.row_t1;
        s.col_t0 = rec.col_t0;
        s.col_t1 = rec.col_t1;
        for (uint32_t k = 0;; k++) {
            float area, height;
            walk_increment(w, s, area, height);
            const int cell = ((s.y & 7) << 3) | (s.x & 7);
            atomicAdd(sa + cell, area);
            atomicAdd(sh + cell, height);
            if (k + 1 >= rec.n) break;
            walk_step(w, s);
        }
    }
    __syncwarp();

    // lane -> cells 2*lane, 2*lane+1 of row lane/4
    const int row = lane >> 2;
    const int c0 = 2 * lane;
    const float a0 = sa[c0], a1 = sa[c0 + 1], h0 = sh[c0], h1 = sh[c0 + 1];
    const float hs = h0 + h1;
    float incl = hs;
    {
        const float u1 = __shfl_up_sync(0xffffffffu, incl, 1, 4);
        if ((lane & 3) >= 1) incl += u1;
        const float u2 = __shfl_up_sync(0xffffffffu, incl, 2, 4);
        if ((lane & 3) >= 2) incl += u2;
    }
    float excl = __shfl_up_sync(0xffffffffu, incl, 1, 4);
    if ((lane & 3) == 0) excl = 0.0f;
    // row totals live in lanes 4*row+3; gather them to lane 0's view
    float ragg[8];
#pragma unroll
    for (int y = 0; y < 8; y++) ragg[y] = __shfl_sync(0xffffffffu, incl, 4 * y + 3);

    if (lane == 0) {
        TileState* me = state + t;
        const bool row_first = t == 0 || info[t - 1].raster != ti.raster || info[t - 1].ty != ti.ty;
        const bool ras_first = t == 0 || info[t - 1].raster != ti.raster;
        // publish aggregates (or inclusive values for segment heads)
        if (row_first) {
            for (int y = 0; y < 8; y++) st_relaxed(reinterpret_cast<uint32_t*>(&me->rinc[y]), __float_as_uint(ragg[y]));
            __threadfence();
            st_release(&me->rflag, 2u);
        } else {
            for (int y = 0; y < 8; y++) st_relaxed(reinterpret_cast<uint32_t*>(&me->ragg[y]), __float_as_uint(ragg[y]));
            __threadfence();
            st_release(&me->rflag, 1u);
        }
        if (ras_first) {
            st_relaxed(reinterpret_cast<uint32_t*>(&me->winc), (uint32_t)ti.lwind);
            __threadfence();
            st_release(&me->wflag, 2u);
        } else {
            st_relaxed(reinterpret_cast<uint32_t*>(&me->wagg), (uint32_t)ti.lwind);
            __threadfence();
            st_release(&me->wflag, 1u);
        }
        // row carry: exclusive prefix of row sums over earlier tiles of the row
        float carry[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        if (!row_first) {
            int64_t j = (int64_t)t - 1;
            long long spins = 0;
            while (j >= 0) {
                const uint32_t f = ld_acquire(&state[j].rflag);
                if (f == 0u) {
                    if (++spins > SPIN_LIMIT) { atomicOr(err, ERR_TIMEOUT); break; }
                    if (spins > 64) __nanosleep(64);
                    continue;
                }
                const float* src = f == 2u ? state[j].rinc : state[j].ragg;
                for (int y = 0; y < 8; y++)
                    carry[y] = __uint_as_float(ld_relaxed(reinterpret_cast<const uint32_t*>(src + y))) + carry[y];
                if (f == 2u) break;
                --j;
            }
            for (int y = 0; y < 8; y++)
                st_relaxed(reinterpret_cast<uint32_t*>(&me->rinc[y]), __float_as_uint(carry[y] + ragg[y]));
            __threadfence();
            st_release(&me->rflag, 2u);
        }
        // winding: inclusive prefix of crossing signs over the raster
        int wind = ti.lwind;
        if (!ras_first) {
            int pre = 0;
            int64_t j = (int64_t)t - 1;
            long long spins = 0;
            while (j >= 0) {
                const uint32_t f = ld_acquire(&state[j].wflag);
                if (f == 0u) {
                    if (++spins > SPIN_LIMIT) { atomicOr(err, ERR_TIMEOUT); break; }
                    if (spins > 64) __nanosleep(64);
                    continue;
                }
                pre += (int)ld_relaxed(reinterpret_cast<const uint32_t*>(f == 2u ? &state[j].winc : &state[j].wagg));
                if (f == 2u) break;
                --j;
            }
            wind = pre + ti.lwind;
            st_relaxed(reinterpret_cast<uint32_t*>(&me->winc), (uint32_t)wind);
            __threadfence();
            st_release(&me->wflag, 2u);
        }
        for (int y = 0; y < 8; y++) s_carry[wid][y] = carry[y];
        // tile position and the span that may follow it
        out_xy[t] = (uint32_t)(uint16_t)(int16_t)(ti.tx * 8) | ((uint32_t)(uint16_t)(int16_t)(ti.ty * 8) << 16);
        uint32_t has_span = 0;
        if (t + 1 < n_tiles) {
            const TileInfo nx = info[t + 1];
            if (nx.raster == ti.raster && nx.ty == ti.ty && nx.tx > ti.tx + 1 && wind != 0) {
                has_span = 1;
                const uint32_t x = (uint16_t)(int16_t)((ti.tx + 1) * 8);
                const uint32_t y = (uint16_t)(int16_t)(ti.ty * 8);
                const uint32_t wd = (uint16_t)((uint16_t)(nx.tx - ti.tx - 1) * 8u);
                span_val[t] = (uint64_t)x | ((uint64_t)y << 16) | ((uint64_t)wd << 32);
            }
        }
        span_flag[t] = has_span;
    }
    __syncwarp();
    const float acc0 = s_carry[wid][row] + excl;
    const float cov0 = fabsf(acc0 + a0);
    const float acc1 = acc0 + h0;
    const float cov1 = fabsf(acc1 + a1);
    const uint32_t al0 = f2u8(rmin(cov0 * 256.0f, 255.0f));
    const uint32_t al1 = f2u8(rmin(cov1 * 256.0f, 255.0f));
    reinterpret_cast<uint16_t*>(out_alpha + (size_t)t * 64)[lane] = (uint16_t)(al0 | (al1 << 8));
    if (out_cov) reinterpret_cast<float2*>(out_cov + (size_t)t * 64)[lane] = make_float2(cov0, cov1);
}

struct SpanIn {
    const uint32_t* flag;
    __device__ __forceinline__ uint32_t operator()(uint64_t t) const { return flag[t]; }
};
struct SpanOut {
    const uint64_t* val;
    const TileInfo* info;
    uint32_t n_tiles, n_rasters;
    uint32_t* xy;
    uint16_t* w;
    uint32_t* tile;
    uint32_t* raster_span_off;
    __device__ __forceinline__ void operator()(uint64_t t, uint32_t ex, uint32_t v) const {
        if (v) {
            const uint64_t s = val[t];
            xy[ex] = (uint32_t)(s & 0xffffffffu);
            w[ex] = (uint16_t)(s >> 32);
            tile[ex] = (uint32_t)t;
        }
        const int r = info[t].raster;
        if (t == 0 || info[t - 1].raster != r) raster_span_off[r] = ex;
        if (t + 1 == n_tiles) raster_span_off[n_rasters] = ex + v;
    }
};

template <class K>
static int tiles_impl(ochre_gpu_ctx* ctx, const ochre_batch* in, uint64_t E, cudaStream_t s, uint32_t* n_tiles_out,
                      uint32_t* n_spans_out) {
    DevScalars* ds = dev_scalars(ctx);
    const uint32_t R = in->n_rasters;
    OCHRE_CUDA_TRY(ctx->tile_head.ensure(E * 4));
    OCHRE_CUDA_TRY(ctx->scan_status.ensure(scan_tiles(E) * sizeof(ScanStatus<HeadScan>)));
    OCHRE_LAUNCH(ctx, "tile_head_scan", s, OCHRE_CUDA_TRY(launch_scan<HeadScan>(E, HeadIn<K>{ctx->keys.as<K>(), ctx->vals.as<uint32_t>()},
                                         HeadOut{ctx->tile_head.as<uint32_t>()}, OpHead{}, HeadScan{0u, 0u}, ctx->scan_status.p,
                                         &ds->ticket, reinterpret_cast<HeadScan*>(&ds->n_tiles), &ds->err, s)));
    int st = read_scalars(ctx, s);
    if (st != OCHRE_OK) return st;
    const uint32_t T = host_scalars(ctx)->n_tiles;
    *n_tiles_out = T;
    OCHRE_CUDA_TRY(ctx->tile_info.ensure((size_t)T * sizeof(TileInfo)));
    OCHRE_CUDA_TRY(ctx->tile_state.ensure((size_t)T * sizeof(TileState)));
    OCHRE_CUDA_TRY(ctx->span_flag.ensure((size_t)T * 4));
    OCHRE_CUDA_TRY(ctx->span_val.ensure((size_t)T * 8));
    OCHRE_CUDA_TRY(ctx->out_tile_xy.ensure((size_t)T * 4));
    OCHRE_CUDA_TRY(ctx->out_tile_alpha.ensure((size_t)T * 64));
    const bool want_cov = (ctx->flags & OCHRE_CTX_WANT_COV) != 0;
    if (want_cov) OCHRE_CUDA_TRY(ctx->out_tile_cov.ensure((size_t)T * 64 * 4));
    OCHRE_CUDA_TRY(ctx->out_raster_tile_off.ensure((size_t)(R + 1) * 4));
    OCHRE_CUDA_TRY(ctx->out_raster_span_off.ensure((size_t)(R + 1) * 4));
    OCHRE_LAUNCH(ctx, "tile_info", s, k_tile_info<K><<<(T + 255) / 256, 256, 0, s>>>(ctx->keys.as<K>(), ctx->vals.as<uint32_t>(), ctx->bins.as<BinRec>(),
                                                   ctx->tile_head.as<uint32_t>(), T, E, R, ctx->tile_info.as<TileInfo>(),
                                                   ctx->out_raster_tile_off.as<uint32_t>()));
    OCHRE_CUDA_TRY(cudaGetLastError());
    OCHRE_CUDA_TRY(cudaMemsetAsync(ctx->tile_state.p, 0, (size_t)T * sizeof(TileState), s));
    OCHRE_CUDA_TRY(cudaMemsetAsync(&ds->ticket, 0, 4, s));
    OCHRE_LAUNCH(ctx, "tile_coverage", s, k_tile_cov<<<(T + COV_WARPS - 1) / COV_WARPS, COV_WARPS * 32, 0, s>>>(
        ctx->vals.as<uint32_t>(), ctx->bins.as<BinRec>(), ctx->lines.as<float4>(), ctx->tile_info.as<TileInfo>(), T,
        ctx->tile_state.as<TileState>(), &ds->ticket, ctx->out_tile_xy.as<uint32_t>(),
        ctx->out_tile_alpha.as<uint8_t>(), want_cov ? ctx->out_tile_cov.as<float>() : nullptr,
        ctx->span_flag.as<uint32_t>(), ctx->span_val.as<uint64_t>(), &ds->err));
    OCHRE_CUDA_TRY(cudaGetLastError());
    // Spans: compact in tile order.  Capacity: at most one span per tile.
    OCHRE_CUDA_TRY(ctx->out_span_xy.ensure((size_t)T * 4));
    OCHRE_CUDA_TRY(ctx->out_span_w.ensure((size_t)T * 2));
    OCHRE_CUDA_TRY(ctx->out_span_tile.ensure((size_t)T * 4));
    OCHRE_CUDA_TRY(ctx->scan_status.ensure(scan_tiles(T) * sizeof(ScanStatus<uint32_t>)));
    OCHRE_LAUNCH(ctx, "span_scan", s, OCHRE_CUDA_TRY(launch_scan<uint32_t>(
        T, SpanIn{ctx->span_flag.as<uint32_t>()},
        SpanOut{ctx->span_val.as<uint64_t>(), ctx->tile_info.as<TileInfo>(), T, R, ctx->out_span_xy.as<uint32_t>(),
                ctx->out_span_w.as<uint16_t>(), ctx->out_span_tile.as<uint32_t>(),
                ctx->out_raster_span_off.as<uint32_t>()},
        OpSumU32{}, 0u, ctx->scan_status.p, &ds->ticket, &ds->n_spans, &ds->err, s)));
    st = read_scalars(ctx, s);
    if (st != OCHRE_OK) return st;
    *n_spans_out = host_scalars(ctx)->n_spans;
    ctx->stats.n_bins = host_scalars(ctx)->n_bins;
    return check_device_error(ctx);
}

int stage_tiles(ochre_gpu_ctx* ctx, const ochre_batch* in, uint64_t E, cudaStream_t s, uint32_t* n_tiles,
                uint32_t* n_spans) {
    *n_tiles = 0;
    *n_spans = 0;
    if (E == 0) return OCHRE_OK;
    return ctx->keys64 ? tiles_impl<uint64_t>(ctx, in, E, s, n_tiles, n_spans)
                       : tiles_impl<uint32_t>(ctx, in, E, s, n_tiles, n_spans);
}

}  // namespace ochre
