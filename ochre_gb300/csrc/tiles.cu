// Stage 4: sorted entries -> 8x8 alpha tiles and solid spans.
//
// Reference: the tile loop of finish (rasterizer.rs:213-267):
//   * scatter-add area/height of every increment of a tile (:223-228);
//   * alpha = min(|accum + area| * 256, 255) as u8 with accum the running
//     sum of heights along the pixel row, seeded by the carry `prev` from
//     the tiles to the left on the same tile row (:232-239, 243-250);
//   * a span between this tile and the next one on the row when there is a
//     gap and the running tile-row-crossing winding (never reset, so a
//     prefix over the whole raster) is nonzero (:252-265).
//
// Tiles are numbered in sorted order, which is the reference's callback
// order.  The winding is a segmented (per raster) scan fused with the pass
// that gathers each tile's metadata.  Coverage runs one warp per aligned
// block of TILES_PER_WARP consecutive tiles: the warp replays the block's
// bins into shared-memory accumulators, then walks its tiles left to right
// keeping the row carry in registers (reset at each row start).  Only a
// block whose first tile continues a row from the previous block needs a
// carry from outside: blocks publish the row sums of their last row segment
// and resolve the carry by decoupled look-back over earlier blocks (taken by
// atomic ticket, bounded spins).
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

// Tile metadata + winding.  The winding value of a tile is the sum of the
// signs of all crossings of its raster whose key is <= the tile's key; each
// tile contributes the crossings sorted between the previous tile and itself,
// and the scan is segmented by raster: (w, head) o (w', head') =
// head' ? (w', 1) : (w + w', head).
struct WindScan {
    int32_t w;
    uint32_t head;
};
struct OpWind {
    __device__ __forceinline__ WindScan operator()(WindScan a, WindScan b) const {
        return b.head ? b : WindScan{a.w + b.w, a.head};
    }
};
template <class K>
struct InfoIn {
    const K* keys;
    const uint32_t* vals;
    const BinRec* bins;
    const uint32_t* head;
    uint32_t n_tiles;
    uint64_t n_entries;
    uint32_t n_rasters;
    TileInfo* info;
    uint32_t* raster_tile_off;
    __device__ WindScan operator()(uint64_t t64) const {
        const uint32_t t = (uint32_t)t64;
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
        bool ras_head = t == 0, row_head = t == 0;
        if (t > 0) {
            const BinRec* pr = bins + vals[head[t - 1]];
            ras_head = (int)pr->raster != r;
            row_head = ras_head || div8((int)pr->y) != ti.ty;
        }
        ti.row_head = row_head ? 1u : 0u;
        ti.wind = 0;
        ti.pad = 0;
        info[t] = ti;
        if (ras_head) raster_tile_off[r] = t;
        if (t + 1 == n_tiles) raster_tile_off[n_rasters] = n_tiles;
        return WindScan{w, ras_head ? 1u : 0u};
    }
};
struct InfoOut {
    TileInfo* info;
    __device__ __forceinline__ void operator()(uint64_t t, WindScan ex, WindScan v) const {
        info[t].wind = OpWind{}(ex, v).w;
    }
};

template <int CH>
__global__ void __launch_bounds__(128) k_tile_cov(
    const uint32_t* __restrict__ vals, const BinRec* __restrict__ bins, const float4* __restrict__ lines,
    const TileInfo* __restrict__ info, uint32_t n_tiles, TileBlockState* state, uint32_t* ticket,
    uint32_t* __restrict__ out_xy, uint8_t* __restrict__ out_alpha, float* __restrict__ out_cov,
    uint32_t* __restrict__ span_flag, uint64_t* __restrict__ span_val, uint32_t* err, bool cov_signed) {
    constexpr int WARPS = 4;
    __shared__ float s_acc[WARPS][CH][128];   // [tile][0..63 area, 64..127 height]
    __shared__ uint32_t s_head[WARPS][CH];
    __shared__ TileInfo s_info[WARPS][CH + 1];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t blk = 0;
    if (lane == 0) blk = atomicAdd(ticket, 1u);
    blk = __shfl_sync(0xffffffffu, blk, 0);
    const uint32_t t0 = blk * CH;
    if (t0 >= n_tiles) return;
    const int nt = (int)min((uint32_t)CH, n_tiles - t0);
    float (*acc)[128] = s_acc[wid];

    // tile metadata (one extra for the span test of the last tile)
    for (int i = lane; i <= nt; i += 32) {
        if (t0 + i < n_tiles) s_info[wid][i] = info[t0 + i];
        else s_info[wid][i].raster = -1;
    }
    for (int i = 0; i < nt; i++) {
        acc[i][lane] = 0.0f;
        acc[i][lane + 32] = 0.0f;
        acc[i][lane + 64] = 0.0f;
        acc[i][lane + 96] = 0.0f;
    }
    __syncwarp();
    if (lane < nt) s_head[wid][lane] = s_info[wid][lane].head;
    __syncwarp();

    // Replay every bin of the block (rasterizer.rs:97-106, 223-228).  The
    // block's entries are contiguous; crossing entries in between are skipped.
    const uint32_t e0 = s_info[wid][0].head;
    const uint32_t e1 = s_info[wid][nt - 1].head + s_info[wid][nt - 1].nbins;
    for (uint32_t e = e0 + lane; e < e1; e += 32) {
        const uint32_t v = vals[e];
        if (v & CROSS_TAG) continue;
        int slot = 0;
#pragma unroll
        for (int i = 1; i < CH; i++)
            if (i < nt && s_head[wid][i] <= e) slot = i;
        const BinRec rec = bins[v];
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
        float* a = acc[slot];
        for (uint32_t k = 0;; k++) {
            float area, height;
            walk_increment(w, s, area, height);
            const int cell = ((s.y & 7) << 3) | (s.x & 7);
            atomicAdd(a + cell, area);
            atomicAdd(a + 64 + cell, height);
            if (k + 1 >= rec.n) break;
            walk_step(w, s);
        }
    }
    __syncwarp();

    // lane -> cells 2*lane, 2*lane+1 of pixel row lane/4
    const int row = lane >> 2;
    const int c0 = 2 * lane;

    // Row sums of the block's last row segment -> publish (decoupled).
    int last_seg = 0;
    for (int i = nt - 1; i > 0; i--)
        if (s_info[wid][i].row_head) { last_seg = i; break; }
    const bool starts_mid_row = !s_info[wid][0].row_head;
    const bool one_segment = last_seg == 0 && starts_mid_row;
    float part = 0.0f;
    for (int i = last_seg; i < nt; i++) part += acc[i][64 + c0] + acc[i][64 + c0 + 1];
    part += __shfl_xor_sync(0xffffffffu, part, 1);
    part += __shfl_xor_sync(0xffffffffu, part, 2);   // all 4 lanes of a row hold its sum
    float seg[8];
#pragma unroll
    for (int y = 0; y < 8; y++) seg[y] = __shfl_sync(0xffffffffu, part, 4 * y);
    float carry_in = 0.0f;   // per lane: carry of this lane's pixel row
    if (lane == 0) {
        TileBlockState* me = state + blk;
        if (!one_segment) {
            for (int y = 0; y < 8; y++) st_relaxed(reinterpret_cast<uint32_t*>(&me->inc[y]), __float_as_uint(seg[y]));
            st_release(&me->flag, 2u);
        } else {
            for (int y = 0; y < 8; y++) st_relaxed(reinterpret_cast<uint32_t*>(&me->agg[y]), __float_as_uint(seg[y]));
            st_release(&me->flag, 1u);
        }
    }
    if (starts_mid_row) {
        float c[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        if (lane == 0) {
            int64_t j = (int64_t)blk - 1;
            long long spins = 0;
            while (j >= 0) {
                const uint32_t f = ld_acquire(&state[j].flag);
                if (f == 0u) {
                    if (++spins > SPIN_LIMIT) { atomicOr(err, ERR_TIMEOUT); break; }
                    if (spins > 64) __nanosleep(64);
                    continue;
                }
                const float* src = f == 2u ? state[j].inc : state[j].agg;
                for (int y = 0; y < 8; y++)
                    c[y] = __uint_as_float(ld_relaxed(reinterpret_cast<const uint32_t*>(src + y))) + c[y];
                if (f == 2u) break;
                --j;
            }
            if (one_segment) {
                TileBlockState* me = state + blk;
                for (int y = 0; y < 8; y++)
                    st_relaxed(reinterpret_cast<uint32_t*>(&me->inc[y]), __float_as_uint(c[y] + seg[y]));
                st_release(&me->flag, 2u);
            }
        }
#pragma unroll
        for (int y = 0; y < 8; y++) {
            const float v = __shfl_sync(0xffffffffu, c[y], 0);
            if (row == y) carry_in = v;
        }
    }

    // Tiles left to right, carry in registers (rasterizer.rs:232-250).
    float carry = carry_in;
    for (int i = 0; i < nt; i++) {
        const TileInfo& ti = s_info[wid][i];
        if (i > 0 && ti.row_head) carry = 0.0f;
        const float a0 = acc[i][c0], a1 = acc[i][c0 + 1];
        const float h0 = acc[i][64 + c0], h1 = acc[i][64 + c0 + 1];
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
        const float rowsum = __shfl_sync(0xffffffffu, incl, (lane & ~3) | 3);
        const float acc0 = carry + excl;
        const float sum0 = acc0 + a0;
        const float cov0 = fabsf(sum0);
        const float acc1 = acc0 + h0;
        const float sum1 = acc1 + a1;
        const float cov1 = fabsf(sum1);
        const uint32_t t = t0 + i;
        const uint32_t al0 = f2u8(rmin(cov0 * 256.0f, 255.0f));
        const uint32_t al1 = f2u8(rmin(cov1 * 256.0f, 255.0f));
        reinterpret_cast<uint16_t*>(out_alpha + (size_t)t * 64)[lane] = (uint16_t)(al0 | (al1 << 8));
        if (out_cov)
            reinterpret_cast<float2*>(out_cov + (size_t)t * 64)[lane] =
                cov_signed ? make_float2(sum0, sum1) : make_float2(cov0, cov1);
        carry = carry + rowsum;
        if (lane == i) {
            out_xy[t] = (uint32_t)(uint16_t)(int16_t)(ti.tx * 8) | ((uint32_t)(uint16_t)(int16_t)(ti.ty * 8) << 16);
            const TileInfo& nx = s_info[wid][i + 1];
            uint32_t has_span = 0;
            if (nx.raster == ti.raster && nx.ty == ti.ty && nx.tx > ti.tx + 1 && ti.wind != 0) {
                has_span = 1;
                const uint32_t x = (uint16_t)(int16_t)((ti.tx + 1) * 8);
                const uint32_t y = (uint16_t)(int16_t)(ti.ty * 8);
                const uint32_t wd = (uint16_t)((uint16_t)(nx.tx - ti.tx - 1) * 8u);
                span_val[t] = (uint64_t)x | ((uint64_t)y << 16) | ((uint64_t)wd << 32);
            }
            span_flag[t] = has_span;
        }
    }
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

// One launch of the coverage kernel with TPW tiles per warp (4 warps per CTA).
template <int TPW>
static void launch_tile_cov(ochre_gpu_ctx* ctx, uint32_t T, bool want_cov, cudaStream_t s) {
    DevScalars* ds = dev_scalars(ctx);
    const uint32_t blocks = (T + TPW - 1) / TPW;
    cudaMemsetAsync(ctx->tile_state.p, 0, (size_t)blocks * sizeof(TileBlockState), s);
    cudaMemsetAsync(&ds->ticket, 0, 4, s);
    k_tile_cov<TPW><<<(blocks + 3) / 4, 128, 0, s>>>(
        ctx->vals.as<uint32_t>(), ctx->bins.as<BinRec>(), ctx->lines.as<float4>(), ctx->tile_info.as<TileInfo>(), T,
        ctx->tile_state.as<TileBlockState>(), &ds->ticket, ctx->out_tile_xy.as<uint32_t>(),
        ctx->out_tile_alpha.as<uint8_t>(), want_cov ? ctx->out_tile_cov.as<float>() : nullptr,
        ctx->span_flag.as<uint32_t>(), ctx->span_val.as<uint64_t>(), &ds->err, ctx->cov_signed);
}

template <class K>
static int tiles_impl(ochre_gpu_ctx* ctx, const ochre_batch* in, uint64_t E, cudaStream_t s, uint32_t* n_tiles_out,
                      uint32_t* n_spans_out) {
    DevScalars* ds = dev_scalars(ctx);
    const uint32_t R = in->n_rasters;
    OCHRE_CUDA_TRY(ctx->tile_head.ensure(E * 4));
    OCHRE_CUDA_TRY(ctx->scan_status.ensure(scan_tiles(E) * sizeof(ScanStatus<HeadScan>)));
    OCHRE_LAUNCH(ctx, "tile_head_scan", s,
                 OCHRE_CUDA_TRY(launch_scan<HeadScan>(E, HeadIn<K>{ctx->keys.as<K>(), ctx->vals.as<uint32_t>()},
                                                      HeadOut{ctx->tile_head.as<uint32_t>()}, OpHead{},
                                                      HeadScan{0u, 0u}, ctx->scan_status.p, &ds->ticket,
                                                      reinterpret_cast<HeadScan*>(&ds->n_tiles), &ds->err, s)));
    int st = read_scalars(ctx, s);
    if (st != OCHRE_OK) return st;
    const uint32_t T = host_scalars(ctx)->n_tiles;
    *n_tiles_out = T;
    const uint32_t blocks = (T + 3) / 4;   // >= blocks of the smallest tiles-per-warp shape
    OCHRE_CUDA_TRY(ctx->tile_info.ensure((size_t)T * sizeof(TileInfo)));
    OCHRE_CUDA_TRY(ctx->tile_state.ensure((size_t)blocks * sizeof(TileBlockState)));
    OCHRE_CUDA_TRY(ctx->span_flag.ensure((size_t)T * 4));
    OCHRE_CUDA_TRY(ctx->span_val.ensure((size_t)T * 8));
    OCHRE_CUDA_TRY(ctx->out_tile_xy.ensure((size_t)T * 4));
    OCHRE_CUDA_TRY(ctx->out_tile_alpha.ensure((size_t)T * 64));
    const bool want_cov = (ctx->flags & OCHRE_CTX_WANT_COV) != 0;
    if (want_cov) OCHRE_CUDA_TRY(ctx->out_tile_cov.ensure((size_t)T * 64 * 4));
    OCHRE_CUDA_TRY(ctx->out_raster_tile_off.ensure((size_t)(R + 1) * 4));
    OCHRE_CUDA_TRY(ctx->out_raster_span_off.ensure((size_t)(R + 1) * 4));
    OCHRE_CUDA_TRY(ctx->scan_status.ensure(scan_tiles(T) * sizeof(ScanStatus<WindScan>)));
    OCHRE_LAUNCH(ctx, "tile_info_wind_scan", s,
                 OCHRE_CUDA_TRY(launch_scan<WindScan>(
                     T,
                     InfoIn<K>{ctx->keys.as<K>(), ctx->vals.as<uint32_t>(), ctx->bins.as<BinRec>(),
                               ctx->tile_head.as<uint32_t>(), T, E, R, ctx->tile_info.as<TileInfo>(),
                               ctx->out_raster_tile_off.as<uint32_t>()},
                     InfoOut{ctx->tile_info.as<TileInfo>()}, OpWind{}, WindScan{0, 0u}, ctx->scan_status.p,
                     &ds->ticket, static_cast<WindScan*>(nullptr), &ds->err, s)));
    switch (ctx->tune_chain_tiles_per_warp) {
    case 4: OCHRE_LAUNCH(ctx, "tile_coverage", s, launch_tile_cov<4>(ctx, T, want_cov, s)); break;
    case 8: OCHRE_LAUNCH(ctx, "tile_coverage", s, launch_tile_cov<8>(ctx, T, want_cov, s)); break;
    case 16: OCHRE_LAUNCH(ctx, "tile_coverage", s, launch_tile_cov<16>(ctx, T, want_cov, s)); break;
    default: return OCHRE_E_INVALID;
    }
    OCHRE_CUDA_TRY(cudaGetLastError());
    // Spans: compact in tile order.  Capacity: at most one span per tile.
    OCHRE_CUDA_TRY(ctx->out_span_xy.ensure((size_t)T * 4));
    OCHRE_CUDA_TRY(ctx->out_span_w.ensure((size_t)T * 2));
    OCHRE_CUDA_TRY(ctx->out_span_tile.ensure((size_t)T * 4));
    OCHRE_CUDA_TRY(ctx->scan_status.ensure(scan_tiles(T) * sizeof(ScanStatus<uint32_t>)));
    OCHRE_LAUNCH(ctx, "span_scan", s,
                 OCHRE_CUDA_TRY(launch_scan<uint32_t>(
                     T, SpanIn{ctx->span_flag.as<uint32_t>()},
                     SpanOut{ctx->span_val.as<uint64_t>(), ctx->tile_info.as<TileInfo>(), T, R,
                             ctx->out_span_xy.as<uint32_t>(), ctx->out_span_w.as<uint16_t>(),
                             ctx->out_span_tile.as<uint32_t>(), ctx->out_raster_span_off.as<uint32_t>()},
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
