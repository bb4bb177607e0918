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
// order.  The tile-head scan also counts bins and sums crossing signs, so
// each tile's metadata and winding follow without a per-tile search.
// Coverage (row form) runs one warp per whole tile row (raster, tile_y) at a
// time, taken by ticket: chunk by chunk of TILES_PER_WARP tiles it adds the
// increments the emit walk stored for the chunk's bins into shared-memory
// accumulators, then walks the tiles left to right keeping the row carry in
// registers, so no carry ever crosses warps.  The block form gives each warp
// an aligned block of tiles and takes the carry from the block before by
// look-back.
#include <algorithm>

#include "common.cuh"
#include "internal.h"
#include "scan.cuh"

namespace ochre {

// Tile heads: the first bin entry of every run of equal keys.  The same
// scan counts bin entries and sums the crossing signs, so that every tile
// learns, at its head, how many bins and how much winding precede it.
struct HeadScan {
    uint32_t heads;
    uint32_t bins;
    int32_t w;
    uint32_t pad;
};
struct OpHead {
    __device__ __forceinline__ HeadScan operator()(HeadScan a, HeadScan b) const {
        return HeadScan{a.heads + b.heads, a.bins + b.bins, a.w + b.w, 0u};
    }
};
template <class K>
struct HeadIn {
    const K* keys;
    const uint32_t* vals;
    __device__ __forceinline__ HeadScan operator()(uint64_t i) const {
        const uint32_t v = vals[i];
        if (v & CROSS_TAG) return HeadScan{0u, 0u, (int32_t)(int8_t)(v & 0xffu), 0u};
        return HeadScan{(i == 0 || keys[i] != keys[i - 1]) ? 1u : 0u, 1u, 0, 0u};
    }
};
struct HeadOut {
    uint32_t* head;
    uint32_t* head_bins;
    int32_t* head_wind;
    __device__ __forceinline__ void operator()(uint64_t i, HeadScan ex, HeadScan v) const {
        if (v.heads) {
            head[ex.heads] = (uint32_t)i;
            head_bins[ex.heads] = ex.bins;
            head_wind[ex.heads] = ex.w;
        }
    }
};

// Tile metadata, one thread per tile.  The tile's bins are the bins between
// its head and the next tile's head; its winding (rasterizer.rs:219, 253-258:
// the signs of all crossings of its raster sorted before it, never reset)
// is the crossing-sign sum before its head minus that of all earlier
// rasters.
__global__ void k_tile_info(const uint32_t* __restrict__ vals, const BinRec* __restrict__ bins,
                            const uint32_t* __restrict__ head, const uint32_t* __restrict__ head_bins,
                            const int32_t* __restrict__ head_wind, const int32_t* __restrict__ raster_wbase,
                            const uint32_t* __restrict__ total_bins, uint32_t n_tiles, const uint32_t* n_dev,
                            uint32_t n_rasters, TileInfo* __restrict__ info, uint32_t* __restrict__ raster_tile_off,
                            const uint32_t* err) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    n_tiles = (uint32_t)dev_count(n_tiles, n_dev);
    // a wait of the sort gave up: the sorted entries are not valid indices
    if (t >= n_tiles || run_aborted(err)) return;
    const uint32_t h = head[t];
    const BinRec* rec = bins + vals[h];
    const int r = (int)rec->raster;
    TileInfo ti;
    ti.raster = r;
    ti.tx = div8((int)rec->x);
    ti.ty = div8((int)rec->y);
    ti.head = h;
    ti.nbins = (t + 1 < n_tiles ? head_bins[t + 1] : *total_bins) - head_bins[t];
    ti.wind = head_wind[t] - raster_wbase[r];
    bool ras_head = t == 0, row_head = t == 0;
    if (t > 0) {
        const BinRec* pr = bins + vals[head[t - 1]];
        ras_head = (int)pr->raster != r;
        row_head = ras_head || div8((int)pr->y) != ti.ty;
    }
    ti.row_head = row_head ? 1u : 0u;
    ti.pad = 0;
    info[t] = ti;
    if (ras_head) raster_tile_off[r] = t;
    if (t + 1 == n_tiles) raster_tile_off[n_rasters] = n_tiles;
}

// Shared-memory accumulators of one tile: 64 area cells, then 64 height
// cells, row-major; pixel rows 4-7 sit 4 floats further on, so the 128-bit
// row loads of eight lanes (rows 0-7 of one tile) hit distinct banks.
constexpr int ACC_H = 68;          // offset of the height cells
constexpr int ACC_STRIDE = 136;    // floats per tile
__device__ __forceinline__ int acc_idx(int cell) { return cell + ((cell >> 5) << 2); }

// Stage of one batch of a chunk's bins (per warp): first increment, first
// cell, packed steps / cell count / directions / accumulator slot, and the
// exclusive prefix of the cell counts.
struct BinStage {
    uint32_t inc[32];
    uint32_t xy[32];     // x (low 16 bits) | y (high 16 bits)
    uint32_t meta[32];   // steps (bits 0-15) | n (16-20) | dirs (21-22) | slot (23-27)
    uint32_t pre[33];
};

constexpr int CELL_UNROLL = 4;

// Adds the stored increments of the bins among entries e0 .. e1 - 1 (the
// entries of the chunk's nt tiles; crossing entries skipped) into the chunk's
// shared accumulators (rasterizer.rs:223-228).  The bins of a batch of 32
// entries are staged, then the warp's lanes take equal contiguous ranges of
// their cells, so every lane has cells whatever the bins' lengths; a cell's
// position follows from its bin's first cell and steps.
template <int CH>
__device__ __forceinline__ void add_chunk_increments(const uint32_t* __restrict__ vals, const BinRec* __restrict__ bins,
                                                     const float2* __restrict__ incs, uint32_t e0, uint32_t e1,
                                                     const uint32_t* s_head, int nt, float (*acc)[ACC_STRIDE],
                                                     BinStage& st) {
    const int lane = threadIdx.x & 31;
    for (uint32_t eb = e0; eb < e1; eb += 32) {
        const uint32_t e = eb + lane;
        uint32_t n = 0, inc = 0, xy = 0, meta = 0;
        if (e < e1) {
            const uint32_t v = vals[e];
            if (!(v & CROSS_TAG)) {
                const BinRec rec = bins[v];
                int slot = 0;
#pragma unroll
                for (int i = 1; i < CH; i++)
                    if (i < nt && s_head[i] <= e) slot = i;
                n = rec.n;
                inc = rec.inc;
                xy = (uint32_t)(uint16_t)rec.x | ((uint32_t)(uint16_t)rec.y << 16);
                meta = (uint32_t)rec.steps | (n << 16) | ((uint32_t)rec.dirs << 21) | ((uint32_t)slot << 23);
            }
        }
        uint32_t pre = n;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t o = __shfl_up_sync(0xffffffffu, pre, d);
            if (lane >= d) pre += o;
        }
        const uint32_t total = __shfl_sync(0xffffffffu, pre, 31);
        st.inc[lane] = inc;
        st.xy[lane] = xy;
        st.meta[lane] = meta;
        st.pre[lane] = pre - n;
        if (lane == 31) st.pre[32] = total;
        __syncwarp();
        // Each lane takes a contiguous range of the batch's cells: one search
        // for the bin of its first cell, then bin after bin; CELL_UNROLL
        // cells at a time, their increment loads all in flight before the
        // first is added.
        const uint32_t per = (total + 31u) >> 5;
        uint32_t c = lane * per;
        const uint32_t c_end = min(c + per, total);
        if (c < c_end) {
            int b = 0;
#pragma unroll
            for (int step = 16; step > 0; step >>= 1)
                if (st.pre[b + step] <= c) b += step;
            uint32_t base = st.pre[b], next = st.pre[b + 1], m = st.meta[b], sxy = st.xy[b], ib = st.inc[b];
            while (c < c_end) {
                float2 ah[CELL_UNROLL];
                int where[CELL_UNROLL];   // slot << 6 | cell, or -1
#pragma unroll
                for (int u = 0; u < CELL_UNROLL; u++) {
                    where[u] = -1;
                    ah[u] = make_float2(0.0f, 0.0f);
                    if (c < c_end) {
                        while (c >= next) {   // on to the next bin with cells
                            b++;
                            base = next;
                            next = st.pre[b + 1];
                            m = st.meta[b];
                            sxy = st.xy[b];
                            ib = st.inc[b];
                        }
                        const uint32_t k = c - base;
                        const uint32_t steps_before = m & ((1u << k) - 1u) & 0xffffu;
                        const int nx = __popc(steps_before), ny = (int)k - nx;
                        const int cx = (int)(sxy & 0xffffu) + ((m >> 21) & 1u ? -nx : nx);
                        const int cy = (int)(sxy >> 16) + ((m >> 22) & 1u ? -ny : ny);
                        where[u] = (int)(((m >> 23) & 31u) << 6) | ((cy & 7) << 3) | (cx & 7);
                        ah[u] = incs[ib + k];
                        c++;
                    }
                }
#pragma unroll
                for (int u = 0; u < CELL_UNROLL; u++) {
                    if (where[u] < 0) continue;
                    float* a = acc[where[u] >> 6];
                    const int cell = where[u] & 63;
                    atomicAdd(a + acc_idx(cell), ah[u].x);
                    atomicAdd(a + ACC_H + acc_idx(cell), ah[u].y);
                }
            }
        }
        __syncwarp();
    }
}

// Coverage, block form: one warp per aligned block of TILES_PER_WARP
// consecutive tiles (blocks may cross rows).  A block that continues a row
// from the previous block resolves its carry by decoupled look-back: blocks
// publish the row sums of their last row segment (taken by atomic ticket,
// bounded spins).  Used when there are too few tile rows to occupy the GPU
// with one warp per row; with many long rows the look-back chains grow long,
// and the row form below is used instead.
template <int CH>
__global__ void __launch_bounds__(128) k_tile_cov_blocks(
    const uint32_t* __restrict__ vals, const BinRec* __restrict__ bins, const float2* __restrict__ incs,
    const TileInfo* __restrict__ info, uint32_t n_tiles, const uint32_t* n_dev, TileBlockState* state,
    uint32_t* ticket, uint32_t* __restrict__ out_xy, uint8_t* __restrict__ out_alpha, float* __restrict__ out_cov,
    uint32_t* __restrict__ span_flag, uint64_t* __restrict__ span_val, uint32_t* err, bool cov_signed) {
    constexpr int WARPS = 4;
    // device-held count (graph replays): blocks past it end before publishing
    n_tiles = (uint32_t)dev_count(n_tiles, n_dev);
    // an earlier wait of the run gave up: the tile data is not valid (the
    // blocks' own waits then give up at once too)
    if (run_aborted(err)) return;
    // [tile][area cells | height cells], ACC_STRIDE floats per tile; see acc_idx
    __shared__ __align__(16) float s_acc[WARPS][CH][ACC_STRIDE];
    __shared__ uint32_t s_head[WARPS][CH];
    __shared__ TileInfo s_info[WARPS][CH + 1];
    __shared__ BinStage s_stage[WARPS];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t blk = 0;
    if (lane == 0) blk = atomicAdd(ticket, 1u);
    blk = __shfl_sync(0xffffffffu, blk, 0);
    const uint32_t t0 = blk * CH;
    if (t0 >= n_tiles) return;
    const int nt = (int)min((uint32_t)CH, n_tiles - t0);
    float (*acc)[ACC_STRIDE] = s_acc[wid];

    // tile metadata (one extra for the span test of the last tile)
    for (int i = lane; i <= nt; i += 32) {
        if (t0 + i < n_tiles) s_info[wid][i] = info[t0 + i];
        else s_info[wid][i].raster = -1;
    }
    for (int k = lane; k < nt * (ACC_STRIDE / 4); k += 32)
        reinterpret_cast<float4*>(acc[0])[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    __syncwarp();
    if (lane < nt) s_head[wid][lane] = s_info[wid][lane].head;
    __syncwarp();

    // The stored increments of every bin of the block (rasterizer.rs:97-106,
    // 223-228).  The block's entries are contiguous; crossing entries in
    // between are skipped.
    const uint32_t e0 = s_info[wid][0].head;
    const uint32_t e1 = s_info[wid][nt - 1].head + s_info[wid][nt - 1].nbins;
    add_chunk_increments<CH>(vals, bins, incs, e0, e1, s_head[wid], nt, acc, s_stage[wid]);

    // Each lane owns one pixel row of one tile: lane = 8 * g + y, four tiles
    // (g) per pass.
    const int y = lane & 7, g = lane >> 3;

    // Row sums of the block's last row segment -> publish (decoupled).
    int last_seg = 0;
    for (int i = nt - 1; i > 0; i--)
        if (s_info[wid][i].row_head) { last_seg = i; break; }
    const bool starts_mid_row = !s_info[wid][0].row_head;
    const bool one_segment = last_seg == 0 && starts_mid_row;
    float part = 0.0f;
    for (int i = last_seg + g; i < nt; i += 4) {
        const float4 h0 = *reinterpret_cast<const float4*>(&acc[i][ACC_H + acc_idx(8 * y)]);
        const float4 h1 = *reinterpret_cast<const float4*>(&acc[i][ACC_H + acc_idx(8 * y + 4)]);
        part += ((h0.x + h0.y) + (h0.z + h0.w)) + ((h1.x + h1.y) + (h1.z + h1.w));
    }
    part += __shfl_xor_sync(0xffffffffu, part, 8);
    part += __shfl_xor_sync(0xffffffffu, part, 16);   // every lane of row y holds its sum
    float seg[8];
#pragma unroll
    for (int r = 0; r < 8; r++) seg[r] = __shfl_sync(0xffffffffu, part, r);
    float carry_in = 0.0f;   // per lane: carry of this lane's pixel row
    if (lane == 0) {
        TileBlockState* me = state + blk;
        if (!one_segment) {
            for (int r = 0; r < 8; r++) st_relaxed(reinterpret_cast<uint32_t*>(&me->inc[r]), __float_as_uint(seg[r]));
            st_release(&me->flag, 2u);
        } else {
            for (int r = 0; r < 8; r++) st_relaxed(reinterpret_cast<uint32_t*>(&me->agg[r]), __float_as_uint(seg[r]));
            st_release(&me->flag, 1u);
        }
    }
    if (starts_mid_row) {
        // Warp-cooperative decoupled look-back over the preceding blocks, 32
        // per round (a long tile row spans many blocks): lane k inspects
        // block top - k; the nearest inclusive value ends the walk.
        float c[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        int64_t top = (int64_t)blk - 1;
        long long spins = 0;
        const long long poll_limit = spin_limit(err);
        while (top >= 0) {
            const int64_t j = top - lane;
            uint32_t f = 2u;   // before block 0: an inclusive zero
            if (j >= 0) f = ld_acquire(&state[j].flag);
            const uint32_t m2 = __ballot_sync(0xffffffffu, f == 2u);
            const int limit = m2 ? __ffs(m2) - 1 : 31;   // lanes [0, limit] are needed
            const uint32_t need = limit == 31 ? 0xffffffffu : ((1u << (limit + 1)) - 1u);
            if (__ballot_sync(0xffffffffu, f == 0u) & need) {
                if (wait_give_up_warp(spins, poll_limit, err)) break;
                if (spins > 16) __nanosleep(64);
                continue;
            }
            float v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            if (lane <= limit && j >= 0) {
                const float* src = f == 2u ? state[j].inc : state[j].agg;
#pragma unroll
                for (int r = 0; r < 8; r++) v[r] = __uint_as_float(ld_relaxed(reinterpret_cast<const uint32_t*>(src + r)));
            }
#pragma unroll
            for (int r = 0; r < 8; r++) {
#pragma unroll
                for (int d = 16; d > 0; d >>= 1) v[r] += __shfl_xor_sync(0xffffffffu, v[r], d);
                c[r] += v[r];
            }
            if (m2) break;
            top -= 32;
        }
        if (one_segment && lane == 0) {
            TileBlockState* me = state + blk;
            for (int r = 0; r < 8; r++)
                st_relaxed(reinterpret_cast<uint32_t*>(&me->inc[r]), __float_as_uint(c[r] + seg[r]));
            st_release(&me->flag, 2u);
        }
#pragma unroll
        for (int r = 0; r < 8; r++)
            if (y == r) carry_in = c[r];
    }

    // Tiles left to right (rasterizer.rs:232-250): along its row a lane adds
    // the cells in the reference's order; the carry into a tile is the carry
    // into the previous tile of the row plus that tile's row sum (reset at
    // each row start), a segmented scan over the four tiles of a pass.
    float carry_row = carry_in;   // carry into the pass's first tile, row y
    for (int i0 = 0; i0 < nt; i0 += 4) {
        const int i = i0 + g;
        const bool valid = i < nt;
        float a[8], h[8];
        if (valid) {
            const float4 a0 = *reinterpret_cast<const float4*>(&acc[i][acc_idx(8 * y)]);
            const float4 a1 = *reinterpret_cast<const float4*>(&acc[i][acc_idx(8 * y + 4)]);
            const float4 h0 = *reinterpret_cast<const float4*>(&acc[i][ACC_H + acc_idx(8 * y)]);
            const float4 h1 = *reinterpret_cast<const float4*>(&acc[i][ACC_H + acc_idx(8 * y + 4)]);
            a[0] = a0.x; a[1] = a0.y; a[2] = a0.z; a[3] = a0.w; a[4] = a1.x; a[5] = a1.y; a[6] = a1.z; a[7] = a1.w;
            h[0] = h0.x; h[1] = h0.y; h[2] = h0.z; h[3] = h0.w; h[4] = h1.x; h[5] = h1.y; h[6] = h1.z; h[7] = h1.w;
        } else {
#pragma unroll
            for (int c = 0; c < 8; c++) a[c] = h[c] = 0.0f;
        }
        const float rs = ((h[0] + h[1]) + (h[2] + h[3])) + ((h[4] + h[5]) + (h[6] + h[7]));
        const bool head = valid && i > 0 && s_info[wid][i].row_head;
        // segmented inclusive scan of rs over g (lanes 8 apart), then shifted
        // by one tile: ex = the sum of rs since the last row start before g
        float v = rs;
        bool f = head;
#pragma unroll
        for (int d = 8; d < 32; d <<= 1) {
            const float vo = __shfl_up_sync(0xffffffffu, v, d);
            const bool fo = __shfl_up_sync(0xffffffffu, f ? 1 : 0, d) != 0;
            if (lane >= d) {
                if (!f) v = vo + v;
                f = f || fo;
            }
        }
        float ex = __shfl_up_sync(0xffffffffu, v, 8);
        bool exf = __shfl_up_sync(0xffffffffu, f ? 1 : 0, 8) != 0;
        if (g == 0) {
            ex = 0.0f;
            exf = false;
        }
        const float carry = head ? 0.0f : (exf ? ex : carry_row + ex);
        carry_row = __shfl_sync(0xffffffffu, carry + rs, 24 + y);
        if (valid) {
            const uint32_t t = t0 + i;
            float accum = carry;
            uint32_t lo = 0, hi = 0;
            float cv[8];
#pragma unroll
            for (int c = 0; c < 8; c++) {
                const float sum = accum + a[c];
                const float cov = fabsf(sum);
                cv[c] = cov_signed ? sum : cov;
                const uint32_t al = f2u8(rmin(cov * 256.0f, 255.0f));
                if (c < 4) lo |= al << (8 * c); else hi |= al << (8 * (c - 4));
                accum = accum + h[c];
            }
            reinterpret_cast<uint2*>(out_alpha + (size_t)t * 64)[y] = make_uint2(lo, hi);
            if (out_cov) {
                float4* o = reinterpret_cast<float4*>(out_cov + (size_t)t * 64 + 8 * y);
                o[0] = make_float4(cv[0], cv[1], cv[2], cv[3]);
                o[1] = make_float4(cv[4], cv[5], cv[6], cv[7]);
            }
            if (y == 0) {
                const TileInfo& ti = s_info[wid][i];
                out_xy[t] = (uint32_t)(uint16_t)(int16_t)(ti.tx * 8) |
                            ((uint32_t)(uint16_t)(int16_t)(ti.ty * 8) << 16);
                const TileInfo& nx = s_info[wid][i + 1];
                uint32_t has_span = 0;
                if (nx.raster == ti.raster && nx.ty == ti.ty && nx.tx > ti.tx + 1 && ti.wind != 0) {
                    has_span = 1;
                    const uint32_t x = (uint16_t)(int16_t)((ti.tx + 1) * 8);
                    const uint32_t yy = (uint16_t)(int16_t)(ti.ty * 8);
                    const uint32_t wd = (uint16_t)((uint16_t)(nx.tx - ti.tx - 1) * 8u);
                    span_val[t] = (uint64_t)x | ((uint64_t)yy << 16) | ((uint64_t)wd << 32);
                }
                span_flag[t] = has_span;
            }
        }
    }
}

// Coverage, row form: one warp per tile row (see the file comment).
template <int CH>
__global__ void __launch_bounds__(128) k_tile_cov(
    const uint32_t* __restrict__ vals, const BinRec* __restrict__ bins, const float2* __restrict__ incs,
    const TileInfo* __restrict__ info, uint32_t n_tiles, const uint32_t* n_dev, const uint32_t* __restrict__ row_start,
    const uint32_t* __restrict__ n_rows_p, uint32_t* ticket, uint32_t* __restrict__ out_xy,
    uint8_t* __restrict__ out_alpha, float* __restrict__ out_cov, uint32_t* __restrict__ span_flag,
    uint64_t* __restrict__ span_val, const uint32_t* err, bool cov_signed) {
    constexpr int WARPS = 4;
    // an earlier wait of the run gave up: the tile data is not valid
    if (run_aborted(err)) return;
    __shared__ __align__(16) float s_acc[WARPS][CH][ACC_STRIDE];
    __shared__ uint32_t s_head[WARPS][CH];
    __shared__ TileInfo s_info[WARPS][CH + 1];
    __shared__ BinStage s_stage[WARPS];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    // lane = 8 * g + y: pixel row y of the g-th tile of a pass of four
    const int y = lane & 7, g = lane >> 3;
    const uint32_t n_rows = *n_rows_p;
    n_tiles = (uint32_t)dev_count(n_tiles, n_dev);
    float (*acc)[ACC_STRIDE] = s_acc[wid];

    for (;;) {
        // one tile row (raster, tile_y) per warp at a time: the row carry
        // (rasterizer.rs:243-250) never leaves the warp
        uint32_t k = 0;
        if (lane == 0) k = atomicAdd(ticket, 1u);
        k = __shfl_sync(0xffffffffu, k, 0);
        if (k >= n_rows) return;
        const uint32_t tb = row_start[k];
        const uint32_t te = k + 1 < n_rows ? row_start[k + 1] : n_tiles;
        float carry_row = 0.0f;   // carry into the next tile, pixel row y
        for (uint32_t t0 = tb; t0 < te; t0 += CH) {
            const int nt = (int)min((uint32_t)CH, te - t0);
            // tile metadata (one extra for the span test of the last tile)
            for (int i = lane; i <= nt; i += 32) {
                if (t0 + i < n_tiles) s_info[wid][i] = info[t0 + i];
                else s_info[wid][i].raster = -1;
            }
            for (int q = lane; q < nt * (ACC_STRIDE / 4); q += 32)
                reinterpret_cast<float4*>(acc[0])[q] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            __syncwarp();
            if (lane < nt) s_head[wid][lane] = s_info[wid][lane].head;
            __syncwarp();

            // The stored increments of every bin of the chunk
            // (rasterizer.rs:97-106, 223-228).  The chunk's entries are
            // contiguous; crossing entries in between are skipped.
            const uint32_t e0 = s_info[wid][0].head;
            const uint32_t e1 = s_info[wid][nt - 1].head + s_info[wid][nt - 1].nbins;
            add_chunk_increments<CH>(vals, bins, incs, e0, e1, s_head[wid], nt, acc, s_stage[wid]);

            // Tiles left to right (rasterizer.rs:232-250): along its row a lane
            // adds the cells in the reference's order; the carry into a tile is
            // the carry into the previous tile plus that tile's row sum.
            for (int i0 = 0; i0 < nt; i0 += 4) {
                const int i = i0 + g;
                const bool valid = i < nt;
                float a[8], h[8];
                if (valid) {
                    const float4 a0 = *reinterpret_cast<const float4*>(&acc[i][acc_idx(8 * y)]);
                    const float4 a1 = *reinterpret_cast<const float4*>(&acc[i][acc_idx(8 * y + 4)]);
                    const float4 h0 = *reinterpret_cast<const float4*>(&acc[i][ACC_H + acc_idx(8 * y)]);
                    const float4 h1 = *reinterpret_cast<const float4*>(&acc[i][ACC_H + acc_idx(8 * y + 4)]);
                    a[0] = a0.x; a[1] = a0.y; a[2] = a0.z; a[3] = a0.w; a[4] = a1.x; a[5] = a1.y; a[6] = a1.z; a[7] = a1.w;
                    h[0] = h0.x; h[1] = h0.y; h[2] = h0.z; h[3] = h0.w; h[4] = h1.x; h[5] = h1.y; h[6] = h1.z; h[7] = h1.w;
                } else {
#pragma unroll
                    for (int c = 0; c < 8; c++) a[c] = h[c] = 0.0f;
                }
                const float rs = ((h[0] + h[1]) + (h[2] + h[3])) + ((h[4] + h[5]) + (h[6] + h[7]));
                // exclusive sum of rs over the tiles of the pass before this one
                float v = rs;
#pragma unroll
                for (int d = 8; d < 32; d <<= 1) {
                    const float vo = __shfl_up_sync(0xffffffffu, v, d);
                    if (lane >= d) v = vo + v;
                }
                float ex = __shfl_up_sync(0xffffffffu, v, 8);
                if (g == 0) ex = 0.0f;
                const float carry = carry_row + ex;
                carry_row = __shfl_sync(0xffffffffu, carry + rs, 24 + y);
                if (valid) {
                    const uint32_t t = t0 + i;
                    float accum = carry;
                    uint32_t lo = 0, hi = 0;
                    float cv[8];
#pragma unroll
                    for (int c = 0; c < 8; c++) {
                        const float sum = accum + a[c];
                        const float cov = fabsf(sum);
                        cv[c] = cov_signed ? sum : cov;
                        const uint32_t al = f2u8(rmin(cov * 256.0f, 255.0f));
                        if (c < 4) lo |= al << (8 * c); else hi |= al << (8 * (c - 4));
                        accum = accum + h[c];
                    }
                    reinterpret_cast<uint2*>(out_alpha + (size_t)t * 64)[y] = make_uint2(lo, hi);
                    if (out_cov) {
                        float4* o = reinterpret_cast<float4*>(out_cov + (size_t)t * 64 + 8 * y);
                        o[0] = make_float4(cv[0], cv[1], cv[2], cv[3]);
                        o[1] = make_float4(cv[4], cv[5], cv[6], cv[7]);
                    }
                    if (y == 0) {
                        const TileInfo& ti = s_info[wid][i];
                        out_xy[t] = (uint32_t)(uint16_t)(int16_t)(ti.tx * 8) |
                                    ((uint32_t)(uint16_t)(int16_t)(ti.ty * 8) << 16);
                        const TileInfo& nx = s_info[wid][i + 1];
                        uint32_t has_span = 0;
                        if (nx.raster == ti.raster && nx.ty == ti.ty && nx.tx > ti.tx + 1 && ti.wind != 0) {
                            has_span = 1;
                            const uint32_t x = (uint16_t)(int16_t)((ti.tx + 1) * 8);
                            const uint32_t yy = (uint16_t)(int16_t)(ti.ty * 8);
                            const uint32_t wd = (uint16_t)((uint16_t)(nx.tx - ti.tx - 1) * 8u);
                            span_val[t] = (uint64_t)x | ((uint64_t)yy << 16) | ((uint64_t)wd << 32);
                        }
                        span_flag[t] = has_span;
                    }
                }
            }
            __syncwarp();
        }
    }
}

// Row starts: the tiles that begin a (raster, tile_y) row, compacted.
struct RowIn {
    const TileInfo* info;
    __device__ __forceinline__ uint32_t operator()(uint64_t t) const { return info[t].row_head; }
};
struct RowOut {
    uint32_t* row_start;
    __device__ __forceinline__ void operator()(uint64_t t, uint32_t ex, uint32_t v) const {
        if (v) row_start[ex] = (uint32_t)t;
    }
};

struct SpanIn {
    const uint32_t* flag;
    __device__ __forceinline__ uint32_t operator()(uint64_t t) const { return flag[t]; }
};
struct SpanOut {
    const uint64_t* val;
    const TileInfo* info;
    uint32_t n_tiles, n_rasters;
    const uint32_t* n_dev;   // device-held tile count (graph replays), else null
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
        if (t + 1 == dev_count(n_tiles, n_dev)) raster_span_off[n_rasters] = ex + v;
    }
};

// One launch of the coverage kernel with TPW tiles per warp (4 warps per CTA).
// Coverage launch.  With at least ROW_FORM_MIN_ROWS_PER_SM tile rows per SM
// the row form runs (persistent warps taking rows by ticket); otherwise the
// block form, whose look-back chains stay short when rows are few.
constexpr uint32_t ROW_FORM_MIN_ROWS_PER_SM = 64;

template <int TPW>
static void launch_tile_cov(ochre_gpu_ctx* ctx, uint32_t T, uint32_t n_rows, bool want_cov, cudaStream_t s) {
    DevScalars* ds = dev_scalars(ctx);
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    cudaMemsetAsync(&ds->ticket, 0, 4, s);
    float* cov = want_cov ? ctx->out_tile_cov.as<float>() : nullptr;
    // graph replays: T is the capacity and n_rows the planned row count; the
    // kernels read both counts on the device
    const uint32_t* t_dev = ctx->plan ? &ds->n_tiles : nullptr;
    const bool row_form = ctx->tune_chain_coverage_form == 2 ||
                          (ctx->tune_chain_coverage_form == 0 && n_rows >= ROW_FORM_MIN_ROWS_PER_SM * (uint32_t)sms);
    if (row_form) {
        // no more warps than rows, nor than the GPU keeps resident (16 CTAs of 4 warps per SM)
        const uint32_t ctas = (uint32_t)std::min<uint64_t>(((uint64_t)n_rows + 3) / 4, (uint64_t)sms * 16);
        k_tile_cov<TPW><<<ctas, 128, 0, s>>>(
            ctx->vals.as<uint32_t>(), ctx->bins.as<BinRec>(), ctx->incs.as<float2>(), ctx->tile_info.as<TileInfo>(),
            T, t_dev, ctx->tile_row_start.as<uint32_t>(), &ds->n_rows, &ds->ticket, ctx->out_tile_xy.as<uint32_t>(),
            ctx->out_tile_alpha.as<uint8_t>(), cov, ctx->span_flag.as<uint32_t>(), ctx->span_val.as<uint64_t>(),
            &ds->err, ctx->cov_signed);
    } else {
        const uint32_t blocks = (T + TPW - 1) / TPW;
        cudaMemsetAsync(ctx->tile_state.p, 0, (size_t)blocks * sizeof(TileBlockState), s);
        k_tile_cov_blocks<TPW><<<(blocks + 3) / 4, 128, 0, s>>>(
            ctx->vals.as<uint32_t>(), ctx->bins.as<BinRec>(), ctx->incs.as<float2>(), ctx->tile_info.as<TileInfo>(),
            T, t_dev, ctx->tile_state.as<TileBlockState>(), &ds->ticket, ctx->out_tile_xy.as<uint32_t>(),
            ctx->out_tile_alpha.as<uint8_t>(), cov, ctx->span_flag.as<uint32_t>(), ctx->span_val.as<uint64_t>(),
            &ds->err, ctx->cov_signed);
    }
}

template <class K>
static int tiles_impl(ochre_gpu_ctx* ctx, const ochre_batch* in, uint64_t E, cudaStream_t s, uint32_t* n_tiles_out,
                      uint32_t* n_spans_out) {
    DevScalars* ds = dev_scalars(ctx);
    const uint32_t R = in->n_rasters;
    OCHRE_CUDA_TRY(ctx->tile_head.ensure(E * 4));
    OCHRE_CUDA_TRY(ctx->tile_head_bins.ensure(E * 4));
    OCHRE_CUDA_TRY(ctx->tile_head_wind.ensure(E * 4));
    OCHRE_CUDA_TRY(ctx->scan_status.ensure(scan_tiles(E) * sizeof(ScanStatus<HeadScan>)));
    // graph replays: E and T are capacities, the counts stay on the device
    const GraphPlan* plan = ctx->plan;
    const uint32_t* t_dev = plan ? &ds->n_tiles : nullptr;
    OCHRE_LAUNCH(ctx, "tile_head_scan", s,
                 OCHRE_CUDA_TRY(launch_scan<HeadScan>(
                     E, HeadIn<K>{ctx->keys.as<K>(), ctx->vals.as<uint32_t>()},
                     HeadOut{ctx->tile_head.as<uint32_t>(), ctx->tile_head_bins.as<uint32_t>(),
                             ctx->tile_head_wind.as<int32_t>()},
                     OpHead{}, HeadScan{0u, 0u, 0, 0u}, ctx->scan_status.p, &ds->ticket,
                     reinterpret_cast<HeadScan*>(&ds->n_tiles), &ds->err, s, plan ? &ds->n_entries : nullptr)));
    int st = OCHRE_OK;
    uint32_t T;
    if (plan) {
        OCHRE_LAUNCH(ctx, "plan_tiles", s, OCHRE_CUDA_TRY(launch_plan_cap(ctx, &ds->n_tiles, plan->tiles, s)));
        T = plan->tiles;
    } else {
        st = read_scalars(ctx, s);
        if (st != OCHRE_OK) return st;
        st = check_device_error(ctx);
        if (st != OCHRE_OK) return st;
        T = host_scalars(ctx)->n_tiles;
    }
    *n_tiles_out = T;
    OCHRE_CUDA_TRY(ctx->tile_info.ensure((size_t)T * sizeof(TileInfo)));
    OCHRE_CUDA_TRY(ctx->tile_row_start.ensure((size_t)T * 4));
    OCHRE_CUDA_TRY(ctx->tile_state.ensure((size_t)((T + 3) / 4) * sizeof(TileBlockState)));
    OCHRE_CUDA_TRY(ctx->span_flag.ensure((size_t)T * 4));
    OCHRE_CUDA_TRY(ctx->span_val.ensure((size_t)T * 8));
    OCHRE_CUDA_TRY(ctx->out_tile_xy.ensure((size_t)T * 4));
    OCHRE_CUDA_TRY(ctx->out_tile_alpha.ensure((size_t)T * 64));
    const bool want_cov = (ctx->flags & OCHRE_CTX_WANT_COV) != 0;
    if (want_cov) OCHRE_CUDA_TRY(ctx->out_tile_cov.ensure((size_t)T * 64 * 4));
    OCHRE_CUDA_TRY(ctx->out_raster_tile_off.ensure((size_t)(R + 1) * 4));
    OCHRE_CUDA_TRY(ctx->out_raster_span_off.ensure((size_t)(R + 1) * 4));
    if (T)
        OCHRE_LAUNCH(ctx, "tile_info", s,
                     k_tile_info<<<(T + 255) / 256, 256, 0, s>>>(
                         ctx->vals.as<uint32_t>(), ctx->bins.as<BinRec>(), ctx->tile_head.as<uint32_t>(),
                         ctx->tile_head_bins.as<uint32_t>(), ctx->tile_head_wind.as<int32_t>(),
                         ctx->raster_wbase.as<int32_t>(), &ds->n_bins, T, t_dev, R, ctx->tile_info.as<TileInfo>(),
                         ctx->out_raster_tile_off.as<uint32_t>(), &ds->err));
    OCHRE_CUDA_TRY(cudaGetLastError());
    if (T) {
        OCHRE_CUDA_TRY(ctx->scan_status.ensure(scan_tiles(T) * sizeof(ScanStatus<uint32_t>)));
        OCHRE_LAUNCH(ctx, "tile_row_scan", s,
                     OCHRE_CUDA_TRY(launch_scan<uint32_t>(
                         T, RowIn{ctx->tile_info.as<TileInfo>()}, RowOut{ctx->tile_row_start.as<uint32_t>()},
                         OpSumU32{}, 0u, ctx->scan_status.p, &ds->ticket, &ds->n_rows, &ds->err, s, t_dev)));
    }
    uint32_t n_rows;
    if (plan) {
        n_rows = plan->rows;
    } else {
        st = read_scalars(ctx, s);
        if (st != OCHRE_OK) return st;
        st = check_device_error(ctx);
        if (st != OCHRE_OK) return st;
        n_rows = host_scalars(ctx)->n_rows;
    }
    switch (ctx->tune_chain_tiles_per_warp) {
    case 4: OCHRE_LAUNCH(ctx, "tile_coverage", s, launch_tile_cov<4>(ctx, T, n_rows, want_cov, s)); break;
    case 8: OCHRE_LAUNCH(ctx, "tile_coverage", s, launch_tile_cov<8>(ctx, T, n_rows, want_cov, s)); break;
    case 16: OCHRE_LAUNCH(ctx, "tile_coverage", s, launch_tile_cov<16>(ctx, T, n_rows, want_cov, s)); break;
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
                     SpanOut{ctx->span_val.as<uint64_t>(), ctx->tile_info.as<TileInfo>(), T, R, t_dev,
                             ctx->out_span_xy.as<uint32_t>(), ctx->out_span_w.as<uint16_t>(),
                             ctx->out_span_tile.as<uint32_t>(), ctx->out_raster_span_off.as<uint32_t>()},
                     OpSumU32{}, 0u, ctx->scan_status.p, &ds->ticket, &ds->n_spans, &ds->err, s, t_dev)));
    if (plan) {
        *n_spans_out = 0;   // on the device; read after the replay
        return OCHRE_OK;
    }
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
