// Stage 2: line segments -> sort entries (pixel DDA binning).
//
// Reference: Rasterizer::line_to (rasterizer.rs:72-140) and the run-length
// binning of finish (rasterizer.rs:185-208).
//
// Every line is walked by one thread with the reference's exact serial
// recurrence.  Invariant used to make lines independent: at the start of
// every line_to, tile_y_prev == div_euclid(floor(last.y) as i16, 8) — move_to
// sets it that way (rasterizer.rs:68) and every walk ends by snapping to
// floor(point) and updating tile_y_prev for that cell (rasterizer.rs:118-131).
//
// A walk stores the increment (area, height) of every cell it visits once,
// line by line (the count pass gives each line its offset), and produces two
// kinds of sort entries:
//   * a *bin* per run of consecutive increment cells in one tile
//     (value = entry index; the BinRec at that index holds the run's first
//     increment, first cell and steps, so the tile kernel finds every cell's
//     increment without walking again);
//   * a *crossing* per tile-row change (rasterizer.rs:123-131)
//     (value = CROSS_TAG | raster << 8 | sign byte).
// Keys order entries by (raster, tile_y, tile_x, kind) inside a compact key
// space: key_base[raster] + ((ty - by0) * w + (tx - bx0)) * 2 + kind, with
// the raster's tile bounding box (bx0, by0)..(bx1, by1) measured in the count
// pass; kind 0 (crossing) sorts before kind 1 (bin) of the same tile.
#include <algorithm>

#include "common.cuh"
#include "internal.h"
#include "scan.cuh"

namespace ochre {

struct BBoxAcc {
    int x0, y0, x1, y1;
};

__device__ __forceinline__ void bbox_add(BBoxAcc& b, int x, int y) {
    const int tx = div8(x), ty = div8(y);
    b.x0 = min(b.x0, tx);
    b.y0 = min(b.y0, ty);
    b.x1 = max(b.x1, tx);
    b.y1 = max(b.y1, ty);
}

// Count bins, crossings and increment cells of a line; extend its raster's
// tile bbox; sum the crossing signs.
__device__ __forceinline__ uint32_t count_line(V2 a, V2 p, BBoxAcc& bb, bool* capped, int* wsum, uint32_t* cells) {
    *wsum = 0;
    *cells = 0;
    if (veq(a, p)) return 0u;
    uint32_t nb = 0, nc = 0, nx = 0, run = 0;
    int ws = 0;
    int ptx = 0x7fffffff, pty = 0x7fffffff;
    const bool ok = walk_line(
        a, p,
        [&](const Walk&, const WalkState& s) {
            const int tx = div8(s.x), ty = div8(s.y);
            if (tx != ptx || ty != pty || run == BIN_MAX_CELLS) { nb++; ptx = tx; pty = ty; run = 0; }
            run++;
            nx++;
        },
        [&](int, int, int sign) {
            nc++;
            ws += sign;
        },
        [&](int x, int y) { bbox_add(bb, x, y); });
    if (!ok) *capped = true;
    *wsum = ws;
    *cells = nx;
    return nb + nc;
}

// Pixel cells a line's walk visits, about: its start cell and one per row
// or column step (the reference's walk may add a cell at a corner tie).
__device__ __forceinline__ uint32_t walk_cells(const float4& l) {
    const float dx = fabsf(floorf(l.z) - floorf(l.x)), dy = fabsf(floorf(l.w) - floorf(l.y));
    const float c = 1.0f + dx + dy;
    return c < 65535.0f ? (uint32_t)c : 65535u;   // also NaN -> 65535 (bucketed last)
}

// Block-local work order by walk length: the BLOCK items of a block are
// grouped by log2 of their cell count (unstable within a group), so each
// warp walks lines of about the same length and a warp of short lines does
// not run as long as the longest line of a random 32.  Returns the item
// (0..BLOCK-1 within the block) this thread walks.  Every thread of the
// block calls it.
template <int BLOCK>
__device__ __forceinline__ uint32_t order_by_length(uint32_t cells, uint32_t* s_cnt, uint16_t* s_item) {
    constexpr int GROUPS = 17;
    const uint32_t g = min(31u - (uint32_t)__clz(max(cells, 1u)), (uint32_t)GROUPS - 1u);
    if (threadIdx.x < GROUPS) s_cnt[threadIdx.x] = 0u;
    __syncthreads();
    const uint32_t k = atomicAdd(&s_cnt[g], 1u);
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t run = 0;
        for (int q = 0; q < GROUPS; q++) {
            const uint32_t c = s_cnt[q];
            s_cnt[q] = run;
            run += c;
        }
    }
    __syncthreads();
    s_item[s_cnt[g] + k] = (uint16_t)threadIdx.x;
    __syncthreads();
    return s_item[threadIdx.x];
}

// Entry counts per line (written in place of the offsets, then scanned)
// and the raster tile boxes.  Counting is a separate kernel, not folded into
// the offset scan: a walk's length varies from one cell to thousands, and a
// single-pass scan would hold every later block behind the slowest walk.
// Boxes (and the rasters' crossing-sign sums) are reduced before any global
// atomic: lanes of one raster (lines of a raster are contiguous) by warp
// reductions, then the block's first BOX_SLOTS rasters in shared memory; the
// block then updates each global box only where it grows.
constexpr int BOX_SLOTS = 8;
__device__ __forceinline__ void box_grow(int4* d, int x0, int y0, int x1, int y1) {
    const int4 cur = ld_words(d);
    if (x0 < cur.x) atomicMin(&d->x, x0);
    if (y0 < cur.y) atomicMin(&d->y, y0);
    if (x1 > cur.z) atomicMax(&d->z, x1);
    if (y1 > cur.w) atomicMax(&d->w, y1);
}
__global__ void __launch_bounds__(256) k_line_count(const float4* __restrict__ lines,
                                                    const uint32_t* __restrict__ line_raster, uint32_t n_cap,
                                                    const uint32_t* n_dev, int4* bbox, int* raster_wsum,
                                                    uint32_t* __restrict__ counts, uint32_t* __restrict__ inc_counts,
                                                    unsigned long long* inc_total, uint32_t* err) {
    __shared__ int4 s_box[BOX_SLOTS];
    __shared__ int s_ws[BOX_SLOTS];
    __shared__ uint32_t s_r0;
    __shared__ uint32_t s_cnt[17];
    __shared__ uint16_t s_item[256];
    __shared__ uint32_t s_incs;
    const uint32_t n_lines = (uint32_t)dev_count(n_cap, n_dev);
    const uint32_t i0 = blockIdx.x * blockDim.x;
    if (i0 >= n_lines) return;
    const uint32_t cells = i0 + threadIdx.x < n_lines ? walk_cells(lines[i0 + threadIdx.x]) : 0u;
    const uint32_t i = i0 + order_by_length<256>(cells, s_cnt, s_item);
    if (threadIdx.x < BOX_SLOTS) {
        s_box[threadIdx.x] = make_int4(0x7fffffff, 0x7fffffff, (int)0x80000000, (int)0x80000000);
        s_ws[threadIdx.x] = 0;
    }
    if (threadIdx.x == 0) {
        s_r0 = line_raster[i0];
        s_incs = 0u;
    }
    __syncthreads();
    const uint32_t r0 = s_r0;
    BBoxAcc bb{0x7fffffff, 0x7fffffff, (int)0x80000000, (int)0x80000000};
    uint32_t r = r0;
    int ws = 0;
    uint32_t nc = 0;
    if (i < n_lines) {
        const float4 l = lines[i];
        bool capped = false;
        counts[i] = count_line(v2(l.x, l.y), v2(l.z, l.w), bb, &capped, &ws, &nc);
        inc_counts[i] = nc;
        if (capped) atomicOr(err, ERR_LIMIT);
        r = line_raster[i];
    }
    const unsigned grp = __match_any_sync(0xffffffffu, r);
    const int x0 = __reduce_min_sync(grp, bb.x0), y0 = __reduce_min_sync(grp, bb.y0);
    const int x1 = __reduce_max_sync(grp, bb.x1), y1 = __reduce_max_sync(grp, bb.y1);
    const int wsg = __reduce_add_sync(grp, ws);
    if ((int)(threadIdx.x & 31) == __ffs(grp) - 1) {
        if (r - r0 < (uint32_t)BOX_SLOTS) {
            if (x0 <= x1) {
                int4* d = s_box + (r - r0);
                atomicMin(&d->x, x0);
                atomicMin(&d->y, y0);
                atomicMax(&d->z, x1);
                atomicMax(&d->w, y1);
            }
            if (wsg) atomicAdd(s_ws + (r - r0), wsg);
        } else {
            if (x0 <= x1) box_grow(bbox + r, x0, y0, x1, y1);
            if (wsg) atomicAdd(raster_wsum + r, wsg);
        }
    }
    // the block's increments (at most 256 lines of a capped walk: 32 bits hold it)
    const uint32_t wi = __reduce_add_sync(0xffffffffu, nc);
    if ((threadIdx.x & 31) == 0 && wi) atomicAdd(&s_incs, wi);
    __syncthreads();
    if (threadIdx.x == 0 && s_incs) atomicAdd(inc_total, (unsigned long long)s_incs);
    if (threadIdx.x < BOX_SLOTS) {
        const int4 b = s_box[threadIdx.x];
        if (b.x <= b.z) box_grow(bbox + r0 + threadIdx.x, b.x, b.y, b.z, b.w);
        if (s_ws[threadIdx.x]) atomicAdd(raster_wsum + r0 + threadIdx.x, s_ws[threadIdx.x]);
    }
}
// Entry and increment offsets of every line, one scan of the pair (in place:
// every count is read by the thread that writes its offset).
struct LinePair {
    uint32_t ent, inc;
};
struct OpLinePair {
    __device__ __forceinline__ LinePair operator()(LinePair a, LinePair b) const {
        return LinePair{a.ent + b.ent, a.inc + b.inc};
    }
};
struct LinePairIn {
    const uint32_t* ent;
    const uint32_t* inc;
    __device__ __forceinline__ LinePair operator()(uint64_t i) const { return LinePair{ent[i], inc[i]}; }
};
struct LinePairOut {
    uint32_t* ent;
    uint32_t* inc;
    __device__ __forceinline__ void operator()(uint64_t i, LinePair ex, LinePair) const {
        ent[i] = ex.ent;
        inc[i] = ex.inc;
    }
};

__global__ void k_bbox_init(int4* bbox, int* wsum, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        bbox[i] = make_int4(0x7fffffff, 0x7fffffff, (int)0x80000000, (int)0x80000000);
        wsum[i] = 0;
    }
}

// Per-raster key space: w * h * 2 keys; rasters without increments get a
// 1x1 box at tile (0,0) and one synthetic bin (finish pushes a bin at (0,0)
// even when there are no increments, rasterizer.rs:194-208).
struct RasterScan {
    uint64_t ks;
    uint32_t ne;
    int32_t w;   // crossing signs of the rasters so far
};
struct OpRaster {
    __device__ __forceinline__ RasterScan operator()(RasterScan a, RasterScan b) const {
        return RasterScan{a.ks + b.ks, a.ne + b.ne, a.w + b.w};
    }
};
struct RasterIn {
    const int4* bbox;
    const int* wsum;
    __device__ __forceinline__ RasterScan operator()(uint64_t r) const {
        const int4 b = bbox[r];
        if (b.x > b.z) return RasterScan{2ull, 1u, wsum[r]};
        const uint64_t w = (uint64_t)(b.z - b.x + 1), h = (uint64_t)(b.w - b.y + 1);
        return RasterScan{w * h * 2ull, 0u, wsum[r]};
    }
};
struct RasterOut {
    int4* bbox;
    uint64_t* key_base;
    uint32_t* empty;   // 0: has increments; else 1 + rank among empty rasters
    int* wbase;        // crossing signs of all earlier rasters
    __device__ __forceinline__ void operator()(uint64_t r, RasterScan ex, RasterScan v) const {
        key_base[r] = ex.ks;
        wbase[r] = ex.w;
        if (v.ne) {
            bbox[r] = make_int4(0, 0, 0, 0);
            empty[r] = ex.ne + 1u;
        } else {
            empty[r] = 0u;
        }
    }
};

template <class K>
__device__ __forceinline__ K make_key(uint64_t base, const int4& bb, int tx, int ty, uint32_t kind) {
    const uint64_t w = (uint64_t)(bb.z - bb.x + 1);
    return (K)(base + (((uint64_t)(ty - bb.y) * w + (uint64_t)(tx - bb.x)) << 1) + kind);
}

// Lines of a block are walked in order of length (order_by_length), so a
// warp's lanes walk lines of about the same length.
template <class K>
__global__ void __launch_bounds__(256) k_line_emit(const float4* __restrict__ lines, const uint32_t* __restrict__ line_raster,
                            const uint32_t* __restrict__ ent_off, const uint32_t* __restrict__ inc_off, uint64_t n_cap,
                            const uint32_t* n_dev, const int4* __restrict__ bbox, const uint64_t* __restrict__ key_base,
                            K* __restrict__ keys, uint32_t* __restrict__ vals, BinRec* __restrict__ bins,
                            float2* __restrict__ incs) {
    __shared__ uint32_t s_cnt[17];
    __shared__ uint16_t s_item[256];
    const uint64_t n_lines = dev_count(n_cap, n_dev);
    const uint64_t i0 = blockIdx.x * (uint64_t)blockDim.x;
    if (i0 >= n_lines) return;
    const uint32_t cells = i0 + threadIdx.x < n_lines ? walk_cells(lines[i0 + threadIdx.x]) : 0u;
    const uint64_t i = i0 + order_by_length<256>(cells, s_cnt, s_item);
    if (i >= n_lines) return;
    const float4 l = lines[i];
    const V2 a = v2(l.x, l.y), p = v2(l.z, l.w);
    if (veq(a, p)) return;
    const uint32_t r = line_raster[i];
    const int4 bb = bbox[r];
    const uint64_t base = key_base[r];
    uint32_t e = ent_off[i];
    uint32_t q = inc_off[i];   // next stored increment
    // increments leave in 16-byte pairs (an even index and the next one):
    // the first of a pair waits in registers
    float2 pend = make_float2(0.0f, 0.0f);
    bool has_pend = false;
    // open bin
    int btx = 0x7fffffff, bty = 0x7fffffff, prev_x = 0;
    uint32_t bcount = 0, bentry = 0;
    BinRec rec;
    auto flush = [&]() {
        if (bcount) {
            rec.n = (uint8_t)bcount;
            *reinterpret_cast<uint4*>(bins + bentry) = *reinterpret_cast<const uint4*>(&rec);
            keys[bentry] = make_key<K>(base, bb, btx, bty, 1u);
            vals[bentry] = bentry;
        }
    };
    walk_line(
        a, p,
        [&](const Walk& w, const WalkState& s) {
            float area, height;
            walk_increment(w, s, area, height);
            const int tx = div8(s.x), ty = div8(s.y);
            if (tx != btx || ty != bty || bcount == BIN_MAX_CELLS) {
                flush();
                btx = tx;
                bty = ty;
                bcount = 0;
                bentry = e++;
                rec.inc = q;
                rec.raster = r;
                rec.x = (int16_t)s.x;
                rec.y = (int16_t)s.y;
                rec.steps = 0;
                rec.dirs = (uint8_t)((w.x_dir < 0 ? 1u : 0u) | (w.y_dir < 0 ? 2u : 0u));
            } else if (s.x != prev_x) {
                rec.steps = (uint16_t)(rec.steps | (1u << (bcount - 1)));   // the step into this cell moved in x
            }
            const float2 v = make_float2(area, height);
            if ((q & 1u) == 0u) {
                pend = v;
                has_pend = true;
            } else if (has_pend) {
                reinterpret_cast<float4*>(incs)[q >> 1] = make_float4(pend.x, pend.y, v.x, v.y);
                has_pend = false;
            } else {
                incs[q] = v;   // the line's first increment at an odd index
            }
            q++;
            prev_x = s.x;
            bcount++;
        },
        [&](int tx, int ty, int sign) {
            const uint32_t c = e++;
            keys[c] = make_key<K>(base, bb, tx, ty, 0u);
            vals[c] = CROSS_TAG | (r << 8) | ((uint32_t)sign & 0xffu);
        },
        [&](int, int) {});
    flush();
    if (has_pend) incs[q - 1] = pend;
}

template <class K>
__global__ void k_empty_emit(const uint32_t* __restrict__ empty, uint32_t n_rasters, uint32_t first_entry,
                             const uint32_t* first_dev, const uint32_t* n_ent_dev,
                             const uint64_t* __restrict__ key_base, K* __restrict__ keys,
                             uint32_t* __restrict__ vals, BinRec* __restrict__ bins) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_rasters) return;
    const uint32_t rank = empty[r];
    if (!rank) return;
    // device-held counts (graph replays): entries after the lines' entries,
    // none when the entry count was over capacity (zeroed)
    if (first_dev != nullptr) first_entry = *first_dev;
    const uint32_t e = first_entry + rank - 1u;
    if (n_ent_dev != nullptr && e >= *n_ent_dev) return;
    BinRec rec;
    rec.inc = 0;
    rec.raster = r;
    rec.x = 0;
    rec.y = 0;
    rec.steps = 0;
    rec.n = 0;
    rec.dirs = 0;
    bins[e] = rec;
    keys[e] = (K)(key_base[r] + 1ull);
    vals[e] = e;
}

int stage_bin(ochre_gpu_ctx* ctx, const ochre_batch* in, uint32_t n_lines, cudaStream_t s, uint64_t* n_entries,
              uint32_t* key_bits) {
    DevScalars* ds = dev_scalars(ctx);
    const uint32_t R = in->n_rasters;
    *n_entries = 0;
    *key_bits = 0;
    if (R == 0) return OCHRE_OK;
    if (R > MAX_RASTERS) return OCHRE_E_CAPACITY;
    OCHRE_CUDA_TRY(ctx->raster_bbox.ensure((size_t)R * sizeof(int4)));
    OCHRE_CUDA_TRY(ctx->raster_keybase.ensure((size_t)R * 8));
    OCHRE_CUDA_TRY(ctx->raster_empty.ensure((size_t)R * 4));
    OCHRE_CUDA_TRY(ctx->raster_wsum.ensure((size_t)R * 4));
    OCHRE_CUDA_TRY(ctx->raster_wbase.ensure((size_t)R * 4));
    OCHRE_LAUNCH(ctx, "bbox_init", s, k_bbox_init<<<(R + 255) / 256, 256, 0, s>>>(ctx->raster_bbox.as<int4>(),
                                                                                 ctx->raster_wsum.as<int>(), R));
    OCHRE_CUDA_TRY(cudaGetLastError());
    // the line pair's totals and the 64-bit increment count
    static_assert(offsetof(DevScalars, inc_total) == offsetof(DevScalars, line_ent_total) + 8, "layout");
    OCHRE_CUDA_TRY(cudaMemsetAsync(&ds->line_ent_total, 0, 16, s));
    // graph replays: n_lines is the capacity, the count is on the device
    const GraphPlan* plan = ctx->plan;
    const uint32_t* lines_dev = plan ? &ds->n_lines : nullptr;
    if (n_lines) {
        OCHRE_CUDA_TRY(ctx->line_ent_off.ensure((size_t)n_lines * 4));
        OCHRE_CUDA_TRY(ctx->line_inc_off.ensure((size_t)n_lines * 4));
        OCHRE_CUDA_TRY(ctx->scan_status.ensure(scan_tiles(n_lines) * sizeof(ScanStatus<LinePair>)));
        OCHRE_LAUNCH(ctx, "dda_count", s, k_line_count<<<(n_lines + 255) / 256, 256, 0, s>>>(
            ctx->lines.as<float4>(), ctx->line_raster.as<uint32_t>(), n_lines, lines_dev, ctx->raster_bbox.as<int4>(),
            ctx->raster_wsum.as<int>(), ctx->line_ent_off.as<uint32_t>(), ctx->line_inc_off.as<uint32_t>(),
            reinterpret_cast<unsigned long long*>(&ds->inc_total), &ds->err));
        OCHRE_CUDA_TRY(cudaGetLastError());
        // in place: every count is read by the thread that writes its offset
        OCHRE_LAUNCH(ctx, "dda_offset_scan", s, OCHRE_CUDA_TRY(launch_scan<LinePair>(
            n_lines, LinePairIn{ctx->line_ent_off.as<uint32_t>(), ctx->line_inc_off.as<uint32_t>()},
            LinePairOut{ctx->line_ent_off.as<uint32_t>(), ctx->line_inc_off.as<uint32_t>()}, OpLinePair{},
            LinePair{0u, 0u}, ctx->scan_status.p, &ds->ticket, reinterpret_cast<LinePair*>(&ds->line_ent_total),
            &ds->err, s, lines_dev)));
    }
    OCHRE_CUDA_TRY(ctx->scan_status.ensure(scan_tiles(R) * sizeof(ScanStatus<RasterScan>)));
    OCHRE_LAUNCH(ctx, "raster_key_scan", s, OCHRE_CUDA_TRY(launch_scan<RasterScan>(
        R, RasterIn{ctx->raster_bbox.as<int4>(), ctx->raster_wsum.as<int>()},
        RasterOut{ctx->raster_bbox.as<int4>(), ctx->raster_keybase.as<uint64_t>(), ctx->raster_empty.as<uint32_t>(),
                  ctx->raster_wbase.as<int>()},
        OpRaster{}, RasterScan{0, 0, 0}, ctx->scan_status.p, &ds->ticket,
        reinterpret_cast<RasterScan*>(&ds->keyspace), &ds->err, s)));
    uint64_t E;
    uint32_t bits;
    uint32_t first_entry = 0;
    uint64_t n_incs;
    bool any_empty = true;
    if (plan) {
        // entry total, key space and stored increments checked against the plan on the device
        OCHRE_LAUNCH(ctx, "plan_entries", s, OCHRE_CUDA_TRY(launch_plan_entries(ctx, plan->entries, plan->key_bits,
                                                                                plan->incs, s)));
        E = plan->entries;
        bits = plan->key_bits;
        n_incs = plan->incs;
    } else {
        int st = read_scalars(ctx, s);
        if (st != OCHRE_OK) return st;
        st = check_device_error(ctx);
        if (st != OCHRE_OK) return st;
        const DevScalars* hs = host_scalars(ctx);
        E = (uint64_t)hs->line_ent_total + hs->n_empty;
        n_incs = hs->inc_total;
        if (E > MAX_COUNT || n_incs > MAX_INCS) return OCHRE_E_CAPACITY;
        ctx->stats.n_incs = (uint32_t)n_incs;
        const uint64_t K = hs->keyspace;
        bits = 1;
        while (bits < 64 && (K - 1) >> bits) bits++;
        first_entry = hs->line_ent_total;
        any_empty = hs->n_empty != 0;
    }
    OCHRE_CUDA_TRY(ctx->incs.ensure((size_t)std::max<uint64_t>(n_incs, 1) * sizeof(float2)));
    *key_bits = bits;
    *n_entries = E;
    ctx->keys64 = bits > 32;
    const size_t ksz = ctx->keys64 ? 8 : 4;
    OCHRE_CUDA_TRY(ctx->keys.ensure(E * ksz));
    OCHRE_CUDA_TRY(ctx->vals.ensure(E * 4));
    OCHRE_CUDA_TRY(ctx->keys_alt.ensure(E * ksz));
    OCHRE_CUDA_TRY(ctx->vals_alt.ensure(E * 4));
    OCHRE_CUDA_TRY(ctx->bins.ensure(E * sizeof(BinRec)));
    if (n_lines) {
        const unsigned blocks = (unsigned)((n_lines + 255) / 256);
        if (ctx->keys64)
            OCHRE_LAUNCH(ctx, "dda_emit", s, k_line_emit<uint64_t><<<blocks, 256, 0, s>>>(
                ctx->lines.as<float4>(), ctx->line_raster.as<uint32_t>(), ctx->line_ent_off.as<uint32_t>(),
                ctx->line_inc_off.as<uint32_t>(), n_lines, lines_dev, ctx->raster_bbox.as<int4>(),
                ctx->raster_keybase.as<uint64_t>(), ctx->keys.as<uint64_t>(), ctx->vals.as<uint32_t>(),
                ctx->bins.as<BinRec>(), ctx->incs.as<float2>()));
        else
            OCHRE_LAUNCH(ctx, "dda_emit", s, k_line_emit<uint32_t><<<blocks, 256, 0, s>>>(
                ctx->lines.as<float4>(), ctx->line_raster.as<uint32_t>(), ctx->line_ent_off.as<uint32_t>(),
                ctx->line_inc_off.as<uint32_t>(), n_lines, lines_dev, ctx->raster_bbox.as<int4>(),
                ctx->raster_keybase.as<uint64_t>(), ctx->keys.as<uint32_t>(), ctx->vals.as<uint32_t>(),
                ctx->bins.as<BinRec>(), ctx->incs.as<float2>()));
        OCHRE_CUDA_TRY(cudaGetLastError());
    }
    if (any_empty) {
        const uint32_t* first_dev = plan ? &ds->line_ent_total : nullptr;
        const uint32_t* ent_dev = plan ? &ds->n_entries : nullptr;
        if (ctx->keys64)
            OCHRE_LAUNCH(ctx, "empty_emit", s, k_empty_emit<uint64_t><<<(R + 255) / 256, 256, 0, s>>>(
                ctx->raster_empty.as<uint32_t>(), R, first_entry, first_dev, ent_dev,
                ctx->raster_keybase.as<uint64_t>(), ctx->keys.as<uint64_t>(), ctx->vals.as<uint32_t>(),
                ctx->bins.as<BinRec>()));
        else
            OCHRE_LAUNCH(ctx, "empty_emit", s, k_empty_emit<uint32_t><<<(R + 255) / 256, 256, 0, s>>>(
                ctx->raster_empty.as<uint32_t>(), R, first_entry, first_dev, ent_dev,
                ctx->raster_keybase.as<uint64_t>(), ctx->keys.as<uint32_t>(), ctx->vals.as<uint32_t>(),
                ctx->bins.as<BinRec>()));
        OCHRE_CUDA_TRY(cudaGetLastError());
    }
    return OCHRE_OK;
}

}  // namespace ochre
