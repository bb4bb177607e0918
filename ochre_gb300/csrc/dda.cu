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

// Persistent count walks of short lines.  A warp takes windows of WIN
// consecutive lines by ticket and walks each window's lines 32 at a time in
// order of length (grouped by log2 of their cell count, unstable within a
// group), so a warp's lanes walk lines of about the same length; no warp
// waits on another, so an SM stays full until the last window (a block of
// lines ordered in the block holds its SM slot until its slowest warp ends:
// count 1.87 -> 1.71 ms on the 20,000-path uneven mix, 0.169 -> 0.143 ms on
// 100,000 glyphs).  The emit walk keeps the block form: there, each group's
// set-up loads (line, offsets, raster box and key base) waited behind the
// previous group of the warp, 9.8 against 7.9 ms.
constexpr int WIN = 256;
constexpr int WIN_PER_LANE = WIN / 32;
constexpr int WALK_BLOCK = 128;
constexpr int LEN_GROUPS = 17;

// Orders this warp's window: item WIN_PER_LANE * ... of lane k is
// k + 32 * j (j < WIN_PER_LANE) with `cells[j]` cells; fills s_item[0..WIN)
// with the items grouped by length.  s_cnt: LEN_GROUPS words of the warp.
__device__ __forceinline__ void order_window(const uint32_t (&cells)[WIN_PER_LANE], uint32_t* s_cnt,
                                             uint16_t* s_item) {
    const uint32_t lane = threadIdx.x & 31u;
    if (lane < LEN_GROUPS) s_cnt[lane] = 0u;
    __syncwarp();
    uint32_t g[WIN_PER_LANE], k[WIN_PER_LANE];
#pragma unroll
    for (int j = 0; j < WIN_PER_LANE; j++) {
        g[j] = min(31u - (uint32_t)__clz(max(cells[j], 1u)), (uint32_t)LEN_GROUPS - 1u);
        k[j] = atomicAdd(&s_cnt[g[j]], 1u);
    }
    __syncwarp();
    const uint32_t c = lane < LEN_GROUPS ? s_cnt[lane] : 0u;
    uint32_t inc = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= (uint32_t)o) inc += t;
    }
    __syncwarp();
    if (lane < LEN_GROUPS) s_cnt[lane] = inc - c;
    __syncwarp();
#pragma unroll
    for (int j = 0; j < WIN_PER_LANE; j++) s_item[s_cnt[g[j]] + k[j]] = (uint16_t)(j * 32 + lane);
    __syncwarp();
}

// The next window of a warp (lane 0 takes the ticket); WIN * it is its first line.
__device__ __forceinline__ uint64_t next_window(uint32_t* ticket) {
    uint32_t w = 0;
    if ((threadIdx.x & 31u) == 0u) w = atomicAdd(ticket, 1u);
    return (uint64_t)__shfl_sync(0xffffffffu, w, 0) * WIN;
}

// A raster's global tile box grows by atomics only where it grows.
__device__ __forceinline__ void box_grow(int4* d, int x0, int y0, int x1, int y1) {
    const int4 cur = ld_words(d);
    if (x0 < cur.x) atomicMin(&d->x, x0);
    if (y0 < cur.y) atomicMin(&d->y, y0);
    if (x1 > cur.z) atomicMax(&d->z, x1);
    if (y1 > cur.w) atomicMax(&d->w, y1);
}

// ---------------------------------------------------------------------
// Long lines: persistent walkers with per-lane refill.
//
// Walk lengths run from one cell to thousands (a path's long edges).  One
// thread per line, as the count and emit kernels walk most lines, would give
// a long line's warp one busy lane for thousands of steps.  The flatten
// stage queues every line of more than `long_cells` (estimated) cells, and
// the first blocks of the count and emit kernels walk that queue this way:
// every lane of a warp makes one DDA step per loop iteration; a lane whose
// line has ended takes the next line from the warp's pool of WALK_POOL
// queued lines, and the warp takes a new pool from a global ticket when its
// pool runs out.  A refill waits until at least `refill` lanes are idle (a
// refill costs the new lines' set-up loads).  Outputs go to the per-line
// offsets of the count scan, so they do not depend on which lane walks which
// line.  (For short lines the per-line set-up, run by the few lanes that
// refill at a time, costs more than the idle lanes it saves: measured
// slower on every configuration, so short lines stay one per thread.)
//
// Job interface (per lane): bool begin(queue index, Walk&, WalkState&) sets
// the walk up (false: the line has no walk); cell(w, s) for every increment
// cell; visit(x, y) for every visited cell; cross(tx, ty, sign) for every
// tile-row crossing; end(capped) when the line's walk is over.  The step
// sequence is walk_line's (common.cuh), including its WALK_CAP.
// ---------------------------------------------------------------------
constexpr uint32_t WALK_POOL = 32;

// The rest of a line's walk from its current state (it steps taken):
// walk_line's loop with the job's callbacks, then job.end.
template <class Job>
__device__ __forceinline__ void walk_rest(const Walk& w, WalkState& s, int ty_prev, uint32_t it, Job& job) {
    bool capped = false;
    for (;;) {
        job.cell(w, s);
        const bool done = walk_step(w, s);
        job.visit(s.x, s.y);
        const int ty = div8(s.y);
        if (ty != ty_prev) {
            job.cross(div8(s.x), min(ty_prev, ty), (int)(int8_t)(int16_t)(ty - ty_prev));
            ty_prev = ty;
        }
        if (done) break;
        if (++it >= WALK_CAP) {
            capped = true;
            break;
        }
    }
    job.end(capped);
}

template <class Job>
__device__ __forceinline__ void walk_refill(uint64_t n_lines, const uint32_t* __restrict__ queue, uint32_t* ticket,
                                            uint32_t refill, Job& job) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t below = (1u << lane) - 1u;
    uint64_t pool = 0, pool_end = 0;   // warp-uniform
    bool more = true;                  // warp-uniform
    bool live = false;
    Walk w;
    WalkState s;
    int ty_prev = 0;
    uint32_t it = 0;
    for (;;) {
        uint32_t idle = __ballot_sync(0xffffffffu, !live);
        if (more && (uint32_t)__popc(idle) >= refill) {
            while (idle != 0u) {
                if (pool == pool_end) {
                    uint32_t b = 0;
                    if (lane == 0) b = atomicAdd(ticket, 1u);
                    const uint64_t first = (uint64_t)__shfl_sync(0xffffffffu, b, 0) * WALK_POOL;
                    if (first >= n_lines) {
                        more = false;
                        break;
                    }
                    pool = first;
                    pool_end = min(first + WALK_POOL, n_lines);
                }
                const uint32_t avail = (uint32_t)(pool_end - pool);
                const uint32_t rank = (uint32_t)__popc(idle & below);
                if (((idle >> lane) & 1u) && rank < avail) {
                    live = job.begin(queue[pool + rank], w, s);
                    if (live) {
                        ty_prev = div8(s.y);
                        it = 0;
                        job.visit(s.x, s.y);
                    }
                }
                pool += min((uint32_t)__popc(idle), avail);
                idle = __ballot_sync(0xffffffffu, !live);
            }
        }
        if (!more) {
            // nothing left to take: the live lanes finish their lines without
            // the per-step votes (the last, longest walks set the kernel's end)
            if (live) walk_rest(w, s, ty_prev, it, job);
            break;
        }
        if (__ballot_sync(0xffffffffu, live) == 0u) continue;
        if (live) {
            job.cell(w, s);
            bool done = walk_step(w, s);
            job.visit(s.x, s.y);
            const int ty = div8(s.y);
            if (ty != ty_prev) {
                job.cross(div8(s.x), min(ty_prev, ty), (int)(int8_t)(int16_t)(ty - ty_prev));
                ty_prev = ty;
            }
            bool capped = false;
            if (!done && ++it >= WALK_CAP) {
                capped = true;
                done = true;
            }
            if (done) {
                job.end(capped);
                live = false;
            }
        }
    }
}

// One line whose walk job.begin has set up.
template <class Job>
__device__ __forceinline__ void walk_one(Walk& w, WalkState& s, Job& job) {
    job.visit(s.x, s.y);
    walk_rest(w, s, div8(s.y), 0u, job);
}

// Counts of the count pass (see k_line_count) for a queued line, per lane.
// The raster boxes and crossing-sign sums gather over the lane's lines of one
// raster and go to memory when the lane moves to another raster.
struct CountJob {
    const float4* lines;
    const uint32_t* line_raster;
    uint32_t* counts;
    uint32_t* inc_counts;
    int4* bbox;
    int* raster_wsum;
    uint32_t* err;
    // the line
    uint32_t line, nb, nc, nx, run;
    int ptx, pty, ws;
    // the lane's current raster
    uint32_t r;
    BBoxAcc bb;
    int wsr;
    uint64_t incs;   // increments of the lane's lines

    __device__ __forceinline__ void flush() {
        if (r == 0xffffffffu) return;
        if (bb.x0 <= bb.x1) box_grow(bbox + r, bb.x0, bb.y0, bb.x1, bb.y1);
        if (wsr) atomicAdd(raster_wsum + r, wsr);
    }
    __device__ __forceinline__ bool begin(uint32_t i, Walk& w, WalkState& s) {
        const float4 l = lines[i];
        const uint32_t ri = line_raster[i];
        if (ri != r) {
            flush();
            r = ri;
            bb = BBoxAcc{0x7fffffff, 0x7fffffff, (int)0x80000000, (int)0x80000000};
            wsr = 0;
        }
        const V2 a = v2(l.x, l.y), p = v2(l.z, l.w);
        if (veq(a, p)) {
            counts[i] = 0u;
            inc_counts[i] = 0u;
            return false;
        }
        walk_setup(a, p, w, s);
        line = i;
        nb = nc = nx = run = 0u;
        ptx = pty = 0x7fffffff;
        ws = 0;
        return true;
    }
    __device__ __forceinline__ void cell(const Walk&, const WalkState& s) {
        const int tx = div8(s.x), ty = div8(s.y);
        if (tx != ptx || ty != pty || run == BIN_MAX_CELLS) {
            nb++;
            ptx = tx;
            pty = ty;
            run = 0;
        }
        run++;
        nx++;
    }
    __device__ __forceinline__ void visit(int x, int y) { bbox_add(bb, x, y); }
    __device__ __forceinline__ void cross(int, int, int sign) {
        nc++;
        ws += sign;
    }
    __device__ __forceinline__ void end(bool capped) {
        counts[line] = nb + nc;
        inc_counts[line] = nx;
        incs += nx;
        wsr += ws;
        if (capped) atomicOr(err, ERR_LIMIT);
    }
};

// The queued long lines' counts (see k_line_count): persistent blocks of
// refilled lanes (walk_refill).
constexpr int LONG_THREADS = 128;
constexpr uint32_t LONG_BLOCKS_PER_SM = 2;
__global__ void __launch_bounds__(LONG_THREADS) k_line_count_long(
    const float4* __restrict__ lines, const uint32_t* __restrict__ line_raster, uint32_t n_cap, const uint32_t* n_dev,
    int4* bbox, int* raster_wsum, uint32_t* __restrict__ counts, uint32_t* __restrict__ inc_counts,
    unsigned long long* inc_total, const uint32_t* __restrict__ queue, const uint32_t* n_queue, uint32_t* ticket,
    uint32_t refill, uint32_t* err) {
    // (a line count zeroed on the device, after an overflow of a graph's
    // plan, stops these walks too)
    if (dev_count(n_cap, n_dev) == 0) return;
    CountJob job;
    job.lines = lines;
    job.line_raster = line_raster;
    job.counts = counts;
    job.inc_counts = inc_counts;
    job.bbox = bbox;
    job.raster_wsum = raster_wsum;
    job.err = err;
    job.r = 0xffffffffu;
    job.bb = BBoxAcc{0x7fffffff, 0x7fffffff, (int)0x80000000, (int)0x80000000};
    job.wsr = 0;
    job.incs = 0;
    walk_refill(*n_queue, queue, ticket, refill, job);
    job.flush();
    unsigned long long t = job.incs;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if ((threadIdx.x & 31u) == 0u && t) atomicAdd(inc_total, t);
}

// Entry counts per line (written in place of the offsets, then scanned)
// and the raster tile boxes.  Counting is a separate kernel, not folded into
// the offset scan: a walk's length varies from one cell to thousands, and a
// single-pass scan would hold every later block behind the slowest walk.
// Persistent warps over windows (see order_window); lines of more than
// long_cells cells are left to k_line_count_long.  Boxes (and the rasters'
// crossing-sign sums) are reduced before any global atomic: lanes of one
// raster by warp reductions, then the window's first BOX_SLOTS rasters (lines
// of a raster are contiguous) in the warp's shared slots; each global box is
// then updated only where it grows.
constexpr int BOX_SLOTS = 8;
__global__ void __launch_bounds__(WALK_BLOCK) k_line_count(const float4* __restrict__ lines,
                                                           const uint32_t* __restrict__ line_raster, uint32_t n_cap,
                                                           const uint32_t* n_dev, int4* bbox, int* raster_wsum,
                                                           uint32_t* __restrict__ counts,
                                                           uint32_t* __restrict__ inc_counts,
                                                           unsigned long long* inc_total, uint32_t long_cells,
                                                           uint32_t* ticket, uint32_t* err) {
    constexpr int WARPS = WALK_BLOCK / 32;
    __shared__ int4 s_box[WARPS][BOX_SLOTS];
    __shared__ int s_ws[WARPS][BOX_SLOTS];
    __shared__ uint32_t s_cnt[WARPS][LEN_GROUPS];
    __shared__ uint16_t s_item[WARPS][WIN];
    const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    const uint64_t n_lines = dev_count(n_cap, n_dev);
    unsigned long long incs = 0;   // the warp's increments (lane 0)
    for (;;) {
        const uint64_t i0 = next_window(ticket);
        if (i0 >= n_lines) break;
        uint32_t cells[WIN_PER_LANE];
#pragma unroll
        for (int j = 0; j < WIN_PER_LANE; j++) {
            const uint64_t i = i0 + j * 32 + lane;
            cells[j] = i < n_lines ? walk_cells(lines[i]) : 0u;
        }
        order_window(cells, s_cnt[wid], s_item[wid]);
        if (lane < BOX_SLOTS) {
            s_box[wid][lane] = make_int4(0x7fffffff, 0x7fffffff, (int)0x80000000, (int)0x80000000);
            s_ws[wid][lane] = 0;
        }
        const uint32_t r0 = line_raster[i0];
        __syncwarp();
        for (int j = 0; j < WIN_PER_LANE; j++) {
            const uint64_t i = i0 + s_item[wid][j * 32 + lane];
            BBoxAcc bb{0x7fffffff, 0x7fffffff, (int)0x80000000, (int)0x80000000};
            uint32_t r = r0;
            int ws = 0;
            uint32_t nc = 0;
            if (i < n_lines) {
                const float4 l = lines[i];
                if (!(long_cells && walk_cells(l) > long_cells)) {
                    bool capped = false;
                    counts[i] = count_line(v2(l.x, l.y), v2(l.z, l.w), bb, &capped, &ws, &nc);
                    inc_counts[i] = nc;
                    if (capped) atomicOr(err, ERR_LIMIT);
                    r = line_raster[i];
                }
            }
            const unsigned grp = __match_any_sync(0xffffffffu, r);
            const int x0 = __reduce_min_sync(grp, bb.x0), y0 = __reduce_min_sync(grp, bb.y0);
            const int x1 = __reduce_max_sync(grp, bb.x1), y1 = __reduce_max_sync(grp, bb.y1);
            const int wsg = __reduce_add_sync(grp, ws);
            if ((int)lane == __ffs(grp) - 1) {
                if (r - r0 < (uint32_t)BOX_SLOTS) {
                    if (x0 <= x1) {
                        int4* d = &s_box[wid][r - r0];
                        atomicMin(&d->x, x0);
                        atomicMin(&d->y, y0);
                        atomicMax(&d->z, x1);
                        atomicMax(&d->w, y1);
                    }
                    if (wsg) atomicAdd(&s_ws[wid][r - r0], wsg);
                } else {
                    if (x0 <= x1) box_grow(bbox + r, x0, y0, x1, y1);
                    if (wsg) atomicAdd(raster_wsum + r, wsg);
                }
            }
            // (at most 32 capped walks: 32 bits hold it)
            incs += __reduce_add_sync(0xffffffffu, nc);
        }
        __syncwarp();
        if (lane < BOX_SLOTS) {
            const int4 b = s_box[wid][lane];
            if (b.x <= b.z) box_grow(bbox + r0 + lane, b.x, b.y, b.z, b.w);
            if (s_ws[wid][lane]) atomicAdd(raster_wsum + r0 + lane, s_ws[wid][lane]);
        }
        __syncwarp();
    }
    if (lane == 0 && incs) atomicAdd(inc_total, incs);
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

// Entries and increments of the emit pass (see k_line_emit) for one line.
template <class K>
struct EmitJob {
    const float4* lines;
    const uint32_t* line_raster;
    const uint32_t* ent_off;
    const uint32_t* inc_off;
    const int4* bbox;
    const uint64_t* key_base;
    K* keys;
    uint32_t* vals;
    BinRec* bins;
    float2* incs;
    // the line's raster (kept while the lane stays in it)
    uint32_t r;
    int4 bb;
    uint64_t base;
    // the line
    uint32_t e, q;   // next entry, next stored increment
    float2 pend;     // increments leave in 16-byte pairs; the first of a pair waits here
    bool has_pend;
    int btx, bty, prev_x;   // open bin
    uint32_t bcount, bentry;
    BinRec rec;

    __device__ __forceinline__ void flush_bin() {
        if (bcount) {
            rec.n = (uint8_t)bcount;
            *reinterpret_cast<uint4*>(bins + bentry) = *reinterpret_cast<const uint4*>(&rec);
            keys[bentry] = make_key<K>(base, bb, btx, bty, 1u);
            vals[bentry] = bentry;
        }
    }
    __device__ __forceinline__ bool begin(uint32_t i, Walk& w, WalkState& s) {
        const float4 l = lines[i];
        const V2 a = v2(l.x, l.y), p = v2(l.z, l.w);
        if (veq(a, p)) return false;
        const uint32_t ri = line_raster[i];
        if (ri != r) {
            r = ri;
            bb = bbox[ri];
            base = key_base[ri];
        }
        e = ent_off[i];
        q = inc_off[i];
        has_pend = false;
        btx = bty = 0x7fffffff;
        prev_x = 0;
        bcount = 0;
        walk_setup(a, p, w, s);
        return true;
    }
    __device__ __forceinline__ void cell(const Walk& w, const WalkState& s) {
        float area, height;
        walk_increment(w, s, area, height);
        const int tx = div8(s.x), ty = div8(s.y);
        if (tx != btx || ty != bty || bcount == BIN_MAX_CELLS) {
            flush_bin();
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
    }
    __device__ __forceinline__ void visit(int, int) {}
    __device__ __forceinline__ void cross(int tx, int ty, int sign) {
        const uint32_t c = e++;
        keys[c] = make_key<K>(base, bb, tx, ty, 0u);
        vals[c] = CROSS_TAG | (r << 8) | ((uint32_t)sign & 0xffu);
    }
    __device__ __forceinline__ void end(bool) {
        flush_bin();
        if (has_pend) incs[q - 1] = pend;
    }
};

// The queued long lines' entries and increments (see k_line_emit):
// persistent blocks of refilled lanes (walk_refill).
template <class K>
__global__ void __launch_bounds__(LONG_THREADS) k_line_emit_long(
    const float4* __restrict__ lines, const uint32_t* __restrict__ line_raster, const uint32_t* __restrict__ ent_off,
    const uint32_t* __restrict__ inc_off, uint64_t n_cap, const uint32_t* n_dev, const int4* __restrict__ bbox,
    const uint64_t* __restrict__ key_base, K* __restrict__ keys, uint32_t* __restrict__ vals,
    BinRec* __restrict__ bins, float2* __restrict__ incs, const uint32_t* __restrict__ queue, const uint32_t* n_queue,
    uint32_t* ticket, uint32_t refill) {
    // (a line count zeroed on the device, after an overflow of a graph's
    // plan, stops these walks too: their offsets were not written)
    if (dev_count(n_cap, n_dev) == 0) return;
    EmitJob<K> job;
    job.lines = lines;
    job.line_raster = line_raster;
    job.ent_off = ent_off;
    job.inc_off = inc_off;
    job.bbox = bbox;
    job.key_base = key_base;
    job.keys = keys;
    job.vals = vals;
    job.bins = bins;
    job.incs = incs;
    job.r = 0xffffffffu;
    walk_refill(*n_queue, queue, ticket, refill, job);
}

// Every thread walks one line, the lines of a block in order of length
// (order_by_length) so a warp's lanes walk lines of about the same length.
// Lines of more than long_cells cells are left to k_line_emit_long.
template <class K>
__global__ void __launch_bounds__(256) k_line_emit(const float4* __restrict__ lines, const uint32_t* __restrict__ line_raster,
                            const uint32_t* __restrict__ ent_off, const uint32_t* __restrict__ inc_off, uint64_t n_cap,
                            const uint32_t* n_dev, const int4* __restrict__ bbox, const uint64_t* __restrict__ key_base,
                            K* __restrict__ keys, uint32_t* __restrict__ vals, BinRec* __restrict__ bins,
                            float2* __restrict__ incs, uint32_t long_cells) {
    __shared__ uint32_t s_cnt[17];
    __shared__ uint16_t s_item[256];
    const uint64_t n_lines = dev_count(n_cap, n_dev);
    const uint64_t i0 = blockIdx.x * (uint64_t)blockDim.x;
    if (i0 >= n_lines) return;
    const uint32_t cells = i0 + threadIdx.x < n_lines ? walk_cells(lines[i0 + threadIdx.x]) : 0u;
    const uint64_t i = i0 + order_by_length<256>(cells, s_cnt, s_item);
    if (i >= n_lines) return;
    if (long_cells && walk_cells(lines[i]) > long_cells) return;
    EmitJob<K> job;
    job.lines = lines;
    job.line_raster = line_raster;
    job.ent_off = ent_off;
    job.inc_off = inc_off;
    job.bbox = bbox;
    job.key_base = key_base;
    job.keys = keys;
    job.vals = vals;
    job.bins = bins;
    job.incs = incs;
    job.r = 0xffffffffu;
    Walk w;
    WalkState s;
    if (job.begin((uint32_t)i, w, s)) walk_one(w, s, job);
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

// The stream the long-line walkers run on: a side stream that waits for
// the run's stream s here (join_walks makes s wait for it in turn), so that
// the walkers, whose time is the longest line's serial walk, overlap the
// per-line kernel.  s itself when the context has no side stream.
static cudaError_t fork_walks(ochre_gpu_ctx* ctx, cudaStream_t s, cudaStream_t* side) {
    *side = s;
    if (ctx->no_side_stream) return cudaSuccess;
    if (!ctx->walk_stream) {
        if (cudaStreamCreateWithFlags(&ctx->walk_stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&ctx->ev_walk_fork, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&ctx->ev_walk_join, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            ctx->no_side_stream = true;
            return cudaSuccess;
        }
    }
    cudaError_t e = cudaEventRecord(ctx->ev_walk_fork, s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->walk_stream, ctx->ev_walk_fork, 0);
    if (e == cudaSuccess) *side = ctx->walk_stream;
    return e;
}
static cudaError_t join_walks(ochre_gpu_ctx* ctx, cudaStream_t side, cudaStream_t s) {
    if (side == s) return cudaSuccess;
    cudaError_t e = cudaEventRecord(ctx->ev_walk_join, side);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, ctx->ev_walk_join, 0);
    return e;
}

// Persistent grid of a windowed walk kernel: the blocks the GPU keeps
// resident, or fewer when there are fewer windows than warps.
template <class Kernel>
static unsigned window_grid(ochre_gpu_ctx* ctx, Kernel kernel, uint64_t n_lines) {
    int sms = 152, occ = 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, WALK_BLOCK, 0) != cudaSuccess || occ < 1) {
        cudaGetLastError();
        occ = 1;
    }
    const uint64_t windows = (n_lines + WIN - 1) / WIN;
    const uint64_t blocks = (windows + WALK_BLOCK / 32 - 1) / (WALK_BLOCK / 32);
    return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(blocks, (uint64_t)sms * (uint64_t)occ));
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
    // the line pair's totals, the 64-bit increment count and the walks' tickets
    static_assert(offsetof(DevScalars, inc_total) == offsetof(DevScalars, line_ent_total) + 8 &&
                      offsetof(DevScalars, walk_ticket) == offsetof(DevScalars, line_ent_total) + 16,
                  "layout");
    OCHRE_CUDA_TRY(cudaMemsetAsync(&ds->line_ent_total, 0, 24, s));
    OCHRE_CUDA_TRY(cudaMemsetAsync(&ds->line_ticket, 0, 4, s));
    // long-line walkers: persistent, LONG_BLOCKS_PER_SM blocks per SM (each
    // refills its lanes from the queue)
    const uint32_t long_cells = (uint32_t)ctx->tune_chain_long_cells;
    const uint32_t refill = (uint32_t)ctx->tune_chain_walk_refill;
    uint32_t long_blocks = 0;
    if (long_cells) {
        int sms = 152;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
        long_blocks = (uint32_t)sms * LONG_BLOCKS_PER_SM;
    }
    const uint32_t* queue = long_cells ? ctx->long_lines.as<uint32_t>() : nullptr;
    // graph replays: n_lines is the capacity, the count is on the device
    const GraphPlan* plan = ctx->plan;
    const uint32_t* lines_dev = plan ? &ds->n_lines : nullptr;
    if (n_lines) {
        OCHRE_CUDA_TRY(ctx->line_ent_off.ensure((size_t)n_lines * 4));
        OCHRE_CUDA_TRY(ctx->line_inc_off.ensure((size_t)n_lines * 4));
        OCHRE_CUDA_TRY(ctx->scan_status.ensure(scan_tiles(n_lines) * sizeof(ScanStatus<LinePair>)));
        cudaStream_t side = s;
        if (long_blocks) {
            OCHRE_CUDA_TRY(fork_walks(ctx, s, &side));
            OCHRE_LAUNCH(ctx, "dda_count_long", side, k_line_count_long<<<long_blocks, LONG_THREADS, 0, side>>>(
                ctx->lines.as<float4>(), ctx->line_raster.as<uint32_t>(), n_lines, lines_dev,
                ctx->raster_bbox.as<int4>(), ctx->raster_wsum.as<int>(), ctx->line_ent_off.as<uint32_t>(),
                ctx->line_inc_off.as<uint32_t>(), reinterpret_cast<unsigned long long*>(&ds->inc_total), queue,
                &ds->n_long, &ds->walk_ticket[0], refill, &ds->err));
            OCHRE_CUDA_TRY(cudaGetLastError());
        }
        OCHRE_LAUNCH(ctx, "dda_count", s, k_line_count<<<window_grid(ctx, k_line_count, n_lines), WALK_BLOCK, 0, s>>>(
            ctx->lines.as<float4>(), ctx->line_raster.as<uint32_t>(), n_lines, lines_dev, ctx->raster_bbox.as<int4>(),
            ctx->raster_wsum.as<int>(), ctx->line_ent_off.as<uint32_t>(), ctx->line_inc_off.as<uint32_t>(),
            reinterpret_cast<unsigned long long*>(&ds->inc_total), long_cells, &ds->line_ticket, &ds->err));
        OCHRE_CUDA_TRY(cudaGetLastError());
        OCHRE_CUDA_TRY(join_walks(ctx, side, s));
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
        cudaStream_t side = s;
        if (long_blocks) OCHRE_CUDA_TRY(fork_walks(ctx, s, &side));
        if (long_blocks && ctx->keys64)
            OCHRE_LAUNCH(ctx, "dda_emit_long", side, k_line_emit_long<uint64_t><<<long_blocks, LONG_THREADS, 0, side>>>(
                ctx->lines.as<float4>(), ctx->line_raster.as<uint32_t>(), ctx->line_ent_off.as<uint32_t>(),
                ctx->line_inc_off.as<uint32_t>(), n_lines, lines_dev, ctx->raster_bbox.as<int4>(),
                ctx->raster_keybase.as<uint64_t>(), ctx->keys.as<uint64_t>(), ctx->vals.as<uint32_t>(),
                ctx->bins.as<BinRec>(), ctx->incs.as<float2>(), queue, &ds->n_long, &ds->walk_ticket[1], refill));
        else if (long_blocks)
            OCHRE_LAUNCH(ctx, "dda_emit_long", side, k_line_emit_long<uint32_t><<<long_blocks, LONG_THREADS, 0, side>>>(
                ctx->lines.as<float4>(), ctx->line_raster.as<uint32_t>(), ctx->line_ent_off.as<uint32_t>(),
                ctx->line_inc_off.as<uint32_t>(), n_lines, lines_dev, ctx->raster_bbox.as<int4>(),
                ctx->raster_keybase.as<uint64_t>(), ctx->keys.as<uint32_t>(), ctx->vals.as<uint32_t>(),
                ctx->bins.as<BinRec>(), ctx->incs.as<float2>(), queue, &ds->n_long, &ds->walk_ticket[1], refill));
        if (ctx->keys64)
            OCHRE_LAUNCH(ctx, "dda_emit", s, k_line_emit<uint64_t><<<(unsigned)((n_lines + 255) / 256), 256, 0, s>>>(
                ctx->lines.as<float4>(), ctx->line_raster.as<uint32_t>(), ctx->line_ent_off.as<uint32_t>(),
                ctx->line_inc_off.as<uint32_t>(), n_lines, lines_dev, ctx->raster_bbox.as<int4>(),
                ctx->raster_keybase.as<uint64_t>(), ctx->keys.as<uint64_t>(), ctx->vals.as<uint32_t>(),
                ctx->bins.as<BinRec>(), ctx->incs.as<float2>(), long_cells));
        else
            OCHRE_LAUNCH(ctx, "dda_emit", s, k_line_emit<uint32_t><<<(unsigned)((n_lines + 255) / 256), 256, 0, s>>>(
                ctx->lines.as<float4>(), ctx->line_raster.as<uint32_t>(), ctx->line_ent_off.as<uint32_t>(),
                ctx->line_inc_off.as<uint32_t>(), n_lines, lines_dev, ctx->raster_bbox.as<int4>(),
                ctx->raster_keybase.as<uint64_t>(), ctx->keys.as<uint32_t>(), ctx->vals.as<uint32_t>(),
                ctx->bins.as<BinRec>(), ctx->incs.as<float2>(), long_cells));
        OCHRE_CUDA_TRY(cudaGetLastError());
        OCHRE_CUDA_TRY(join_walks(ctx, side, s));
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
