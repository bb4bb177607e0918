// Fused path for batches of small rasters, one warp per raster.
//
// Reference: Rasterizer::fill/command/move_to/line_to/finish
// (rasterizer.rs:61-268), PathCmd::transform/flatten (path.rs:16-109).
//
// Each warp of a persistent grid takes rasters by atomic ticket and runs the
// whole reference pipeline for one raster in its own slice of shared memory,
// synchronising only with __syncwarp (no block barrier couples it to the
// other warps of its CTA):
//   A. commands -> lines: rounds of 32 commands, one per lane; `last` and
//      `first` of every command by warp max-scans carried across rounds;
//      flatten counts (the serial t recurrence per curve), a warp scan, line
//      emission into shared memory.
//   B. the tile grid: the lines' end points' tile box plus one tile of
//      margin (GDIM x GDIM at most).
//   C. the pixel walk (the reference's exact DDA) of every line, lanes taking
//      lines from a queue as they finish their last one: each cell's
//      increment (area, height) is stored once (shared memory, then a per-warp
//      spill area in global memory), touched tiles are marked in a bitmap and
//      tile-row crossings appended to a list, slots allocated warp-wide by
//      ballot.
//   D. touched tiles compacted row-major (the reference's (tile_y, tile_x)
//      order); a tile is followed by a span when the next tile on its row
//      leaves a gap and the crossings with keys <= its own sum to a nonzero
//      winding.  The raster's tile and span counts are published, and the warp
//      helps turn published counts into inclusive output offsets.
//   E. coverage in groups of GROUP tiles: the stored increments of the group
//      are scatter-added into shared accumulators, then each lane shades one
//      pixel row of one tile (the reference's sequential accumulation along
//      the row, carried from tile to tile on a grid row); alpha goes to the
//      warp's staging slot.
//   F. the raster's output offsets (its own slot, usually made inclusive by
//      the helpers already, else a look-back), then the staged alpha, tile
//      positions and spans are written out.
// A raster beyond a limit (commands, lines, grid size, tiles, crossings,
// increments, a cell outside the grid) raises the fallback flag: the host
// then runs the CTA-per-raster kernel, and failing that the general chain.
#include <algorithm>

#include "common.cuh"
#include "fused.cuh"
#include "internal.h"

namespace ochre {

constexpr int WR_CMAX = 128;          // commands per raster (four rounds of 32)
constexpr int WR_LMAX = 256;          // lines per raster
constexpr int WR_GDIM = 32;           // grid side in tiles (one bitmap word per row)
constexpr int WR_TMAX = 128;          // touched tiles per raster
constexpr int WR_XMAX = 64;           // tile-row crossings per raster (two per lane)
constexpr int WR_GROUP = 8;           // tiles per coverage group
constexpr uint32_t WR_INC_MAX = 2048; // stored increments per raster (shared + spill)
// Accumulators of one tile: 64 area cells, then 64 height cells, row-major;
// pixel rows 4-7 sit 4 floats further on, so that the 16-byte row loads of
// eight lanes (rows 0-7 of one tile) fall in distinct bank groups.
constexpr int WR_ACC_H = 68;
constexpr int WR_ACC_STRIDE = 136;
__device__ __forceinline__ int wr_acc(int cell) { return cell + ((cell >> 5) << 2); }

template <int INC_S>
struct WarpSmem {
    union {
        float4 lines[WR_LMAX];                      // A -> C
        float acc[WR_GROUP][WR_ACC_STRIDE];         // E
    } u;
    float2 inc_ah[INC_S];      // stored increments: area, height
    uint16_t inc_id[INC_S];    // grid tile << 6 | cell (row-major 8x8)
    uint16_t tile_g[WR_TMAX];  // tile slot -> grid tile (row-major order)
    uint32_t touched[WR_GDIM]; // one word per grid row
    uint32_t cross[WR_XMAX];   // grid tile << 16 | sign (i16)
    uint32_t span_mask[WR_TMAX / 32];
    uint16_t row_base[WR_GDIM + 2];
};

template <int INC_S>
__host__ __device__ constexpr uint32_t wr_spill_per_warp() { return WR_INC_MAX - (uint32_t)INC_S; }

// Resident CTAs per SM that shared memory allows (about 214 KB of the 227 KB
// hold 7 CTAs of the 256-slot form, 6 of the larger ones); the register
// budget follows from it.
template <int INC_S>
__host__ __device__ constexpr int wr_min_ctas() { return INC_S <= 256 ? 7 : INC_S <= 384 ? 6 : 5; }

template <int WARPS, int INC_S>
__global__ void __launch_bounds__(WARPS * 32, wr_min_ctas<INC_S>()) k_raster_warp(FusedArgs A) {
    constexpr uint32_t FULL = 0xffffffffu;
    constexpr uint32_t SPILL = wr_spill_per_warp<INC_S>();
    __shared__ WarpSmem<INC_S> S_all[WARPS];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    WarpSmem<INC_S>& S = S_all[wid];
    const uint32_t gwarp = blockIdx.x * WARPS + wid;   // this warp's staging and spill slot
    const uint32_t lt = (1u << lane) - 1u;
    uint16_t* spill_id = A.spill_id + (size_t)gwarp * SPILL;
    float2* spill_ah = A.spill_ah + (size_t)gwarp * SPILL;
    // the command scan before this launch gave up a wait: its offsets are not valid
    if (run_aborted(A.err)) return;

    for (;;) {
        uint32_t r = 0, fb = 0;
        if (lane == 0) {
            r = atomicAdd(A.ticket, 1u);
            fb = ld_relaxed(A.fallback);
        }
        r = __shfl_sync(FULL, r, 0);
        if (r >= A.n_rasters) return;
        // the batch already falls back: skip the work, keep the output chain moving
        bool bail = __shfl_sync(FULL, fb, 0) != 0u;

        // ---------------- A. commands -> lines ----------------
        uint32_t f0, f1;
        if (A.raster_off) { f0 = __ldg(A.raster_off + r); f1 = __ldg(A.raster_off + r + 1); }
        else { f0 = r; f1 = r + 1; }
        const uint32_t c0 = __ldg(A.fill_off + f0), c1 = __ldg(A.fill_off + f1);
        const int n_cmd = (int)(c1 - c0);
        bail = bail || n_cmd > WR_CMAX;
        int n_lines = 0;
        V2 car_ep = v2(0, 0), car_mv = v2(0, 0);   // last non-Close end point / Move point so far
        bool invalid = false, capped = false;
        for (int base = 0; base < n_cmd && !bail; base += 32) {
            const int k = base + lane;
            const bool active = k < n_cmd;
            uint8_t verb = V_CLOSE;
            V2 pt0 = v2(0, 0), pt1 = v2(0, 0), pt2 = v2(0, 0);
            float wgt = 0.0f;
            if (active) {
                verb = __ldg(A.verbs + c0 + k);
                const uint32_t foff = __ldg(A.cmd_foff + c0 + k);
                uint32_t f = f0;
                if (f1 - f0 > 1) {   // the fill holding the command, within the raster's fills
                    uint32_t lo = f0, hi = f1;   // last f in [f0, f1) with fill_off[f] <= c0 + k
                    while (hi - lo > 1) {
                        const uint32_t mid = (lo + hi) >> 1;
                        if (__ldg(A.fill_off + mid) <= c0 + (uint32_t)k) lo = mid; else hi = mid;
                    }
                    f = lo;
                }
                const bool raw = A.fill_flags != nullptr && (__ldg(A.fill_flags + f) & OCHRE_FILL_RAW);
                const float* xf = A.fill_xf + 6 * (size_t)f;
                const float* fp = A.pts + foff;
                const int np = verb == V_MOVE || verb == V_LINE ? 1 : verb == V_QUAD || verb == V_CONIC ? 2
                             : verb == V_CUBIC ? 3 : 0;
                bool ok = !((uint64_t)foff + floats_per_verb(verb) > A.n_floats || verb > V_CLOSE);
                if (ok && np >= 1) pt0 = load_pt(fp);
                if (ok && np >= 2) pt1 = load_pt(fp + 2);
                if (ok && np >= 3) pt2 = load_pt(fp + 4);
                if (!raw) {   // PathCmd::transform (path.rs:16-37)
                    if (np >= 1) pt0 = xf_apply(xf, pt0);
                    if (np >= 2) pt1 = xf_apply(xf, pt1);
                    if (np >= 3) pt2 = xf_apply(xf, pt2);
                }
                if (!finite2(pt0) || !finite2(pt1) || !finite2(pt2)) ok = false;
                if (verb == V_CONIC && ok) {
                    wgt = __ldg(fp + 4);
                    if (!isfinite(wgt)) ok = false;
                }
                invalid = invalid || !ok;
            }
            const V2 ep = verb == V_CUBIC ? pt2 : (verb == V_QUAD || verb == V_CONIC) ? pt1 : pt0;
            // last: end point of the most recent earlier non-Close command;
            // first: point of the most recent earlier Move (rasterizer.rs:61-69, 145-157)
            int i_ep = active && verb != V_CLOSE ? lane : -1, i_mv = active && verb == V_MOVE ? lane : -1;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const int o_ep = __shfl_up_sync(FULL, i_ep, d), o_mv = __shfl_up_sync(FULL, i_mv, d);
                if (lane >= d) {
                    i_ep = max(i_ep, o_ep);
                    i_mv = max(i_mv, o_mv);
                }
            }
            int x_ep = __shfl_up_sync(FULL, i_ep, 1), x_mv = __shfl_up_sync(FULL, i_mv, 1);
            if (lane == 0) x_ep = x_mv = -1;
            const V2 from_ep = v2(__shfl_sync(FULL, ep.x, max(x_ep, 0)), __shfl_sync(FULL, ep.y, max(x_ep, 0)));
            const V2 from_mv = v2(__shfl_sync(FULL, ep.x, max(x_mv, 0)), __shfl_sync(FULL, ep.y, max(x_mv, 0)));
            const V2 last = x_ep >= 0 ? from_ep : car_ep;
            const V2 first = x_mv >= 0 ? from_mv : car_mv;
            const int t_ep = __shfl_sync(FULL, i_ep, 31), t_mv = __shfl_sync(FULL, i_mv, 31);
            const V2 round_ep = v2(__shfl_sync(FULL, ep.x, max(t_ep, 0)), __shfl_sync(FULL, ep.y, max(t_ep, 0)));
            const V2 round_mv = v2(__shfl_sync(FULL, ep.x, max(t_mv, 0)), __shfl_sync(FULL, ep.y, max(t_mv, 0)));
            if (t_ep >= 0) car_ep = round_ep;
            if (t_mv >= 0) car_mv = round_mv;
            // the raster's final implicit close (rasterizer.rs:181-183) is the
            // last command's last line
            const bool close_end = active && k == n_cmd - 1 && !veq(car_ep, car_mv);
            int n_l = 0;
            if (active) {
                bool cap = false;
                switch (verb) {
                case V_MOVE: n_l = veq(last, first) ? 0 : 1; break;
                case V_LINE: n_l = 1; break;
                case V_QUAD: n_l = (int)flatten_steps(quad_dt(last, pt0, pt1), &cap); break;
                case V_CUBIC: n_l = (int)flatten_steps(cubic_dt(last, pt0, pt1, pt2), &cap); break;
                case V_CONIC: {
                    int n = 0;
                    conic_flatten(last, pt0, pt1, wgt, &cap, [&](V2) { n++; });
                    n_l = n;
                    break;
                }
                default: break;
                }
                if (close_end) n_l++;
                capped = capped || cap;
                if (n_l > WR_LMAX) n_l = WR_LMAX + 1;
            }
            int off = n_l;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const int o = __shfl_up_sync(FULL, off, d);
                if (lane >= d) off += o;
            }
            const int total = __shfl_sync(FULL, off, 31);
            off -= n_l;
            if (n_lines + total > WR_LMAX) {
                bail = true;
                break;
            }
            if (active && n_l > 0) {
                // emit (path.rs:49-104; closing lines rasterizer.rs:62-64, 181-183)
                int o = n_lines + off;
                const int o_end = o + n_l;
                V2 prev = last;
                auto put = [&](V2 a, V2 b) {
                    if (o < o_end) S.u.lines[o++] = make_float4(a.x, a.y, b.x, b.y);
                };
                auto to = [&](V2 p) { put(prev, p); prev = p; };
                bool cap = false;
                switch (verb) {
                case V_MOVE: if (!veq(last, first)) put(last, first); break;
                case V_LINE: to(pt0); break;
                case V_QUAD: {
                    const float dt = quad_dt(last, pt0, pt1);
                    float t = 0.0f;
                    while (t < 1.0f && o < o_end) {
                        t = rmin(__fadd_rn(t, dt), 1.0f);
                        to(quad_point(t, last, pt0, pt1));
                    }
                    break;
                }
                case V_CUBIC: {
                    const float dt = cubic_dt(last, pt0, pt1, pt2);
                    float t = 0.0f;
                    while (t < 1.0f && o < o_end) {
                        t = rmin(__fadd_rn(t, dt), 1.0f);
                        to(cubic_point(t, last, pt0, pt1, pt2));
                    }
                    break;
                }
                case V_CONIC: conic_flatten(last, pt0, pt1, wgt, &cap, to); break;
                default: break;
                }
                if (close_end) {
                    o = o_end - 1;
                    put(car_ep, car_mv);
                }
            }
            n_lines += total;
        }
        if (invalid) atomicOr(A.err, ERR_INVALID);
        if (capped) atomicOr(A.err, ERR_LIMIT);
        __syncwarp();

        // ---------------- B. the tile grid ----------------
        int gx0 = 0, gy0 = 0, gw = 0, gh = 0;
        if (!bail) {
            int x0 = 0x7fffffff, y0 = 0x7fffffff, x1 = (int)0x80000000, y1 = (int)0x80000000;
            for (int l = lane; l < n_lines; l += 32) {
                const float4 L = S.u.lines[l];
                const int ax = div8(f2i16(floorf(L.x))), ay = div8(f2i16(floorf(L.y)));
                const int px = div8(f2i16(floorf(L.z))), py = div8(f2i16(floorf(L.w)));
                x0 = min(x0, min(ax, px));
                y0 = min(y0, min(ay, py));
                x1 = max(x1, max(ax, px));
                y1 = max(y1, max(ay, py));
            }
            x0 = __reduce_min_sync(FULL, x0);
            y0 = __reduce_min_sync(FULL, y0);
            x1 = __reduce_max_sync(FULL, x1);
            y1 = __reduce_max_sync(FULL, y1);
            if (x0 > x1) { x0 = 0; y0 = 0; x1 = 0; y1 = 0; }   // no lines: the (0,0) tile
            gx0 = x0 - 1;
            gy0 = y0 - 1;
            gw = x1 - x0 + 3;
            gh = y1 - y0 + 3;
            bail = gw > WR_GDIM || gh > WR_GDIM;
            S.touched[lane] = 0u;
        }
        __syncwarp();

        // ---------------- C. pixel walks: increments, touched tiles, crossings ----------------
        uint32_t n_inc = 0, n_cross = 0;
        if (!bail) {
            bool out = false, lim = false;
            Walk w;
            WalkState s;
            int ty_prev = 0, last_g = -1;
            uint32_t steps = 0;
            bool have = false;
            int next = 0;
            for (;;) {
                const uint32_t m_need = __ballot_sync(FULL, !have);
                if (next >= n_lines && m_need == FULL) break;
                if (next < n_lines && m_need != 0u) {
                    if (!have) {
                        const int idx = next + __popc(m_need & lt);
                        if (idx < n_lines) {
                            const float4 L = S.u.lines[idx];
                            if (!(L.x == L.z && L.y == L.w)) {   // rasterizer.rs:73
                                walk_setup(v2(L.x, L.y), v2(L.z, L.w), w, s);
                                ty_prev = div8(s.y);   // == floor(last.y) as i16 div 8, see dda.cu
                                last_g = -1;
                                steps = 0;
                                have = true;
                            }
                        }
                    }
                    next += __popc(m_need);
                }
                // the increment of the current cell (rasterizer.rs:97-106)
                bool has_inc = false;
                uint32_t id = 0;
                float area = 0.0f, height = 0.0f;
                if (have) {
                    walk_increment(w, s, area, height);
                    const int gx = div8(s.x) - gx0, gy = div8(s.y) - gy0;
                    if ((unsigned)gx >= (unsigned)gw || (unsigned)gy >= (unsigned)gh) {
                        out = true;
                    } else {
                        const int g = gy * WR_GDIM + gx;
                        if (g != last_g) {
                            atomicOr(&S.touched[gy], 1u << gx);
                            last_g = g;
                        }
                        id = ((uint32_t)g << 6) | (uint32_t)(((s.y & 7) << 3) | (s.x & 7));
                        has_inc = true;
                    }
                }
                const uint32_t m_inc = __ballot_sync(FULL, has_inc);
                if (has_inc) {
                    const uint32_t q = n_inc + __popc(m_inc & lt);
                    if (q < (uint32_t)INC_S) {
                        S.inc_id[q] = (uint16_t)id;
                        S.inc_ah[q] = make_float2(area, height);
                    } else if (q < WR_INC_MAX) {
                        spill_id[q - INC_S] = (uint16_t)id;
                        spill_ah[q - INC_S] = make_float2(area, height);
                    } else {
                        out = true;
                    }
                }
                n_inc += __popc(m_inc);
                // step; tile-row crossing of the new cell (rasterizer.rs:108-131)
                bool has_x = false;
                uint32_t xv = 0;
                if (have) {
                    const bool done = walk_step(w, s);
                    const int ty = div8(s.y);
                    if (ty != ty_prev) {
                        const int cgx = div8(s.x) - gx0, cgy = min(ty_prev, ty) - gy0;
                        if ((unsigned)cgx >= (unsigned)gw || (unsigned)cgy >= (unsigned)gh) {
                            out = true;
                        } else {
                            const int sign = (int)(int8_t)(int16_t)(ty - ty_prev);
                            xv = ((uint32_t)(cgy * WR_GDIM + cgx) << 16) | ((uint32_t)sign & 0xffffu);
                            has_x = true;
                        }
                        ty_prev = ty;
                    }
                    if (done) {
                        have = false;
                    } else if (++steps >= WALK_CAP) {
                        lim = true;
                        out = true;
                        have = false;
                    }
                }
                const uint32_t m_x = __ballot_sync(FULL, has_x);
                if (has_x) {
                    const uint32_t q = n_cross + __popc(m_x & lt);
                    if (q < (uint32_t)WR_XMAX) S.cross[q] = xv;
                    else out = true;
                }
                n_cross += __popc(m_x);
                if (__any_sync(FULL, out)) break;
            }
            if (lim) atomicOr(A.err, ERR_LIMIT);
            bail = __any_sync(FULL, out);
        }
        __syncwarp();

        // ---------------- D. compaction (row-major), spans ----------------
        int n_real = 0, n_spans = 0;
        if (!bail) {
            const uint32_t bits = S.touched[lane];
            const int cnt = __popc(bits);
            int inc = cnt;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const int o = __shfl_up_sync(FULL, inc, d);
                if (lane >= d) inc += o;
            }
            n_real = __shfl_sync(FULL, inc, 31);
            S.row_base[lane] = (uint16_t)(inc - cnt);
            if (lane == 31) S.row_base[WR_GDIM] = (uint16_t)inc;
            if (n_real > WR_TMAX) {
                bail = true;
            } else {
                int slot = inc - cnt;
                uint32_t b = bits;
                while (b) {
                    const int gx = __ffs(b) - 1;
                    b &= b - 1;
                    S.tile_g[slot++] = (uint16_t)(lane * WR_GDIM + gx);
                }
                __syncwarp();
                // spans (rasterizer.rs:252-265): the running winding before a
                // gap is the sum of the crossings with keys <= the tile's
                const uint32_t xa = lane < (int)n_cross ? S.cross[lane] : 0xffff0000u;
                const uint32_t xb = lane + 32 < (int)n_cross ? S.cross[lane + 32] : 0xffff0000u;
                for (int base = 0; base < n_real; base += 32) {
                    const int t = base + lane;
                    bool cand = false;
                    int g = 0;
                    if (t < n_real) {
                        g = S.tile_g[t];
                        const int gy = g >> 5, gx = g & 31;
                        const uint32_t right = gx == 31 ? 0u : S.touched[gy] >> (gx + 1);
                        cand = right != 0u && !(right & 1u);
                    }
                    uint32_t mc = __ballot_sync(FULL, cand), mspan = 0;
                    while (mc) {
                        const int j = __ffs(mc) - 1;
                        mc &= mc - 1;
                        const int gj = __shfl_sync(FULL, g, j);
                        int ws = ((int)(xa >> 16) <= gj ? (int)(int16_t)(xa & 0xffffu) : 0) +
                                 ((int)(xb >> 16) <= gj ? (int)(int16_t)(xb & 0xffffu) : 0);
                        ws = __reduce_add_sync(FULL, ws);
                        if (ws != 0) mspan |= 1u << j;
                    }
                    if (lane == 0) S.span_mask[base >> 5] = mspan;
                    n_spans += __popc(mspan);
                }
            }
        }
        const int n_tiles = n_real == 0 ? 1 : n_real;   // rasterizer.rs:194-208
        // The raster's counts go out now; its offsets are resolved after the
        // coverage, by when the helpers have usually made its slot inclusive.
        if (lane == 0) {
            chain_publish(A.co, r, bail ? 0u : (uint32_t)n_tiles, bail ? 0u : (uint32_t)n_spans);
            if (bail) atomicOr(A.fallback, 1u);
        }
        __syncwarp();
        frontier_help(A.co, A.frontier, A.n_rasters);

        // ---------------- E. coverage, GROUP tiles at a time ----------------
        // Alpha (and coverage) of tile i of the raster are staged at
        // (gwarp * WR_TMAX + i) * 64.
        if (!bail && n_real > 0) {
            const size_t stage0 = (size_t)gwarp * WR_TMAX;
            const int y = lane & 7, gq = lane >> 3;   // this lane: pixel row y of the gq-th tile of a pass
            float carry_row = 0.0f;                    // carry into the next pass's first tile, row y
            for (int lo = 0; lo < n_real; lo += WR_GROUP) {
                const int nch = min(WR_GROUP, n_real - lo);
                const int g_lo = S.tile_g[lo], g_hi = S.tile_g[lo + nch - 1];
                float4* accv = reinterpret_cast<float4*>(&S.u.acc[0][0]);
                for (int q = lane; q < nch * (WR_ACC_STRIDE / 4); q += 32) accv[q] = make_float4(0.f, 0.f, 0.f, 0.f);
                __syncwarp();
                // scatter-add the group's increments (rasterizer.rs:223-228)
                for (uint32_t q = lane; q < n_inc; q += 32) {
                    const uint32_t id = q < (uint32_t)INC_S ? S.inc_id[q] : spill_id[q - INC_S];
                    const int g = (int)(id >> 6);
                    if (g < g_lo || g > g_hi) continue;
                    const float2 ah = q < (uint32_t)INC_S ? S.inc_ah[q] : spill_ah[q - INC_S];
                    const int gy = g >> 5, gx = g & 31;
                    const int i = S.row_base[gy] + __popc(S.touched[gy] & ((1u << gx) - 1u)) - lo;
                    const int cell = (int)(id & 63u);
                    atomicAdd(&S.u.acc[i][wr_acc(cell)], ah.x);
                    atomicAdd(&S.u.acc[i][WR_ACC_H + wr_acc(cell)], ah.y);
                }
                __syncwarp();
                // shade (rasterizer.rs:230-250): along its row a lane adds the
                // cells in the reference's order; the carry into a tile is the
                // carry into the previous tile of the grid row plus that tile's
                // row sum (reset at each grid row), a segmented scan over the
                // four tiles of a pass
                for (int p0 = 0; p0 < nch; p0 += 4) {
                    const int i = p0 + gq;
                    const bool valid = i < nch;
                    const int t = lo + i;
                    float a[8], h[8];
                    if (valid) {
                        const float* ac = S.u.acc[i];
                        const float4 a0 = *reinterpret_cast<const float4*>(ac + wr_acc(8 * y));
                        const float4 a1 = *reinterpret_cast<const float4*>(ac + wr_acc(8 * y + 4));
                        const float4 h0 = *reinterpret_cast<const float4*>(ac + WR_ACC_H + wr_acc(8 * y));
                        const float4 h1 = *reinterpret_cast<const float4*>(ac + WR_ACC_H + wr_acc(8 * y + 4));
                        a[0] = a0.x; a[1] = a0.y; a[2] = a0.z; a[3] = a0.w; a[4] = a1.x; a[5] = a1.y; a[6] = a1.z; a[7] = a1.w;
                        h[0] = h0.x; h[1] = h0.y; h[2] = h0.z; h[3] = h0.w; h[4] = h1.x; h[5] = h1.y; h[6] = h1.z; h[7] = h1.w;
                    } else {
#pragma unroll
                        for (int c = 0; c < 8; c++) a[c] = h[c] = 0.0f;
                    }
                    const float rs = ((h[0] + h[1]) + (h[2] + h[3])) + ((h[4] + h[5]) + (h[6] + h[7]));
                    const bool head = valid && (t == 0 || (S.tile_g[t] >> 5) != (S.tile_g[t - 1] >> 5));
                    float v = rs;
                    bool fl = head;
#pragma unroll
                    for (int d = 8; d < 32; d <<= 1) {
                        const float vo = __shfl_up_sync(FULL, v, d);
                        const bool fo = __shfl_up_sync(FULL, fl ? 1 : 0, d) != 0;
                        if (lane >= d) {
                            if (!fl) v = vo + v;
                            fl = fl || fo;
                        }
                    }
                    float ex = __shfl_up_sync(FULL, v, 8);
                    bool exf = __shfl_up_sync(FULL, fl ? 1 : 0, 8) != 0;
                    if (gq == 0) {
                        ex = 0.0f;
                        exf = false;
                    }
                    const float carry = head ? 0.0f : (exf ? ex : carry_row + ex);
                    carry_row = __shfl_sync(FULL, carry + rs, 24 + y);
                    if (valid) {
                        float accum = carry;
                        uint32_t lo4 = 0, hi4 = 0;
                        float cv[8];
#pragma unroll
                        for (int c = 0; c < 8; c++) {
                            const float cov = fabsf(accum + a[c]);
                            cv[c] = cov;
                            const uint32_t al = f2u8(rmin(cov * 256.0f, 255.0f));
                            if (c < 4) lo4 |= al << (8 * c); else hi4 |= al << (8 * (c - 4));
                            accum = accum + h[c];
                        }
                        const size_t st = stage0 + (size_t)t;
                        reinterpret_cast<uint2*>(A.stage_alpha + st * 64)[y] = make_uint2(lo4, hi4);
                        if (A.out_cov) {
                            float4* o = reinterpret_cast<float4*>(A.stage_cov + st * 64 + 8 * y);
                            o[0] = make_float4(cv[0], cv[1], cv[2], cv[3]);
                            o[1] = make_float4(cv[4], cv[5], cv[6], cv[7]);
                        }
                    }
                }
                __syncwarp();
            }
        }

        // ---------------- F. offsets, then every output of the raster ----------------
        {
            const uint32_t a0 = bail ? 0u : (uint32_t)n_tiles, a1 = bail ? 0u : (uint32_t)n_spans;
            uint64_t own = 0;
            if (lane == 0) own = ld_relaxed64(A.co + r);
            own = __shfl_sync(FULL, own, 0);
            if ((own >> 62) != 2u) {
                frontier_help(A.co, A.frontier, A.n_rasters);
                if (lane == 0) own = ld_relaxed64(A.co + r);
                own = __shfl_sync(FULL, own, 0);
            }
            uint32_t p0, p1;
            if ((own >> 62) == 2u) {
                p0 = (uint32_t)(own & CH_MAX) - a0;
                p1 = (uint32_t)((own >> 30) & CH_MAX) - a1;
            } else {
                chain_lookback(A.co, r, a0, a1, A.err, p0, p1);
            }
            if (!bail) {
                if (lane == 0) {
                    A.raster_tile_off[r] = p0;
                    A.raster_span_off[r] = p1;
                    if (r + 1 == A.n_rasters) {
                        A.raster_tile_off[r + 1] = p0 + n_tiles;
                        A.raster_span_off[r + 1] = p1 + n_spans;
                        A.totals[0] = p0 + n_tiles;
                        A.totals[1] = p1 + n_spans;
                    }
                }
                if ((uint64_t)p0 + n_tiles > A.tile_cap || (uint64_t)p1 + n_spans > A.span_cap) {
                    if (lane == 0) atomicOr(A.err, ERR_CAPACITY);
                } else if (n_real == 0) {
                    // no increments: one all-zero tile at (0, 0)
                    if (lane < 16) reinterpret_cast<uint32_t*>(A.out_alpha + (size_t)p0 * 64)[lane] = 0u;
                    if (A.out_cov) {
                        A.out_cov[(size_t)p0 * 64 + lane] = 0.0f;
                        A.out_cov[(size_t)p0 * 64 + 32 + lane] = 0.0f;
                    }
                    if (lane == 0) A.out_xy[p0] = 0u;
                } else {
                    const size_t stage0 = (size_t)gwarp * WR_TMAX;
                    const uint2* sa = reinterpret_cast<const uint2*>(A.stage_alpha + stage0 * 64);
                    uint2* da = reinterpret_cast<uint2*>(A.out_alpha + (size_t)p0 * 64);
                    for (int q = lane; q < n_real * 8; q += 32) da[q] = sa[q];
                    if (A.out_cov) {
                        const float2* sc = reinterpret_cast<const float2*>(A.stage_cov + stage0 * 64);
                        float2* dc = reinterpret_cast<float2*>(A.out_cov + (size_t)p0 * 64);
                        for (int q = lane; q < n_real * 32; q += 32) dc[q] = sc[q];
                    }
                    for (int t = lane; t < n_real; t += 32) {
                        const int g = S.tile_g[t];
                        const int tx = gx0 + (g & 31), ty = gy0 + (g >> 5);
                        A.out_xy[p0 + t] = (uint32_t)(uint16_t)(int16_t)(tx * 8) |
                                           ((uint32_t)(uint16_t)(int16_t)(ty * 8) << 16);
                        const uint32_t m = S.span_mask[t >> 5];
                        if (m >> (t & 31) & 1u) {
                            // span rank: the span tiles before t (tile order = callback order)
                            int sr = __popc(m & ((1u << (t & 31)) - 1u));
                            for (int k = 0; k < (t >> 5); k++) sr += __popc(S.span_mask[k]);
                            const uint32_t right = S.touched[g >> 5] >> ((g & 31) + 1);
                            const int gap = __ffs(right) - 1;
                            A.span_xy[p1 + sr] = (uint32_t)(uint16_t)(int16_t)((tx + 1) * 8) |
                                                 ((uint32_t)(uint16_t)(int16_t)(ty * 8) << 16);
                            A.span_w[p1 + sr] = (uint16_t)((uint16_t)gap * 8u);
                            A.span_tile[p1 + sr] = p0 + t;
                        }
                    }
                }
            }
        }
        __syncwarp();
    }
}

template <int WARPS, int INC_S>
static int warp_full_grid() {
    static int grid = 0;
    if (grid == 0) {
        int dev = 0, sms = 0, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_raster_warp<WARPS, INC_S>, WARPS * 32, 0);
        grid = sms * (per > 0 ? per : 1);
    }
    return grid;
}

constexpr int WR_WARPS = 4;   // rasters (warps) per CTA

// The tuned increment slots: with a == nullptr, the full grid (CTAs) and the
// spill size per warp; else one launch over `grid` CTAs.
static int warp_shape(ochre_gpu_ctx* ctx, const FusedArgs* a, int* grid, uint32_t* spill, cudaStream_t s) {
#define OCHRE_WARP_CASE(I)                                                                          \
    case I:                                                                                         \
        if (!a) {                                                                                   \
            *grid = warp_full_grid<WR_WARPS, I>();                                                  \
            *spill = wr_spill_per_warp<I>();                                                        \
            return OCHRE_OK;                                                                        \
        }                                                                                           \
        OCHRE_LAUNCH(ctx, "raster_warp", s, k_raster_warp<WR_WARPS, I><<<*grid, WR_WARPS * 32, 0, s>>>(*a)); \
        OCHRE_CUDA_TRY(cudaGetLastError());                                                         \
        return OCHRE_OK;
    switch (ctx->tune_fused_warp_inc) {
        OCHRE_WARP_CASE(256)
        OCHRE_WARP_CASE(384)
        OCHRE_WARP_CASE(512)
    default: return OCHRE_E_INVALID;
    }
#undef OCHRE_WARP_CASE
}

int fused_warp_prepare(ochre_gpu_ctx* ctx, uint32_t n_rasters, int* grid_ctas, bool want_cov) {
    int grid = 0;
    uint32_t spill = 0;
    const int st = warp_shape(ctx, nullptr, &grid, &spill, nullptr);
    if (st != OCHRE_OK) return st;
    // no more warps than rasters
    uint32_t ctas = (uint32_t)std::min<uint64_t>((uint64_t)grid, ((uint64_t)n_rasters + WR_WARPS - 1) / WR_WARPS);
    if (ctx->fused_max_warps) ctas = std::min<uint32_t>(ctas, std::max<uint32_t>(1u, ctx->fused_max_warps / WR_WARPS));
    *grid_ctas = (int)ctas;
    const size_t warps = (size_t)ctas * WR_WARPS;
    OCHRE_CUDA_TRY(ctx->fused_stage.ensure(warps * WR_TMAX * 64 * (want_cov ? 5 : 1)));
    OCHRE_CUDA_TRY(ctx->fused_spill.ensure(warps * spill * (sizeof(uint16_t) + sizeof(float2)) + 16));
    return OCHRE_OK;
}

int fused_warp_launch(ochre_gpu_ctx* ctx, FusedArgs* a, int grid_ctas, bool want_cov, cudaStream_t s) {
    int g = 0;
    uint32_t spill = 0;
    int st = warp_shape(ctx, nullptr, &g, &spill, nullptr);
    if (st != OCHRE_OK) return st;
    const size_t warps = (size_t)grid_ctas * WR_WARPS;
    a->stage_alpha = ctx->fused_stage.as<uint8_t>();
    a->stage_cov = want_cov ? reinterpret_cast<float*>(ctx->fused_stage.as<uint8_t>() + warps * WR_TMAX * 64) : nullptr;
    // spill: the float2 part first (8-byte aligned), then the ids
    a->spill_ah = reinterpret_cast<float2*>(ctx->fused_spill.p);
    a->spill_id = reinterpret_cast<uint16_t*>(ctx->fused_spill.as<uint8_t>() + warps * spill * sizeof(float2));
    return warp_shape(ctx, a, &grid_ctas, &spill, s);
}

}  // namespace ochre
