// Fused path for batches of small rasters (glyph-sized paths): one CTA per
// raster does the whole reference pipeline on chip.
//
// Reference: Rasterizer::fill/command/move_to/line_to/finish
// (rasterizer.rs:61-268), PathCmd::transform/flatten (path.rs:16-109).
//
// Before the launch a command scan gives every command's float offset.
// Per raster (CTA of FUSED_THREADS threads, rasters taken in index order by
// atomic ticket):
//   A. commands -> lines in shared memory: points at the scanned float
//      offsets; `last` / `first` of every command by block max-scans; flatten
//      counts (the serial t recurrence per curve) -> line offsets -> line
//      emission.
//   B. a GDIM x GDIM tile grid around the lines' end points (one tile of
//      margin); a count walk per line (the reference's exact DDA) marks
//      touched tiles in a bitmap, appends tile-row crossings to a list and
//      records each line's range of grid tiles.  Touched tiles are compacted
//      row-major (the reference's (tile_y, tile_x) order).  A tile is
//      followed by a span when the next tile on its row leaves a gap and the
//      crossings with keys <= its own sum to a nonzero winding (the
//      reference's running winding over its sorted TileIncrements).  The
//      raster's tile and span counts are published (look-back aggregate).
//   C. tiles in chunks of CHUNK: the lines touching a chunk are walked again
//      and their increments scatter-added into shared per-tile accumulators;
//      row sums give the carries along grid rows; alpha goes to the CTA's
//      staging slot.
//   D. the raster's output offsets are resolved by decoupled look-back (the
//      predecessors published their counts while this raster ran C), and
//      the staged alpha, the tile positions and the spans are written out.
// Any limit exceeded (commands, lines, grid size, tiles, crossings, a cell
// outside the grid) raises the fallback flag: the host then
// runs the general chain for the whole batch.  Every wait is bounded.
#include <algorithm>

#include "common.cuh"
#include "internal.h"
#include "scan.cuh"
#include "fused.cuh"

namespace ochre {

// Kernel shape (template parameters, chosen by the autotuner):
//   THREADS  threads per raster (= max commands per raster), 64, 96 or 128;
//   CHUNK    tiles accumulated per pass (shared accumulators of CHUNK x 512 B).
constexpr int F_LMAX = 256;             // lines per raster
constexpr int GDIM = 32;                // grid side in tiles (one bitmap word per row)
constexpr int F_TMAX = 128;             // touched tiles per raster
constexpr int F_XMAX = 256;             // tile-row crossings per raster
// Resident CTAs per SM the register budget keeps (the shared memory of the
// 16-tile chunk shapes allows about 14): 64 threads 14, 96 threads 12, 128
// threads 9.
__host__ __device__ constexpr int fused_min_ctas(int threads) { return threads <= 64 ? 14 : threads <= 96 ? 12 : 9; }

template <int THREADS, int CHUNK>
struct FusedSmem {
    float4 lines[F_LMAX];
    // The coverage accumulators and the data of the earlier phases are
    // never live together: they share storage (more CTAs per SM).
    struct Early {
        V2 ep[THREADS];            // transformed end point (or Move point) per command
        uint32_t cross[F_XMAX];    // grid tile << 16 | sign (i16)
    };
    union {
        float acc[CHUNK][128];     // [tile][64 area | 64 height]
        Early early;
    } u;
    uint16_t line_g0[F_LMAX], line_g1[F_LMAX];   // grid-tile range of each line's cells
    uint16_t tile_g[F_TMAX];       // tile slot -> grid tile (row-major order)
    uint32_t touched[GDIM];        // one word per grid row
    uint32_t span_mask[F_TMAX / 32];   // tile slot t is followed by a span
    uint16_t row_base[GDIM + 1];   // first tile slot of each grid row
    float rs[CHUNK][8];
    float carry[CHUNK][8];
    float pend[8];                 // running carry of the row continuing into the next chunk
    int32_t warp_tmp[THREADS / 32][4];
    uint32_t raster;
    uint32_t flag;                 // per-raster fallback
    uint32_t n_cross;
    uint32_t tile_base, span_base;
    int32_t gx0, gy0, gw, gh;
};

// ---- block-wide scans over WARPS * 32 threads (one value each) ----
template <int WARPS>
__device__ __forceinline__ int block_excl_sum(int v, int& total, int32_t (*tmp)[4]) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int inc = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int o = __shfl_up_sync(0xffffffffu, inc, d);
        if (lane >= d) inc += o;
    }
    __syncthreads();
    if (lane == 31) tmp[w][0] = inc;
    __syncthreads();
    int base = 0, tot = 0;
#pragma unroll
    for (int k = 0; k < WARPS; k++) {
        const int t = tmp[k][0];
        if (k < w) base += t;
        tot += t;
    }
    total = tot;
    return base + inc - v;
}
// Two exclusive max-scans at once (values >= -1, identity -1): one pair of
// barriers for both.
template <int WARPS>
__device__ __forceinline__ void block_excl_max2(int a, int b, int& a_ex, int& b_ex, int& a_last, int& b_last,
                                                int32_t (*tmp)[4]) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int ia = a, ib = b;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int oa = __shfl_up_sync(0xffffffffu, ia, d);
        const int ob = __shfl_up_sync(0xffffffffu, ib, d);
        if (lane >= d) {
            ia = max(ia, oa);
            ib = max(ib, ob);
        }
    }
    __syncthreads();
    if (lane == 31) {
        tmp[w][1] = ia;
        tmp[w][2] = ib;
    }
    __syncthreads();
    int base_a = -1, base_b = -1, tot_a = -1, tot_b = -1;
#pragma unroll
    for (int k = 0; k < WARPS; k++) {
        const int ta = tmp[k][1], tb = tmp[k][2];
        if (k < w) {
            base_a = max(base_a, ta);
            base_b = max(base_b, tb);
        }
        tot_a = max(tot_a, ta);
        tot_b = max(tot_b, tb);
    }
    a_last = tot_a;
    b_last = tot_b;
    int ea = __shfl_up_sync(0xffffffffu, ia, 1), eb = __shfl_up_sync(0xffffffffu, ib, 1);
    if (lane == 0) ea = eb = -1;
    a_ex = max(base_a, ea);
    b_ex = max(base_b, eb);
}



template <int THREADS, int CHUNK>
__global__ void __launch_bounds__(THREADS, fused_min_ctas(THREADS)) k_raster_fused(FusedArgs A) {
    constexpr int FUSED_THREADS = THREADS;
    constexpr int F_WARPS = THREADS / 32;
    constexpr int F_CMAX = THREADS;   // commands per raster
    __shared__ FusedSmem<THREADS, CHUNK> S;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    // the command scan before this launch gave up a wait: its offsets are not valid
    if (run_aborted(A.err)) return;
    for (;;) {
        if (tid == 0) {
            S.raster = atomicAdd(A.ticket, 1u);
            // batch already falls back: skip the work, keep the output chain moving
            S.flag = ld_relaxed(A.fallback) != 0u ? 1u : 0u;
            S.n_cross = 0;
        }
        __syncthreads();
        const uint32_t r = S.raster;
        if (r >= A.n_rasters) return;

        // ---------------- A. commands -> lines ----------------
        uint32_t f0, f1;
        if (A.raster_off) { f0 = __ldg(A.raster_off + r); f1 = __ldg(A.raster_off + r + 1); }
        else { f0 = r; f1 = r + 1; }
        const uint32_t c0 = __ldg(A.fill_off + f0), c1 = __ldg(A.fill_off + f1);
        const int n_cmd = (int)(c1 - c0);
        bool bail = S.flag != 0 || n_cmd > F_CMAX;

        uint8_t verb = V_CLOSE;
        V2 pt0 = v2(0, 0), pt1 = v2(0, 0), pt2 = v2(0, 0);
        float wgt = 0.0f;
        float dt = 0.0f;   // a curve's parameter step, kept for the emission
        int n_lines_cmd = 0;
        V2 last = v2(0, 0), first = v2(0, 0);
        bool is_last_cmd = false;
        V2 last_end = v2(0, 0), first_end = v2(0, 0);
        if (!bail) {
            const bool active = tid < n_cmd;
            verb = active ? __ldg(A.verbs + c0 + tid) : V_CLOSE;
            const uint32_t foff = active ? __ldg(A.cmd_foff + c0 + tid) : 0u;
            bool ok = true;
            if (active) {
                uint32_t f = f0;
                if (f1 - f0 > 1) f = upper_bound_u32(A.fill_off, A.n_fills + 1, c0 + tid) - 1u;
                const bool raw = A.fill_flags != nullptr && (__ldg(A.fill_flags + f) & OCHRE_FILL_RAW);
                const float* xf = A.fill_xf + 6 * (size_t)f;
                const float* fp = A.pts + foff;
                const int np = verb == V_MOVE || verb == V_LINE ? 1 : verb == V_QUAD || verb == V_CONIC ? 2
                             : verb == V_CUBIC ? 3 : 0;
                if ((uint64_t)foff + floats_per_verb(verb) > A.n_floats || verb > V_CLOSE) ok = false;
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
                S.u.early.ep[tid] = verb == V_CUBIC ? pt2 : (verb == V_QUAD || verb == V_CONIC) ? pt1 : pt0;
            }
            if (!ok) atomicOr(A.err, ERR_INVALID);
            // last: endpoint of the most recent earlier non-Close command;
            // first: point of the most recent earlier Move.
            int ep_last, mv_last, ep_ex, mv_ex;
            block_excl_max2<F_WARPS>(active && verb != V_CLOSE ? tid : -1, active && verb == V_MOVE ? tid : -1, ep_ex,
                                     mv_ex, ep_last, mv_last, S.warp_tmp);
            if (active) {
                last = ep_ex >= 0 ? S.u.early.ep[ep_ex] : v2(0, 0);
                first = mv_ex >= 0 ? S.u.early.ep[mv_ex] : v2(0, 0);
                is_last_cmd = tid == n_cmd - 1;
                if (is_last_cmd) {
                    last_end = ep_last >= 0 ? S.u.early.ep[ep_last] : v2(0, 0);
                    first_end = mv_last >= 0 ? S.u.early.ep[mv_last] : v2(0, 0);
                }
                bool capped = false;
                switch (verb) {
                case V_MOVE: n_lines_cmd = veq(last, first) ? 0 : 1; break;
                case V_LINE: n_lines_cmd = 1; break;
                case V_QUAD:
                    dt = quad_dt(last, pt0, pt1);
                    n_lines_cmd = (int)flatten_steps(dt, &capped);
                    break;
                case V_CUBIC:
                    dt = cubic_dt(last, pt0, pt1, pt2);
                    n_lines_cmd = (int)flatten_steps(dt, &capped);
                    break;
                case V_CONIC: {
                    int n = 0;
                    conic_flatten(last, pt0, pt1, wgt, &capped, [&](V2) { n++; });
                    n_lines_cmd = n;
                    break;
                }
                default: break;
                }
                if (is_last_cmd && !veq(last_end, first_end)) n_lines_cmd++;
                if (capped) atomicOr(A.err, ERR_LIMIT);
                if (n_lines_cmd > F_LMAX) n_lines_cmd = F_LMAX + 1;
            }
        }
        // (block_excl_sum's own barriers order the end-point reads above)
        int n_lines = 0;
        int loff = 0;
        if (!bail) {
            loff = block_excl_sum<F_WARPS>(n_lines_cmd, n_lines, S.warp_tmp);
            if (n_lines > F_LMAX) bail = true;
        }
        if (!bail && tid < n_cmd) {
            // emit (path.rs:49-104; closing lines rasterizer.rs:62-64, 181-183)
            int o = loff;
            const int o_end = loff + n_lines_cmd;
            V2 prev = last;
            auto put = [&](V2 a, V2 b) {
                if (o < o_end) S.lines[o++] = make_float4(a.x, a.y, b.x, b.y);
            };
            auto to = [&](V2 p) { put(prev, p); prev = p; };
            bool capped = false;
            switch (verb) {
            case V_MOVE: if (!veq(last, first)) put(last, first); break;
            case V_LINE: to(pt0); break;
            case V_QUAD: {
                float t = 0.0f;
                while (t < 1.0f && o < o_end) {
                    t = rmin(__fadd_rn(t, dt), 1.0f);
                    to(quad_point(t, last, pt0, pt1));
                }
                break;
            }
            case V_CUBIC: {
                float t = 0.0f;
                while (t < 1.0f && o < o_end) {
                    t = rmin(__fadd_rn(t, dt), 1.0f);
                    to(cubic_point(t, last, pt0, pt1, pt2));
                }
                break;
            }
            case V_CONIC:
                conic_flatten(last, pt0, pt1, wgt, &capped, to);
                break;
            default: break;
            }
            if (is_last_cmd && !veq(last_end, first_end)) {
                o = o_end - 1;   // the final closing line is the command's last line
                put(last_end, first_end);
            }
        }
        __syncthreads();

        // ---------------- B. count walk: touched tiles, crossings, line ranges ----------------
        int bx0 = 0x7fffffff, by0 = 0x7fffffff, bx1 = (int)0x80000000, by1 = (int)0x80000000;
        if (!bail) {
            for (int l = tid; l < n_lines; l += FUSED_THREADS) {
                const float4 L = S.lines[l];
                const int ax = div8(f2i16(floorf(L.x))), ay = div8(f2i16(floorf(L.y)));
                const int px = div8(f2i16(floorf(L.z))), py = div8(f2i16(floorf(L.w)));
                bx0 = min(bx0, min(ax, px));
                by0 = min(by0, min(ay, py));
                bx1 = max(bx1, max(ax, px));
                by1 = max(by1, max(ay, py));
            }
        }
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) {
            bx0 = min(bx0, __shfl_xor_sync(0xffffffffu, bx0, d));
            by0 = min(by0, __shfl_xor_sync(0xffffffffu, by0, d));
            bx1 = max(bx1, __shfl_xor_sync(0xffffffffu, bx1, d));
            by1 = max(by1, __shfl_xor_sync(0xffffffffu, by1, d));
        }
        if (lane == 0) {
            S.warp_tmp[wid][0] = bx0;
            S.warp_tmp[wid][1] = by0;
            S.warp_tmp[wid][2] = bx1;
            S.warp_tmp[wid][3] = by1;
        }
        if (tid < GDIM) S.touched[tid] = 0u;
        __syncthreads();
        // every thread derives the grid from the warps' boxes (no second barrier)
        int gx0, gy0, gw, gh;
        {
            int x0 = 0x7fffffff, y0 = 0x7fffffff, x1 = (int)0x80000000, y1 = (int)0x80000000;
#pragma unroll
            for (int k = 0; k < F_WARPS; k++) {
                x0 = min(x0, S.warp_tmp[k][0]);
                y0 = min(y0, S.warp_tmp[k][1]);
                x1 = max(x1, S.warp_tmp[k][2]);
                y1 = max(y1, S.warp_tmp[k][3]);
            }
            if (x0 > x1) { x0 = 0; y0 = 0; x1 = 0; y1 = 0; }   // no lines: the (0,0) tile
            gx0 = x0 - 1;
            gy0 = y0 - 1;
            gw = x1 - x0 + 3;
            gh = y1 - y0 + 3;
        }
        if (tid == 0) {
            S.gx0 = gx0;
            S.gy0 = gy0;
            S.gw = gw;
            S.gh = gh;
        }
        bail = bail || gw > GDIM || gh > GDIM;
        if (!bail) {
            for (int l = tid; l < n_lines; l += FUSED_THREADS) {
                const float4 L = S.lines[l];
                int gmin = 0xffff, gmax = -1;
                if (!(L.x == L.z && L.y == L.w)) {
                    bool out = false;
                    const bool ok = walk_line(
                        v2(L.x, L.y), v2(L.z, L.w),
                        [&](const Walk&, const WalkState& s) {
                            const int gx = div8(s.x) - gx0, gy = div8(s.y) - gy0;
                            if ((unsigned)gx >= (unsigned)gw || (unsigned)gy >= (unsigned)gh) { out = true; return; }
                            const int g = gy * GDIM + gx;
                            gmin = min(gmin, g);
                            gmax = max(gmax, g);
                            atomicOr(&S.touched[gy], 1u << gx);
                        },
                        [&](int tx, int ty, int sign) {
                            const int gx = tx - gx0, gy = ty - gy0;
                            if ((unsigned)gx >= (unsigned)gw || (unsigned)gy >= (unsigned)gh) { out = true; return; }
                            const uint32_t c = atomicAdd(&S.n_cross, 1u);
                            if (c < (uint32_t)F_XMAX)
                                S.u.early.cross[c] = ((uint32_t)(gy * GDIM + gx) << 16) | ((uint32_t)sign & 0xffffu);
                            else
                                out = true;
                        },
                        [&](int, int) {});
                    if (!ok) { atomicOr(A.err, ERR_LIMIT); out = true; }
                    if (out) S.flag = 1;
                }
                S.line_g0[l] = (uint16_t)gmin;
                S.line_g1[l] = (uint16_t)(gmax < 0 ? 0 : gmax);
            }
        }
        __syncthreads();
        bail = bail || S.flag != 0;

        // ---------------- compaction (row-major) and spans, by warp 0 ----------------
        if (!bail && wid == 0) {
            const uint32_t bits = S.touched[lane];
            const int cnt = __popc(bits);
            int inc = cnt;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const int o = __shfl_up_sync(0xffffffffu, inc, d);
                if (lane >= d) inc += o;
            }
            const int total = __shfl_sync(0xffffffffu, inc, 31);
            S.row_base[lane] = (uint16_t)(inc - cnt);
            if (lane == 31) S.row_base[GDIM] = (uint16_t)total;
            if (total > F_TMAX) {
                if (lane == 0) S.flag = 1;
            } else {
                int slot = inc - cnt;
                uint32_t b = bits;
                while (b) {
                    const int gx = __ffs(b) - 1;
                    b &= b - 1;
                    S.tile_g[slot++] = (uint16_t)(lane * GDIM + gx);
                }
                __syncwarp();
                // spans (rasterizer.rs:252-265): a tile is followed by one when
                // the next tile of its row leaves a gap and the crossings with
                // keys <= its own sum to a nonzero winding; one bit per tile
                const int nc = min((int)S.n_cross, F_XMAX);
                for (int base = 0; base < F_TMAX; base += 32) {
                    const int t = base + lane;
                    bool has = false;
                    if (t < total) {
                        const int g = S.tile_g[t];
                        const int gy = g >> 5, gx = g & 31;
                        const uint32_t right = gx == 31 ? 0u : S.touched[gy] >> (gx + 1);
                        if (right != 0u && !(right & 1u)) {
                            int w = 0;
                            for (int c = 0; c < nc; c++) {
                                const uint32_t e = S.u.early.cross[c];
                                if ((int)(e >> 16) <= g) w += (int)(int16_t)(e & 0xffffu);
                            }
                            has = w != 0;
                        }
                    }
                    const uint32_t m = __ballot_sync(0xffffffffu, has);
                    if (lane == 0) S.span_mask[base >> 5] = m;
                }
            }
        }
        __syncthreads();
        bail = bail || S.flag != 0;
        int n_real = 0, n_tiles = 0, n_spans = 0;
        if (!bail) {
            n_real = S.row_base[GDIM];
            n_tiles = n_real == 0 ? 1 : n_real;   // rasterizer.rs:194-208
#pragma unroll
            for (int k = 0; k < F_TMAX / 32; k++) n_spans += __popc(S.span_mask[k]);
        }
        // The raster's counts go out now; its output offsets are resolved
        // after the coverage below, when its predecessors have long
        // published theirs.  A raster that does not fit publishes zeros and
        // turns the batch over to the general chain.
        if (wid == 0) lb_publish(A, r, bail ? 0u : (uint32_t)n_tiles, bail ? 0u : (uint32_t)n_spans);
        if (tid == 0 && bail) atomicOr(A.fallback, 1u);

        // ---------------- C. accumulate and shade, CHUNK tiles at a time ----------------
        // Alpha (and coverage) go to this CTA's staging slots: tile i of the
        // raster at stage + (blockIdx.x * F_TMAX + i) * 64.
        if (!bail && n_real > 0) {
            const size_t stage0 = (size_t)blockIdx.x * F_TMAX;
            const int gx0 = S.gx0, gy0 = S.gy0;
            for (int lo = 0; lo < n_real; lo += CHUNK) {
                const int nch = min(CHUNK, n_real - lo);
                const int g_lo = S.tile_g[lo], g_hi = S.tile_g[lo + nch - 1];
                for (int q = tid; q < nch * 128; q += FUSED_THREADS) (&S.u.acc[0][0])[q] = 0.0f;
                __syncthreads();
                // walk the lines touching the chunk again, scatter-adding the
                // increments of its tiles (rasterizer.rs:97-106, 223-228)
                for (int l = tid; l < n_lines; l += FUSED_THREADS) {
                    if ((int)S.line_g1[l] < g_lo || (int)S.line_g0[l] > g_hi) continue;
                    const float4 L = S.lines[l];
                    walk_line(
                        v2(L.x, L.y), v2(L.z, L.w),
                        [&](const Walk& w, const WalkState& s) {
                            const int gx = div8(s.x) - gx0, gy = div8(s.y) - gy0;
                            const int g = gy * GDIM + gx;
                            if (g < g_lo || g > g_hi) return;
                            const int i = S.row_base[gy] + __popc(S.touched[gy] & ((1u << gx) - 1u)) - lo;
                            float area, height;
                            walk_increment(w, s, area, height);
                            const int cell = ((s.y & 7) << 3) | (s.x & 7);
                            atomicAdd(&S.u.acc[i][cell], area);
                            atomicAdd(&S.u.acc[i][64 + cell], height);
                        },
                        [&](int, int, int) {}, [&](int, int) {});
                }
                __syncthreads();
                // row sums, then carries along grid rows (rasterizer.rs:232-250)
                for (int q = tid; q < nch * 8; q += FUSED_THREADS) {
                    const int i = q >> 3, y = q & 7;
                    const float* h = S.u.acc[i] + 64 + y * 8;
                    float rs = 0.0f;
#pragma unroll
                    for (int x = 0; x < 8; x++) rs += h[x];
                    S.rs[i][y] = rs;
                }
                __syncthreads();
                if (tid < 8) {
                    float c = 0.0f;
                    int prev_row = -1;
                    if (lo > 0) {
                        prev_row = S.tile_g[lo - 1] >> 5;
                        c = S.pend[tid];
                    }
                    for (int i = 0; i < nch; i++) {
                        const int row = S.tile_g[lo + i] >> 5;
                        if (row != prev_row) c = 0.0f;
                        prev_row = row;
                        S.carry[i][tid] = c;
                        c += S.rs[i][tid];
                    }
                    S.pend[tid] = c;
                }
                __syncthreads();
                const int row = lane >> 2, c0 = 2 * lane;
                for (int i = wid; i < nch; i += F_WARPS) {
                    const float* acc = S.u.acc[i];
                    const float a0 = acc[c0], a1 = acc[c0 + 1];
                    const float h0 = acc[64 + c0];
                    float incl = h0 + acc[64 + c0 + 1];
                    const float u1 = __shfl_up_sync(0xffffffffu, incl, 1, 4);
                    if ((lane & 3) >= 1) incl += u1;
                    const float u2 = __shfl_up_sync(0xffffffffu, incl, 2, 4);
                    if ((lane & 3) >= 2) incl += u2;
                    float excl = __shfl_up_sync(0xffffffffu, incl, 1, 4);
                    if ((lane & 3) == 0) excl = 0.0f;
                    const float acc0 = S.carry[i][row] + excl;
                    const float cov0 = fabsf(acc0 + a0);
                    const float cov1 = fabsf((acc0 + h0) + a1);
                    const size_t t = stage0 + lo + i;
                    const uint32_t al0 = f2u8(rmin(cov0 * 256.0f, 255.0f));
                    const uint32_t al1 = f2u8(rmin(cov1 * 256.0f, 255.0f));
                    reinterpret_cast<uint16_t*>(A.stage_alpha + t * 64)[lane] = (uint16_t)(al0 | (al1 << 8));
                    if (A.out_cov) reinterpret_cast<float2*>(A.stage_cov + t * 64)[lane] = make_float2(cov0, cov1);
                }
                __syncthreads();
            }
        }

        // ---------------- offsets, then every output of the raster ----------------
        if (wid == 0) {
            uint32_t p0, p1;
            const uint32_t a0 = bail ? 0u : (uint32_t)n_tiles, a1 = bail ? 0u : (uint32_t)n_spans;
            lb_resolve(A, r, a0, a1, p0, p1);
            if (lane == 0) {
                S.tile_base = p0;
                S.span_base = p1;
                if (!bail) {
                    A.raster_tile_off[r] = p0;
                    A.raster_span_off[r] = p1;
                    if (r + 1 == A.n_rasters) {
                        A.raster_tile_off[r + 1] = p0 + n_tiles;
                        A.raster_span_off[r + 1] = p1 + n_spans;
                        A.totals[0] = p0 + n_tiles;
                        A.totals[1] = p1 + n_spans;
                    }
                }
            }
        }
        __syncthreads();
        if (!bail) {
            const uint32_t tb = S.tile_base, sb = S.span_base;
            if ((uint64_t)tb + n_tiles > A.tile_cap || (uint64_t)sb + n_spans > A.span_cap) {
                if (tid == 0) atomicOr(A.err, ERR_CAPACITY);
            } else if (n_real == 0) {
                // no increments: one all-zero tile at (0, 0)
                if (tid < 16) reinterpret_cast<uint32_t*>(A.out_alpha + (size_t)tb * 64)[tid] = 0u;
                if (A.out_cov && tid < 64) A.out_cov[(size_t)tb * 64 + tid] = 0.0f;
                if (tid == 0) A.out_xy[tb] = 0u;
            } else {
                // staged alpha / coverage -> their final place (8-byte pieces)
                const size_t stage0 = (size_t)blockIdx.x * F_TMAX;
                const uint2* sa = reinterpret_cast<const uint2*>(A.stage_alpha + stage0 * 64);
                uint2* da = reinterpret_cast<uint2*>(A.out_alpha + (size_t)tb * 64);
                for (int q = tid; q < n_real * 8; q += FUSED_THREADS) da[q] = sa[q];
                if (A.out_cov) {
                    const float2* sc = reinterpret_cast<const float2*>(A.stage_cov + stage0 * 64);
                    float2* dc = reinterpret_cast<float2*>(A.out_cov + (size_t)tb * 64);
                    for (int q = tid; q < n_real * 32; q += FUSED_THREADS) dc[q] = sc[q];
                }
                for (int t = tid; t < n_real; t += FUSED_THREADS) {
                    const int g = S.tile_g[t];
                    const int tx = S.gx0 + (g & 31), ty = S.gy0 + (g >> 5);
                    A.out_xy[tb + t] = (uint32_t)(uint16_t)(int16_t)(tx * 8) |
                                       ((uint32_t)(uint16_t)(int16_t)(ty * 8) << 16);
                    const uint32_t m = S.span_mask[t >> 5];
                    if (m >> (t & 31) & 1u) {
                        // span rank: the span tiles before t (tile order = callback order)
                        int sr = __popc(m & ((1u << (t & 31)) - 1u));
                        for (int k = 0; k < (t >> 5); k++) sr += __popc(S.span_mask[k]);
                        const uint32_t right = S.touched[g >> 5] >> ((g & 31) + 1);
                        const int gap = __ffs(right) - 1;
                        A.span_xy[sb + sr] = (uint32_t)(uint16_t)(int16_t)((tx + 1) * 8) |
                                             ((uint32_t)(uint16_t)(int16_t)(ty * 8) << 16);
                        A.span_w[sb + sr] = (uint16_t)((uint16_t)gap * 8u);
                        A.span_tile[sb + sr] = tb + t;
                    }
                }
            }
        }
        __syncthreads();
    }
}

// Persistent grid of a kernel shape: SMs x resident CTAs.
template <int T, int C>
static int fused_full_grid() {
    static int grid = 0;
    if (grid == 0) {
        int dev = 0, sms = 0, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_raster_fused<T, C>, T, 0);
        grid = sms * (per > 0 ? per : 1);
    }
    return grid;
}

// The tuned shape: with a == nullptr, its full grid into *grid; else one
// launch over *grid CTAs.
static int fused_shape(ochre_gpu_ctx* ctx, const FusedArgs* a, int* grid, cudaStream_t s) {
#define OCHRE_FUSED_CASE(T, C)                                                        \
    case T * 1000 + C:                                                                \
        if (!a) {                                                                     \
            *grid = fused_full_grid<T, C>();                                          \
            return OCHRE_OK;                                                          \
        }                                                                             \
        OCHRE_LAUNCH(ctx, "raster_fused", s, k_raster_fused<T, C><<<*grid, T, 0, s>>>(*a)); \
        OCHRE_CUDA_TRY(cudaGetLastError());                                           \
        return OCHRE_OK;
    switch (ctx->tune_fused_threads * 1000 + ctx->tune_fused_chunk) {
        OCHRE_FUSED_CASE(64, 8)
        OCHRE_FUSED_CASE(64, 16)
        OCHRE_FUSED_CASE(64, 32)
        OCHRE_FUSED_CASE(96, 8)
        OCHRE_FUSED_CASE(96, 16)
        OCHRE_FUSED_CASE(128, 16)
        OCHRE_FUSED_CASE(128, 32)
    default: return OCHRE_E_INVALID;
    }
#undef OCHRE_FUSED_CASE
}

struct VerbFloats {
    const uint8_t* verbs;
    __device__ __forceinline__ uint32_t operator()(uint64_t i) const { return floats_per_verb(__ldg(verbs + i)); }
};
struct FloatOff {
    uint32_t* off;
    __device__ __forceinline__ void operator()(uint64_t i, uint32_t ex, uint32_t) const { off[i] = ex; }
};

// Runs the fused kernel over the whole batch.  *handled is false when some
// raster does not fit (the caller then runs the general chain).
static int run_fused(ochre_gpu_ctx* ctx, const ochre_batch* in, cudaStream_t s, bool* handled, uint32_t* n_tiles,
                     uint32_t* n_spans) {
    *handled = false;
    DevScalars* ds = dev_scalars(ctx);
    const uint32_t R = in->n_rasters;
    const bool want_cov = (ctx->flags & OCHRE_CTX_WANT_COV) != 0;
    // look-back words: per raster (aggregate, inclusive), per block
    // (aggregate, inclusive) and the blocks' publish counters, zeroed per run
    const size_t nb = ((size_t)R + LB_BLOCK - 1) / LB_BLOCK;
    const size_t lb_bytes = (2 * (size_t)R + 2 * nb) * sizeof(uint64_t) + nb * sizeof(uint32_t);
    OCHRE_CUDA_TRY(ctx->fused_chain.ensure(lb_bytes));
    uint64_t* lb = ctx->fused_chain.as<uint64_t>();
    // no more CTAs than rasters; each stages the coverage of its raster
    int grid = 0;
    {
        const int st = fused_shape(ctx, nullptr, &grid, s);
        if (st != OCHRE_OK) return st;
    }
    grid = (int)std::min<uint32_t>((uint32_t)grid, R);
    if (ctx->fused_max_ctas) grid = std::min<int>(grid, std::max<int>(1, (int)ctx->fused_max_ctas));
    const size_t stage_tiles = (size_t)grid * F_TMAX;
    OCHRE_CUDA_TRY(ctx->fused_stage.ensure(stage_tiles * 64 * (want_cov ? 5 : 1)));
    // float offset of every command (the kernel reads its points there)
    const uint64_t n_cmds = in->n_cmds;
    OCHRE_CUDA_TRY(ctx->cmd_foff.ensure((size_t)std::max<uint64_t>(n_cmds, 1) * 4));
    OCHRE_CUDA_TRY(ctx->scan_status.ensure(scan_tiles(n_cmds) * sizeof(ScanStatus<uint32_t>)));
    // capacity guess: the last run's totals, else 48 tiles per raster; with
    // caller-provided (fixed) outputs, their capacity
    const bool fixed_out = ctx->out_tile_xy.fixed;
    uint64_t cap_guess = ctx->fused_tile_cap ? ctx->fused_tile_cap : (uint64_t)R * 48u;
    if (cap_guess > MAX_COUNT) cap_guess = MAX_COUNT;
    uint32_t tile_cap = (uint32_t)cap_guess;
    uint32_t span_cap_fixed = 0;
    const GraphPlan* plan = ctx->plan;
    if (plan) tile_cap = plan->tiles;   // graph replays: the planned capacity, no retry
    if (fixed_out) {
        tile_cap = (uint32_t)std::min(ctx->out_tile_xy.cap / 4, ctx->out_tile_alpha.cap / 64);
        span_cap_fixed = (uint32_t)std::min(std::min(ctx->out_span_xy.cap / 4, ctx->out_span_w.cap / 2),
                                            ctx->out_span_tile.cap / 4);
    }
    for (int attempt = 0; attempt < 2; attempt++) {
        const uint32_t span_cap = fixed_out ? span_cap_fixed : tile_cap;
        OCHRE_CUDA_TRY(ctx->out_tile_xy.ensure((size_t)tile_cap * 4));
        OCHRE_CUDA_TRY(ctx->out_tile_alpha.ensure((size_t)tile_cap * 64));
        if (want_cov) OCHRE_CUDA_TRY(ctx->out_tile_cov.ensure((size_t)tile_cap * 256));
        OCHRE_CUDA_TRY(ctx->out_span_xy.ensure((size_t)span_cap * 4));
        OCHRE_CUDA_TRY(ctx->out_span_w.ensure((size_t)span_cap * 2));
        OCHRE_CUDA_TRY(ctx->out_span_tile.ensure((size_t)span_cap * 4));
        OCHRE_CUDA_TRY(ctx->out_raster_tile_off.ensure((size_t)(R + 1) * 4));
        OCHRE_CUDA_TRY(ctx->out_raster_span_off.ensure((size_t)(R + 1) * 4));
        OCHRE_CUDA_TRY(cudaMemsetAsync(lb, 0, lb_bytes, s));
        OCHRE_CUDA_TRY(reset_scalars(ctx, s));
        if (n_cmds)
            OCHRE_LAUNCH(ctx, "fused_float_scan", s, OCHRE_CUDA_TRY(launch_scan<uint32_t>(
                n_cmds, VerbFloats{in->verbs}, FloatOff{ctx->cmd_foff.as<uint32_t>()}, OpSumU32{}, 0u,
                ctx->scan_status.p, &ds->sort_ticket, &ds->n_floats, &ds->err, s, nullptr,
                ctx->test_skip_first_ticket ? 1u : 0u)));
        FusedArgs a{};
        a.verbs = in->verbs;
        a.pts = in->pts;
        a.cmd_foff = ctx->cmd_foff.as<uint32_t>();
        a.stage_alpha = ctx->fused_stage.as<uint8_t>();
        a.stage_cov = want_cov ? reinterpret_cast<float*>(ctx->fused_stage.as<uint8_t>() + stage_tiles * 64) : nullptr;
        a.fill_off = in->fill_cmd_off;
        a.fill_xf = in->fill_xf;
        a.fill_flags = in->fill_flags;
        a.raster_off = in->raster_fill_off;
        a.n_fills = in->n_fills;
        a.n_rasters = R;
        a.n_floats = in->n_floats;
        a.r_agg = lb;
        a.r_inc = lb + R;
        a.b_agg = lb + 2 * (size_t)R;
        a.b_inc = lb + 2 * (size_t)R + nb;
        a.b_cnt = reinterpret_cast<uint32_t*>(lb + 2 * (size_t)R + 2 * nb);
        a.ticket = &ds->ticket;
        a.fallback = &ds->fused_fallback;
        a.err = &ds->err;
        a.totals = &ds->fused_tiles;
        a.tile_cap = tile_cap;
        a.span_cap = span_cap;
        a.out_xy = ctx->out_tile_xy.as<uint32_t>();
        a.out_alpha = ctx->out_tile_alpha.as<uint8_t>();
        a.out_cov = want_cov ? ctx->out_tile_cov.as<float>() : nullptr;
        a.span_xy = ctx->out_span_xy.as<uint32_t>();
        a.span_w = ctx->out_span_w.as<uint16_t>();
        a.span_tile = ctx->out_span_tile.as<uint32_t>();
        a.raster_tile_off = ctx->out_raster_tile_off.as<uint32_t>();
        a.raster_span_off = ctx->out_raster_span_off.as<uint32_t>();
        wait_inputs(ctx, s);   // the kernel reads points
        const int st0 = fused_shape(ctx, &a, &grid, s);
        if (st0 != OCHRE_OK) return st0;
        if (plan) {
            // totals, fallback and errors are read after the replay
            *handled = true;
            return OCHRE_OK;
        }
        int st = read_scalars(ctx, s);
        if (st != OCHRE_OK) return st;
        const DevScalars* hs = host_scalars(ctx);
        if (hs->fused_fallback) return OCHRE_OK;   // not handled
        const uint32_t e = hs->err;
        if (e & ERR_INVALID) return OCHRE_E_INVALID;
        if (e & ERR_LIMIT) return OCHRE_E_LIMIT;
        if (e & ERR_TIMEOUT) return OCHRE_E_TIMEOUT;
        if (e & ERR_CAPACITY) {
            // outputs did not fit the guess: the totals are exact, retry once
            const uint64_t need = (uint64_t)hs->fused_tiles;
            if (need > MAX_COUNT || fixed_out) return OCHRE_E_CAPACITY;
            tile_cap = (uint32_t)std::min<uint64_t>(need + 1024u, MAX_COUNT);
            continue;
        }
        *n_tiles = hs->fused_tiles;
        *n_spans = hs->fused_spans;
        if (!fixed_out)
            ctx->fused_tile_cap =
                (uint32_t)std::min<uint64_t>((uint64_t)hs->fused_tiles + hs->fused_tiles / 4 + 1024u, MAX_COUNT);
        *handled = true;
        return OCHRE_OK;
    }
    return OCHRE_E_CAPACITY;
}

// The fused path over the whole batch; *handled is false when some raster
// does not fit it (the caller then runs the general chain).
int stage_fused(ochre_gpu_ctx* ctx, const ochre_batch* in, cudaStream_t s, bool* handled, uint32_t* n_tiles,
                uint32_t* n_spans) {
    *handled = false;
    if (in->n_rasters == 0) return OCHRE_OK;
    return run_fused(ctx, in, s, handled, n_tiles, n_spans);
}

}  // namespace ochre
