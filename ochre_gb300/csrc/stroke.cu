// Stroked fills: Rasterizer::stroke (rasterizer.rs:169-171) is
//   fill(&stroke(&flatten(path, TOLERANCE), width), transform)
// i.e. the path is flattened in its own space (path.rs:113-142), each
// polyline contour is offset by width / 2 on both sides with the reference's
// joins and butt caps (path.rs:150-274), and the resulting Move / Line /
// Close path is filled with the fill's transform.
//
// This stage rewrites a batch whose fills carry OCHRE_FILL_STROKE into a
// plain fill batch on the device (other fills are copied unchanged), then
// the normal path rasterizes it:
//   1. command scan of the input (float offsets, most recent endpoint);
//   2. polyline sizes per command (path-space flatten counts), scan, emit;
//   3. units: one per stroked contour, one per copied command; compaction;
//   4. output sizes per unit (the offset sides counted join by join, one
//      warp per unit), scan in place, emit; fill offsets of the output.
// A side's join at step i needs only the side's point before it (point i - 1)
// and the normal of the nearest earlier step that emitted a join, so a warp
// computes 32 joins at a time and carries one normal between rounds.
// Contours start at a Move or after a Close; `closed` is
// set by a Close ending the contour or by any earlier Close of the path
// (the reference never resets it, path.rs:218-256).
#include "common.cuh"
#include "flatten.cuh"
#include "internal.h"
#include "scan.cuh"

namespace ochre {

__device__ __forceinline__ bool is_stroke(const uint8_t* flags, uint32_t f) {
    return flags != nullptr && (__ldg(flags + f) & OCHRE_FILL_STROKE);
}

// Path-space `last` of command c in fill f: the end point of the most recent
// earlier non-Close command of the same path, or the origin.
__device__ __forceinline__ V2 path_last(const uint8_t* verbs, const float* pts, const uint32_t* cmd_foff,
                                        const uint32_t* cmd_ep, const uint32_t* fill_off, uint32_t f, uint32_t c) {
    const uint32_t ep = cmd_ep[c];
    if (ep == 0 || ep - 1u < __ldg(fill_off + f)) return v2(0.0f, 0.0f);
    const uint32_t j = ep - 1u;
    const float* fp = pts + cmd_foff[j] + endpoint_float(__ldg(verbs + j));
    return v2(__ldg(fp), __ldg(fp + 1));
}

// ---- 2. polyline sizes ----
struct Pair {
    uint32_t n;
    uint32_t nf;
};
struct OpPair {
    __device__ __forceinline__ Pair operator()(Pair a, Pair b) const { return Pair{a.n + b.n, a.nf + b.nf}; }
};
struct PolyCount {
    const uint8_t* verbs;
    const float* pts;
    const uint32_t* fill_off;
    uint32_t n_fills;
    const uint8_t* flags;
    const uint32_t* cmd_foff;
    const uint32_t* cmd_ep;
    uint32_t* err;
    __device__ Pair operator()(uint64_t i) const {
        const uint32_t c = (uint32_t)i;
        const uint8_t v = __ldg(verbs + c);
        const uint32_t f = upper_bound_u32(fill_off, n_fills + 1, c) - 1u;
        if (!is_stroke(flags, f)) return Pair{1u, floats_per_verb(v)};
        if (v == V_MOVE || v == V_LINE) return Pair{1u, 2u};
        if (v == V_CLOSE) return Pair{1u, 0u};
        const V2 last = path_last(verbs, pts, cmd_foff, cmd_ep, fill_off, f, c);
        const float* fp = pts + cmd_foff[c];
        bool capped = false;
        uint32_t n = 0;
        if (v == V_QUAD) {
            n = flatten_steps(quad_dt(last, v2(fp[0], fp[1]), v2(fp[2], fp[3])), &capped);
        } else if (v == V_CUBIC) {
            n = flatten_steps(cubic_dt(last, v2(fp[0], fp[1]), v2(fp[2], fp[3]), v2(fp[4], fp[5])), &capped);
        } else {
            conic_flatten(last, v2(fp[0], fp[1]), v2(fp[2], fp[3]), fp[4], &capped, [&](V2) { n++; });
        }
        if (capped) atomicOr(err, ERR_LIMIT);
        return Pair{n, 2u * n};
    }
};
struct PairOut {
    uint32_t* off;
    uint32_t* foff;
    __device__ __forceinline__ void operator()(uint64_t i, Pair ex, Pair) const {
        off[i] = ex.n;
        foff[i] = ex.nf;
    }
};
// Counts already stored in the two offset arrays (scanned in place).
struct PairIn {
    const uint32_t* n;
    const uint32_t* nf;
    __device__ __forceinline__ Pair operator()(uint64_t i) const { return Pair{n[i], nf[i]}; }
};

// One thread per item: a count functor with a long serial walk per item runs
// at full occupancy here, and the scan over the stored counts stays light.
template <class Count>
__global__ void __launch_bounds__(128) k_pair_count(uint64_t n, const uint32_t* n_dev, Count count,
                                                    uint32_t* __restrict__ out_n, uint32_t* __restrict__ out_nf) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= dev_count(n, n_dev)) return;
    const Pair p = count(i);
    out_n[i] = p.n;
    out_nf[i] = p.nf;
}

__global__ void k_poly_emit(const uint8_t* __restrict__ verbs, const float* __restrict__ pts,
                            const uint32_t* __restrict__ fill_off, uint32_t n_fills, const uint8_t* __restrict__ flags,
                            uint64_t n_cmds, const uint32_t* __restrict__ cmd_foff, const uint32_t* __restrict__ cmd_ep,
                            const uint32_t* __restrict__ poly_off, const uint32_t* __restrict__ poly_foff,
                            uint8_t* __restrict__ pverbs, float* __restrict__ ppts, uint32_t p_cap, uint32_t pf_cap) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n_cmds) return;
    const uint32_t c = (uint32_t)i;
    const uint8_t v = __ldg(verbs + c);
    const uint32_t f = upper_bound_u32(fill_off, n_fills + 1, c) - 1u;
    uint32_t o = poly_off[c], fo = poly_foff[c];
    const float* fp = pts + cmd_foff[c];
    // writes stay below the buffers' capacities (a planned run whose
    // polyline outgrew them is flagged by the check after the scan)
    auto verb = [&](uint32_t at, uint8_t x) {
        if (at < p_cap) pverbs[at] = x;
    };
    auto flt = [&](uint32_t at, float x) {
        if (at < pf_cap) ppts[at] = x;
    };
    if (!is_stroke(flags, f)) {
        verb(o, v);
        for (uint32_t k = 0; k < floats_per_verb(v); k++) flt(fo + k, __ldg(fp + k));
        return;
    }
    auto line = [&](V2 p) {
        verb(o++, V_LINE);
        flt(fo++, p.x);
        flt(fo++, p.y);
    };
    switch (v) {
    case V_MOVE:
    case V_LINE:
        verb(o, v);
        flt(fo, __ldg(fp));
        flt(fo + 1, __ldg(fp + 1));
        break;
    case V_CLOSE:
        verb(o, V_CLOSE);
        break;
    case V_QUAD: {
        // path.rs:49-58 in path space
        const V2 last = path_last(verbs, pts, cmd_foff, cmd_ep, fill_off, f, c);
        const V2 p1 = v2(fp[0], fp[1]), p2 = v2(fp[2], fp[3]);
        const float dt = quad_dt(last, p1, p2);
        float t = 0.0f;
        uint32_t n = 0;
        while (t < 1.0f) {
            t = rmin(__fadd_rn(t, dt), 1.0f);
            line(quad_point(t, last, p1, p2));
            if (++n >= FLATTEN_CAP) break;
        }
        break;
    }
    case V_CUBIC: {
        // path.rs:59-74 in path space
        const V2 last = path_last(verbs, pts, cmd_foff, cmd_ep, fill_off, f, c);
        const V2 p1 = v2(fp[0], fp[1]), p2 = v2(fp[2], fp[3]), p3 = v2(fp[4], fp[5]);
        const float dt = cubic_dt(last, p1, p2, p3);
        float t = 0.0f;
        uint32_t n = 0;
        while (t < 1.0f) {
            t = rmin(__fadd_rn(t, dt), 1.0f);
            line(cubic_point(t, last, p1, p2, p3));
            if (++n >= FLATTEN_CAP) break;
        }
        break;
    }
    default: {   // conic, path.rs:75-104
        const V2 last = path_last(verbs, pts, cmd_foff, cmd_ep, fill_off, f, c);
        bool capped = false;
        conic_flatten(last, v2(fp[0], fp[1]), v2(fp[2], fp[3]), fp[4], &capped, line);
        break;
    }
    }
}

// ---- 3. units ----
// A unit is a stroked contour (starting at a Move, at the path's first
// command or after a Close) or one copied command of a plain fill.
struct UnitIn {
    const uint8_t* pverbs;
    const uint32_t* pfill_off;   // polyline offsets of the fills (n_fills + 1)
    uint32_t n_fills;
    const uint8_t* flags;
    __device__ __forceinline__ uint32_t operator()(uint64_t i) const {
        const uint32_t p = (uint32_t)i;
        const uint32_t f = upper_bound_u32(pfill_off, n_fills + 1, p) - 1u;
        if (!is_stroke(flags, f)) return 1u;
        const uint8_t v = pverbs[p];
        if (v == V_CLOSE) return 0u;
        return (v == V_MOVE || p == __ldg(pfill_off + f) || pverbs[p - 1] == V_CLOSE) ? 1u : 0u;
    }
};
struct UnitOut {
    uint32_t* unit_start;
    __device__ __forceinline__ void operator()(uint64_t i, uint32_t ex, uint32_t v) const {
        if (v) unit_start[ex] = (uint32_t)i;
    }
};

struct PolyFloats {
    const uint8_t* v;
    __device__ __forceinline__ uint32_t operator()(uint64_t i) const { return floats_per_verb(v[i]); }
};
struct OffOutU32 {
    uint32_t* off;
    __device__ __forceinline__ void operator()(uint64_t i, uint32_t ex, uint32_t) const { off[i] = ex; }
};

__global__ void k_first_close(const uint8_t* __restrict__ pverbs, uint64_t n_poly, const uint32_t* n_dev,
                              const uint32_t* __restrict__ pfill_off, uint32_t n_fills, const uint8_t* __restrict__ flags,
                              uint32_t* __restrict__ first_close) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= dev_count(n_poly, n_dev) || pverbs[i] != V_CLOSE) return;
    const uint32_t f = upper_bound_u32(pfill_off, n_fills + 1, (uint32_t)i) - 1u;
    if (is_stroke(flags, f)) atomicMin(first_close + f, (uint32_t)i);
}

__global__ void k_fill_init(uint32_t* __restrict__ first_close, const uint32_t* __restrict__ fill_off,
                            const uint32_t* __restrict__ poly_off, uint64_t n_cmds, uint32_t n_poly,
                            const uint32_t* n_poly_dev, uint32_t n_fills, uint32_t* __restrict__ pfill_off) {
    const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f > n_fills) return;
    const uint32_t np = (uint32_t)dev_count(n_poly, n_poly_dev);
    const uint32_t c = __ldg(fill_off + f);
    pfill_off[f] = c < n_cmds ? min(poly_off[c], np) : np;
    if (f < n_fills) first_close[f] = 0xffffffffu;
}

// ---- 4. the offset sides (path.rs:160-212) ----
// One side of contour [c0, c1) of the polyline (points P(k), 2 floats each),
// walked by a whole warp, 32 steps at a time.  In the reference's loop the
// point before step i is always the side's point i - 1 (at i = 0 its first
// point: a step whose point equals the one before emits nothing and changes
// nothing), and the normal before step i is that of the last step before i
// that emitted a join.  So the lanes compute the joins of their steps at
// once, with the reference's operations in its order, and only the last
// normal is carried from one round of 32 steps to the next; a scan of the
// joins' point counts (1 or 2) gives each point its place.  emit(k, point)
// receives the side's k-th point; every lane returns the side's point count.
template <class Emit>
__device__ uint32_t stroke_side_warp(const float* __restrict__ P, uint32_t len, bool closed, bool reverse, float width,
                                     Emit emit) {
    const uint32_t lane = threadIdx.x & 31u;
    auto pt = [&](uint32_t k) { return v2(P[2 * k], P[2 * k + 1]); };
    auto side = [&](uint32_t k) { return reverse ? pt(len - k - 1) : pt(k); };   // the side's k-th point
    const V2 first_point = closed == reverse ? pt(0) : pt(len - 1);
    const float half = __fmul_rn(0.5f, width);
    float cnx = 0.0f, cny = 0.0f;   // normal of the last join so far
    uint32_t base = 0;              // points emitted so far
    for (uint32_t i0 = 0; i0 <= len; i0 += 32) {
        const uint32_t i = i0 + lane;
        const bool valid = i <= len;
        V2 next = v2(0.0f, 0.0f), prev = v2(0.0f, 0.0f);
        if (valid) {
            next = i < len ? side(i) : first_point;
            prev = i == 0 ? first_point : side(i - 1);
        }
        const bool join = valid && (!veq(next, prev) || i == len);
        V2 nn = v2(0.0f, 0.0f);
        if (join) {
            const V2 tan = vsub(next, prev);
            nn = v2(-tan.y, tan.x);
            const float nlen = vlength(nn);
            if (nlen == 0.0f) {
                nn = v2(0.0f, 0.0f);
            } else {
                const float r = __fdiv_rn(1.0f, nlen);
                nn = v2(__fmul_rn(nn.x, r), __fmul_rn(nn.y, r));
            }
        }
        // the normal before this step: the nearest join below in this round,
        // else the one carried from the rounds before
        const uint32_t jm = __ballot_sync(0xffffffffu, join);
        const uint32_t below = jm & ((1u << lane) - 1u);
        const int src = below ? 31 - __clz(below) : (int)lane;
        const float px = __shfl_sync(0xffffffffu, nn.x, src), py = __shfl_sync(0xffffffffu, nn.y, src);
        const V2 pn = below ? v2(px, py) : v2(cnx, cny);
        uint32_t cnt = 0;
        V2 e0 = v2(0.0f, 0.0f), e1 = v2(0.0f, 0.0f);
        if (join) {
            // join (path.rs:160-168)
            const float dot = __fadd_rn(__fmul_rn(pn.x, nn.x), __fmul_rn(pn.y, nn.y));
            const float offset = __fdiv_rn(1.0f, __fadd_rn(1.0f, dot));
            if (fabsf(offset) > 2.0f) {
                e0 = vadd(prev, vscale(half, pn));
                e1 = vadd(prev, vscale(half, nn));
                cnt = 2;
            } else {
                e0 = vadd(prev, vscale(__fmul_rn(half, offset), vadd(pn, nn)));
                cnt = 1;
            }
        }
        uint32_t incl = cnt;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t o = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= (uint32_t)d) incl += o;
        }
        const uint32_t pos = base + incl - cnt;
        if (cnt >= 1) emit(pos, e0);
        if (cnt == 2) emit(pos + 1, e1);
        base += __shfl_sync(0xffffffffu, incl, 31);
        if (jm) {
            const int last = 31 - __clz(jm);
            cnx = __shfl_sync(0xffffffffu, nn.x, last);
            cny = __shfl_sync(0xffffffffu, nn.y, last);
        }
    }
    return base;
}

struct UnitGeom {
    uint32_t p0, len;   // first polyline command and length (contours)
    uint32_t fill;
    uint32_t closed;    // 1: closed contour; 2: copied command
};

// Unit u's contour (every lane of the warp, the same answer).  A contour runs
// from its start to the first polyline command after it that is not a Line
// (32 checked per round).
__device__ __forceinline__ UnitGeom unit_geom_warp(uint32_t u, const uint32_t* unit_start, const uint8_t* pverbs,
                                                   const uint32_t* pfill_off, uint32_t n_fills, const uint8_t* flags,
                                                   const uint32_t* first_close) {
    const uint32_t lane = threadIdx.x & 31u;
    UnitGeom g;
    g.p0 = unit_start[u];
    g.fill = upper_bound_u32(pfill_off, n_fills + 1, g.p0) - 1u;
    if (!is_stroke(flags, g.fill)) {
        g.len = 1;
        g.closed = 2;
        return g;
    }
    const uint32_t pe = __ldg(pfill_off + g.fill + 1);
    uint32_t e = g.p0 + 1;
    for (;;) {
        const uint32_t k = e + lane;
        const uint32_t stop = __ballot_sync(0xffffffffu, k >= pe || pverbs[k] != V_LINE);
        if (stop) {
            e += (uint32_t)__ffs(stop) - 1u;
            break;
        }
        e += 32;
    }
    g.len = e - g.p0;
    const bool term_close = e < pe && pverbs[e] == V_CLOSE;
    g.closed = (term_close || first_close[g.fill] < g.p0) ? 1u : 0u;
    return g;
}

// Output commands and floats of every unit, one warp per unit.
__global__ void __launch_bounds__(128) k_out_count(uint32_t n_units, const uint32_t* n_dev,
                                                   const uint32_t* __restrict__ unit_start,
                                                   const uint8_t* __restrict__ pverbs, const float* __restrict__ ppts,
                                                   const uint32_t* __restrict__ poly_foff_of,
                                                   const uint32_t* __restrict__ pfill_off, uint32_t n_fills,
                                                   const uint8_t* __restrict__ flags,
                                                   const uint32_t* __restrict__ first_close,
                                                   const float* __restrict__ width, uint32_t* __restrict__ out_n,
                                                   uint32_t* __restrict__ out_nf) {
    const uint64_t u = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    if (u >= dev_count(n_units, n_dev)) return;   // whole warps
    const uint32_t lane = threadIdx.x & 31u;
    const UnitGeom g = unit_geom_warp((uint32_t)u, unit_start, pverbs, pfill_off, n_fills, flags, first_close);
    if (g.closed == 2) {
        if (lane == 0) {
            out_n[u] = 1u;
            out_nf[u] = floats_per_verb(pverbs[g.p0]);
        }
        return;
    }
    const float* P = ppts + poly_foff_of[g.p0];
    const float w = __ldg(width + g.fill);
    auto none = [](uint32_t, V2) {};
    const uint32_t n = stroke_side_warp(P, g.len, g.closed != 0, false, w, none) +
                       stroke_side_warp(P, g.len, g.closed != 0, true, w, none);
    if (lane == 0) {
        out_n[u] = n + (g.closed ? 2u : 1u);
        out_nf[u] = 2u * n;
    }
}

// Every unit's output commands and points (path.rs:214-274), one warp per unit.
__global__ void __launch_bounds__(128) k_out_emit(uint32_t n_units, const uint32_t* n_dev,
                                                  const uint32_t* __restrict__ unit_start,
                                                  const uint8_t* __restrict__ pverbs, const float* __restrict__ ppts,
                                                  const uint32_t* __restrict__ poly_foff_of,
                                                  const uint32_t* __restrict__ pfill_off, uint32_t n_fills,
                                                  const uint8_t* __restrict__ flags,
                                                  const uint32_t* __restrict__ first_close,
                                                  const float* __restrict__ width, const uint32_t* __restrict__ out_off,
                                                  const uint32_t* __restrict__ out_foff, uint8_t* __restrict__ overbs,
                                                  float* __restrict__ opts, uint32_t* __restrict__ unit_fill) {
    const uint64_t u = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    if (u >= dev_count(n_units, n_dev)) return;   // whole warps
    const uint32_t lane = threadIdx.x & 31u;
    const UnitGeom g = unit_geom_warp((uint32_t)u, unit_start, pverbs, pfill_off, n_fills, flags, first_close);
    uint32_t o = out_off[u], fo = out_foff[u];
    const float* P = ppts + poly_foff_of[g.p0];
    if (g.closed == 2) {
        if (lane == 0) {
            unit_fill[u] = g.fill;
            const uint8_t v = pverbs[g.p0];
            overbs[o] = v;
            for (uint32_t k = 0; k < floats_per_verb(v); k++) opts[fo + k] = P[k];
        }
        return;
    }
    if (lane == 0) unit_fill[u] = g.fill;
    const float w = __ldg(width + g.fill);
    const bool closed = g.closed != 0;
    // forward side: its first point becomes a Move (path.rs:249-250)
    const uint32_t nf = stroke_side_warp(P, g.len, closed, false, w, [&](uint32_t k, V2 p) {
        overbs[o + k] = k == 0 ? V_MOVE : V_LINE;
        opts[fo + 2 * k] = p.x;
        opts[fo + 2 * k + 1] = p.y;
    });
    o += nf;
    fo += 2 * nf;
    if (closed) {
        if (lane == 0) overbs[o] = V_CLOSE;
        o++;
    }
    // backward side: a Move only when closed (path.rs:254-257), then Close
    const uint32_t nb = stroke_side_warp(P, g.len, closed, true, w, [&](uint32_t k, V2 p) {
        overbs[o + k] = k == 0 && closed ? V_MOVE : V_LINE;
        opts[fo + 2 * k] = p.x;
        opts[fo + 2 * k + 1] = p.y;
    });
    if (lane == 0) overbs[o + nb] = V_CLOSE;
}

// A planned run (pad_end > 0) ends the last fill at pad_end: the output
// commands from the true total up to it are Close commands.
__global__ void k_out_fill_off(const uint32_t* __restrict__ unit_fill, uint32_t n_units, const uint32_t* units_dev,
                               const uint32_t* __restrict__ out_off, uint32_t total, const uint32_t* total_dev,
                               uint32_t pad_end, uint32_t n_fills, uint32_t* __restrict__ ofill_off,
                               const uint8_t* __restrict__ flags, uint8_t* __restrict__ oflags) {
    const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f > n_fills) return;
    n_units = (uint32_t)dev_count(n_units, units_dev);
    total = (uint32_t)dev_count(total, total_dev);
    // first unit of fill >= f
    uint32_t lo = 0, hi = n_units;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (unit_fill[mid] < f) lo = mid + 1; else hi = mid;
    }
    ofill_off[f] = f == n_fills && pad_end ? pad_end : lo < n_units ? min(out_off[lo], total) : total;
    if (f < n_fills) oflags[f] = flags ? (uint8_t)(__ldg(flags + f) & ~OCHRE_FILL_STROKE) : 0u;
}

// A planned run (CUDA graph): a count pair above its capacities zeroes the
// pair and the count that bounds the next kernels, and flags ERR_CAPACITY,
// so no later kernel of the run reads or writes past a buffer (the graph
// then re-plans).
__global__ void k_stroke_cap(uint32_t* a, uint32_t cap_a, uint32_t* b, uint32_t cap_b, uint32_t* also,
                             uint32_t* err) {
    if (*a > cap_a || *b > cap_b) {
        *a = 0u;
        *b = 0u;
        *also = 0u;
        atomicOr(err, ERR_CAPACITY);
    }
}

// Eager: sizes read back at four points.  Planned (ctx->plan->stroke, inside
// a CUDA graph): no read-backs; buffers at the plan's capacities, counts on
// the device, and the output padded with Close commands to the planned
// command count (the caller zeroed the device scalars).
int stage_stroke(ochre_gpu_ctx* ctx, const ochre_batch* in, cudaStream_t s, ochre_batch* out) {
    *out = *in;
    out->fill_width = nullptr;
    if (!in->fill_width || !in->fill_flags || in->n_cmds == 0 || in->n_fills == 0) return OCHRE_OK;
    const GraphPlan* plan = ctx->plan != nullptr && ctx->plan->stroke ? ctx->plan : nullptr;
    DevScalars* ds = dev_scalars(ctx);
    const uint64_t n = in->n_cmds;
    const uint32_t F = in->n_fills;
    int st = OCHRE_OK;
    // 1. command scan of the input
    OCHRE_CUDA_TRY(ctx->sk_cmd_foff.ensure(n * 4));
    OCHRE_CUDA_TRY(ctx->sk_cmd_mv.ensure(n * 4));
    OCHRE_CUDA_TRY(ctx->sk_cmd_ep.ensure(n * 4));
    OCHRE_CUDA_TRY(ctx->scan_status.ensure(scan_tiles(n) * sizeof(ScanStatus<CmdScan>)));
    if (!plan) OCHRE_CUDA_TRY(reset_scalars(ctx, s));
    OCHRE_LAUNCH(ctx, "stroke_cmd_scan", s, OCHRE_CUDA_TRY(launch_scan<CmdScan>(
        n, CmdIn{in->verbs, &ds->err},
        CmdOut{ctx->sk_cmd_foff.as<uint32_t>(), ctx->sk_cmd_mv.as<uint32_t>(), ctx->sk_cmd_ep.as<uint32_t>()},
        OpCmd{}, CmdScan{0, 0, 0}, ctx->scan_status.p, &ds->ticket, reinterpret_cast<CmdScan*>(&ds->n_floats),
        &ds->err, s)));
    if (!plan) {
        st = read_scalars(ctx, s);
        if (st != OCHRE_OK) return st;
        if (host_scalars(ctx)->n_floats > in->n_floats) return OCHRE_E_INVALID;
        st = check_device_error(ctx);
        if (st != OCHRE_OK) return st;
    }
    // 2. polyline
    wait_inputs(ctx, s);   // path-space flatten counts read points
    OCHRE_CUDA_TRY(ctx->sk_poly_off.ensure((n + 1) * 4));
    OCHRE_CUDA_TRY(ctx->sk_poly_foff.ensure((n + 1) * 4));
    OCHRE_CUDA_TRY(ctx->scan_status.ensure(scan_tiles(n) * sizeof(ScanStatus<Pair>)));
    OCHRE_LAUNCH(ctx, "stroke_poly_count", s, k_pair_count<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(
        n, nullptr,
        PolyCount{in->verbs, in->pts, in->fill_cmd_off, F, in->fill_flags, ctx->sk_cmd_foff.as<uint32_t>(),
                  ctx->sk_cmd_ep.as<uint32_t>(), &ds->err},
        ctx->sk_poly_off.as<uint32_t>(), ctx->sk_poly_foff.as<uint32_t>()));
    OCHRE_CUDA_TRY(cudaGetLastError());
    OCHRE_LAUNCH(ctx, "stroke_poly_scan", s, OCHRE_CUDA_TRY(launch_scan<Pair>(
        n, PairIn{ctx->sk_poly_off.as<uint32_t>(), ctx->sk_poly_foff.as<uint32_t>()},
        PairOut{ctx->sk_poly_off.as<uint32_t>(), ctx->sk_poly_foff.as<uint32_t>()}, OpPair{}, Pair{0u, 0u},
        ctx->scan_status.p, &ds->ticket, reinterpret_cast<Pair*>(&ds->n_lines), &ds->err, s)));
    // (n_lines, n_line_ent) hold the polyline totals here; the fill chain resets them
    uint32_t P, PF;   // polyline commands and floats (planned: the capacities)
    if (plan) {
        P = plan->stroke_poly;
        PF = plan->stroke_poly_floats;
        OCHRE_LAUNCH(ctx, "plan_stroke_poly", s,
                     k_stroke_cap<<<1, 1, 0, s>>>(&ds->n_lines, P, &ds->n_line_ent, PF, &ds->n_tiles, &ds->err));
        OCHRE_CUDA_TRY(cudaGetLastError());
    } else {
        st = read_scalars(ctx, s);
        if (st != OCHRE_OK) return st;
        st = check_device_error(ctx);
        if (st != OCHRE_OK) return st;
        P = host_scalars(ctx)->n_lines;
        PF = host_scalars(ctx)->n_line_ent;
        if (P > MAX_COUNT) return OCHRE_E_CAPACITY;
        ctx->stroke_counts[0] = P;
        ctx->stroke_counts[1] = PF;
    }
    const uint32_t* p_dev = plan ? &ds->n_lines : nullptr;
    OCHRE_CUDA_TRY(ctx->sk_pverbs.ensure(P ? P : 1));
    OCHRE_CUDA_TRY(ctx->sk_ppts.ensure((size_t)(PF ? PF : 1) * 4));
    OCHRE_CUDA_TRY(ctx->sk_pfoff.ensure((size_t)(P ? P : 1) * 4));
    OCHRE_CUDA_TRY(ctx->sk_pfill_off.ensure(((size_t)F + 1) * 4));
    OCHRE_CUDA_TRY(ctx->sk_first_close.ensure((size_t)F * 4));
    const unsigned cb = (unsigned)((n + 255) / 256);
    OCHRE_LAUNCH(ctx, "stroke_poly_emit", s, k_poly_emit<<<cb, 256, 0, s>>>(
        in->verbs, in->pts, in->fill_cmd_off, F, in->fill_flags, n, ctx->sk_cmd_foff.as<uint32_t>(),
        ctx->sk_cmd_ep.as<uint32_t>(), ctx->sk_poly_off.as<uint32_t>(), ctx->sk_poly_foff.as<uint32_t>(),
        ctx->sk_pverbs.as<uint8_t>(), ctx->sk_ppts.as<float>(), P, PF));
    OCHRE_LAUNCH(ctx, "stroke_fill_init", s, k_fill_init<<<(F + 256) / 256, 256, 0, s>>>(
        ctx->sk_first_close.as<uint32_t>(), in->fill_cmd_off, ctx->sk_poly_off.as<uint32_t>(), n, P, p_dev, F,
        ctx->sk_pfill_off.as<uint32_t>()));
    OCHRE_CUDA_TRY(cudaGetLastError());
    if (P == 0) {
        ctx->stroke_counts[2] = ctx->stroke_counts[3] = 0;
        out->n_cmds = 0;
        out->n_floats = 0;
        OCHRE_CUDA_TRY(ctx->sk_ofill_off.ensure(((size_t)F + 1) * 4));
        OCHRE_CUDA_TRY(cudaMemsetAsync(ctx->sk_ofill_off.p, 0, ((size_t)F + 1) * 4, s));
        out->fill_cmd_off = ctx->sk_ofill_off.as<uint32_t>();
        return OCHRE_OK;
    }
    // float offset of every polyline command: an exclusive scan of its float counts
    OCHRE_CUDA_TRY(ctx->scan_status.ensure(scan_tiles(P) * sizeof(ScanStatus<uint32_t>)));
    OCHRE_LAUNCH(ctx, "stroke_pfoff_scan", s, OCHRE_CUDA_TRY(launch_scan<uint32_t>(
        P, PolyFloats{ctx->sk_pverbs.as<uint8_t>()}, OffOutU32{ctx->sk_pfoff.as<uint32_t>()}, OpSumU32{}, 0u,
        ctx->scan_status.p, &ds->ticket, static_cast<uint32_t*>(nullptr), &ds->err, s, p_dev)));
    OCHRE_LAUNCH(ctx, "stroke_first_close", s, k_first_close<<<(P + 255) / 256, 256, 0, s>>>(
        ctx->sk_pverbs.as<uint8_t>(), P, p_dev, ctx->sk_pfill_off.as<uint32_t>(), F, in->fill_flags,
        ctx->sk_first_close.as<uint32_t>()));
    OCHRE_CUDA_TRY(cudaGetLastError());
    // 3. units
    OCHRE_CUDA_TRY(ctx->sk_unit_start.ensure((size_t)P * 4));
    OCHRE_LAUNCH(ctx, "stroke_unit_scan", s, OCHRE_CUDA_TRY(launch_scan<uint32_t>(
        P, UnitIn{ctx->sk_pverbs.as<uint8_t>(), ctx->sk_pfill_off.as<uint32_t>(), F, in->fill_flags},
        UnitOut{ctx->sk_unit_start.as<uint32_t>()}, OpSumU32{}, 0u, ctx->scan_status.p, &ds->ticket,
        &ds->n_tiles, &ds->err, s, p_dev)));
    uint32_t U;   // units (planned: at most P, the count stays on the device)
    if (plan) {
        U = P;
    } else {
        st = read_scalars(ctx, s);
        if (st != OCHRE_OK) return st;
        st = check_device_error(ctx);
        if (st != OCHRE_OK) return st;
        U = host_scalars(ctx)->n_tiles;
    }
    const uint32_t* u_dev = plan ? &ds->n_tiles : nullptr;
    // 4. output sizes and emission
    OCHRE_CUDA_TRY(ctx->sk_out_off.ensure(((size_t)U + 1) * 4));
    OCHRE_CUDA_TRY(ctx->sk_out_foff.ensure(((size_t)U + 1) * 4));
    OCHRE_CUDA_TRY(ctx->sk_unit_fill.ensure(((size_t)U + 1) * 4));
    OCHRE_CUDA_TRY(ctx->scan_status.ensure(scan_tiles(U ? U : 1) * sizeof(ScanStatus<Pair>)));
    // the output totals: a scan that covers no unit writes none
    OCHRE_CUDA_TRY(cudaMemsetAsync(&ds->n_lines, 0, 8, s));
    if (U) {
        OCHRE_LAUNCH(ctx, "stroke_out_count", s, k_out_count<<<(unsigned)(((uint64_t)U * 32 + 127) / 128), 128, 0, s>>>(
            U, u_dev, ctx->sk_unit_start.as<uint32_t>(), ctx->sk_pverbs.as<uint8_t>(), ctx->sk_ppts.as<float>(),
            ctx->sk_pfoff.as<uint32_t>(), ctx->sk_pfill_off.as<uint32_t>(), F, in->fill_flags,
            ctx->sk_first_close.as<uint32_t>(), in->fill_width, ctx->sk_out_off.as<uint32_t>(),
            ctx->sk_out_foff.as<uint32_t>()));
        OCHRE_CUDA_TRY(cudaGetLastError());
        OCHRE_LAUNCH(ctx, "stroke_out_scan", s, OCHRE_CUDA_TRY(launch_scan<Pair>(
            U, PairIn{ctx->sk_out_off.as<uint32_t>(), ctx->sk_out_foff.as<uint32_t>()},
            PairOut{ctx->sk_out_off.as<uint32_t>(), ctx->sk_out_foff.as<uint32_t>()}, OpPair{}, Pair{0u, 0u},
            ctx->scan_status.p, &ds->ticket, reinterpret_cast<Pair*>(&ds->n_lines), &ds->err, s, u_dev)));
    }
    uint32_t ON, OF;   // output commands and floats (planned: the capacities)
    if (plan) {
        ON = plan->stroke_cmds;
        OF = plan->stroke_floats;
        OCHRE_LAUNCH(ctx, "plan_stroke_out", s,
                     k_stroke_cap<<<1, 1, 0, s>>>(&ds->n_lines, ON, &ds->n_line_ent, OF, &ds->n_tiles, &ds->err));
        OCHRE_CUDA_TRY(cudaGetLastError());
    } else {
        st = read_scalars(ctx, s);
        if (st != OCHRE_OK) return st;
        st = check_device_error(ctx);
        if (st != OCHRE_OK) return st;
        ON = host_scalars(ctx)->n_lines;
        OF = host_scalars(ctx)->n_line_ent;
        if (ON > MAX_COUNT) return OCHRE_E_CAPACITY;
        ctx->stroke_counts[2] = ON;
        ctx->stroke_counts[3] = OF;
    }
    OCHRE_CUDA_TRY(ctx->sk_overbs.ensure(ON ? ON : 1));
    OCHRE_CUDA_TRY(ctx->sk_opts.ensure((size_t)(OF ? OF : 1) * 4));
    OCHRE_CUDA_TRY(ctx->sk_ofill_off.ensure(((size_t)F + 1) * 4));
    OCHRE_CUDA_TRY(ctx->sk_oflags.ensure(F));
    // planned: every output command past the true total is a Close
    if (plan) OCHRE_CUDA_TRY(cudaMemsetAsync(ctx->sk_overbs.p, V_CLOSE, ON, s));
    if (U)
        OCHRE_LAUNCH(ctx, "stroke_out_emit", s, k_out_emit<<<(unsigned)(((uint64_t)U * 32 + 127) / 128), 128, 0, s>>>(
            U, u_dev, ctx->sk_unit_start.as<uint32_t>(), ctx->sk_pverbs.as<uint8_t>(), ctx->sk_ppts.as<float>(),
            ctx->sk_pfoff.as<uint32_t>(), ctx->sk_pfill_off.as<uint32_t>(), F, in->fill_flags,
            ctx->sk_first_close.as<uint32_t>(), in->fill_width, ctx->sk_out_off.as<uint32_t>(),
            ctx->sk_out_foff.as<uint32_t>(), ctx->sk_overbs.as<uint8_t>(), ctx->sk_opts.as<float>(),
            ctx->sk_unit_fill.as<uint32_t>()));
    OCHRE_LAUNCH(ctx, "stroke_fill_off", s, k_out_fill_off<<<(F + 256) / 256, 256, 0, s>>>(
        ctx->sk_unit_fill.as<uint32_t>(), U, u_dev, ctx->sk_out_off.as<uint32_t>(), ON, plan ? &ds->n_lines : nullptr,
        plan ? ON : 0u, F, ctx->sk_ofill_off.as<uint32_t>(), in->fill_flags, ctx->sk_oflags.as<uint8_t>()));
    OCHRE_CUDA_TRY(cudaGetLastError());
    out->verbs = ctx->sk_overbs.as<uint8_t>();
    out->n_cmds = ON;
    out->pts = ctx->sk_opts.as<float>();
    out->n_floats = OF;
    out->fill_cmd_off = ctx->sk_ofill_off.as<uint32_t>();
    out->fill_flags = ctx->sk_oflags.as<uint8_t>();
    return OCHRE_OK;
}

}  // namespace ochre
