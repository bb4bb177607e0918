// Device helpers shared by every kernel of the rasterization chain.
//
// Bit-exactness: the discrete structure (segment counts, visited pixel
// cells, tile set, tile-row crossings) depends on serial f32 recurrences in
// the reference (path.rs:52-57, 65-73; rasterizer.rs:97-136).  Every float
// operation below that feeds it is an explicit round-to-nearest intrinsic in
// the reference's evaluation order, so the result does not depend on
// -fmad (which the build also turns off).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace ochre {

constexpr int TILE = 8;                // rasterizer.rs:4
constexpr float TOLERANCE = 0.1f;      // rasterizer.rs:6

// Verb codes (path.rs:5-12) and floats consumed per verb.
enum : uint8_t { V_MOVE = 0, V_LINE = 1, V_QUAD = 2, V_CUBIC = 3, V_CONIC = 4, V_CLOSE = 5 };
__host__ __device__ inline uint32_t floats_per_verb(uint8_t v) {
    // MOVE 2, LINE 2, QUAD 4, CUBIC 6, CONIC 5, CLOSE 0
    return v == V_MOVE || v == V_LINE ? 2u : v == V_QUAD ? 4u : v == V_CUBIC ? 6u : v == V_CONIC ? 5u : 0u;
}
// Float index (within the command) of the command's end point.
__host__ __device__ inline uint32_t endpoint_float(uint8_t v) {
    return v == V_QUAD || v == V_CONIC ? 2u : v == V_CUBIC ? 4u : 0u;
}

// Device error bits, ORed into the context's status word.
enum : uint32_t {
    ERR_TIMEOUT = 1u,    // a bounded wait gave up
    ERR_LIMIT = 2u,      // flatten / walk / conic-depth cap
    ERR_INVALID = 4u,    // non-finite point or malformed command
    ERR_CAPACITY = 8u,   // a count exceeded a buffer
};

// Caps: the reference loops (or allocates) without bound past these.
constexpr uint32_t FLATTEN_CAP = 1u << 20;   // lines per curve segment
constexpr uint32_t WALK_CAP = 1u << 20;      // pixel cells per line
constexpr int CONIC_DEPTH_CAP = 40;          // conic subdivision depth
constexpr long long SPIN_LIMIT = 1ll << 21;  // polls of a look-back flag (about a second under load)
// Word index, counted from the run's error word, of the run's poll-limit
// override (log2 of the limit; 0: SPIN_LIMIT).  Every kernel that waits is
// given the address of the error word of its run's device scalars, which
// holds both (internal.h checks the layout).
constexpr int SPIN_LOG2_WORD = 22;

// The count a kernel works on: its launch-time value, or, when the count is
// held on the device (launch chains replayed from a CUDA graph), the device
// value, never more than the launch-time capacity.
__device__ __forceinline__ uint64_t dev_count(uint64_t cap, const uint32_t* n_dev) {
    return n_dev != nullptr ? min(cap, (uint64_t)*n_dev) : cap;
}

// ---------------------------------------------------------------------
// Rust scalar semantics
// ---------------------------------------------------------------------
// `v as i16`: truncate toward zero, saturate, NaN -> 0.
__device__ __forceinline__ int f2i16(float v) {
    if (v != v) return 0;
    if (v <= -32768.0f) return -32768;
    if (v >= 32767.0f) return 32767;
    return __float2int_rz(v);
}
// `v as u8`: truncate toward zero, saturate, NaN -> 0.
__device__ __forceinline__ uint32_t f2u8(float v) {
    if (!(v > 0.0f)) return 0u;
    if (v >= 255.0f) return 255u;
    return __float2uint_rz(v);
}
// `(v).signum() as i16`: +-1 by sign bit, NaN -> 0.
__device__ __forceinline__ int signum_i16(float v) {
    if (v != v) return 0;
    return signbit(v) ? -1 : 1;
}
// i16 wrapping arithmetic.
__device__ __forceinline__ int wrap16(int v) { return (int)(int16_t)v; }
// i16::wrapping_div_euclid(8) == arithmetic shift for a two's complement i16.
__device__ __forceinline__ int div8(int v) { return v >> 3; }
// f32::min / f32::max: the non-NaN operand wins (IEEE minNum / maxNum).
__device__ __forceinline__ float rmin(float a, float b) { return fminf(a, b); }
__device__ __forceinline__ float rmax(float a, float b) { return fmaxf(a, b); }

// ---------------------------------------------------------------------
// geom.rs restated with explicit rounding
// ---------------------------------------------------------------------
struct V2 { float x, y; };
__device__ __forceinline__ V2 v2(float x, float y) { return V2{x, y}; }
__device__ __forceinline__ V2 vadd(V2 a, V2 b) { return v2(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y)); }
__device__ __forceinline__ V2 vsub(V2 a, V2 b) { return v2(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y)); }
__device__ __forceinline__ V2 vscale(float s, V2 a) { return v2(__fmul_rn(s, a.x), __fmul_rn(s, a.y)); }
__device__ __forceinline__ bool veq(V2 a, V2 b) { return a.x == b.x && a.y == b.y; }
// Vec2::length = sqrt(x*x + y*y)  (geom.rs:19-21, 38-40)
__device__ __forceinline__ float vlength(V2 a) {
    return __fsqrt_rn(__fadd_rn(__fmul_rn(a.x, a.x), __fmul_rn(a.y, a.y)));
}
// Vec2::lerp(t, a, b) = (1 - t) * a + t * b  (geom.rs:50-52)
__device__ __forceinline__ V2 vlerp(float t, V2 a, V2 b) {
    const float u = __fsub_rn(1.0f, t);
    return v2(__fadd_rn(__fmul_rn(u, a.x), __fmul_rn(t, b.x)), __fadd_rn(__fmul_rn(u, a.y), __fmul_rn(t, b.y)));
}
// Transform::apply = matrix * v + offset, row-major matrix (geom.rs:170-178, 260-262)
__device__ __forceinline__ V2 xf_apply(const float* xf, V2 v) {
    const float mx = __fadd_rn(__fmul_rn(xf[0], v.x), __fmul_rn(xf[1], v.y));
    const float my = __fadd_rn(__fmul_rn(xf[2], v.x), __fmul_rn(xf[3], v.y));
    return v2(__fadd_rn(mx, xf[4]), __fadd_rn(my, xf[5]));
}
__device__ __forceinline__ bool finite2(V2 p) { return isfinite(p.x) && isfinite(p.y); }

// ---------------------------------------------------------------------
// Flattening (path.rs:49-104): parameter step and serial t recurrence.
// ---------------------------------------------------------------------
// dt for a quadratic: sqrt((4 * tol) / |last - 2c + p|)       path.rs:50
__device__ __forceinline__ float quad_dt(V2 last, V2 c, V2 p) {
    const V2 v = vadd(vsub(last, vscale(2.0f, c)), p);
    return __fsqrt_rn(__fdiv_rn(__fmul_rn(4.0f, TOLERANCE), vlength(v)));
}
// dt for a cubic: sqrt((sqrt(8) * tol) / max(|b|, |a + b|))   path.rs:60-63
__device__ __forceinline__ float cubic_dt(V2 last, V2 c1, V2 c2, V2 p) {
    const V2 a = vadd(vsub(vadd(vscale(-1.0f, last), vscale(3.0f, c1)), vscale(3.0f, c2)), p);
    const V2 b = vscale(3.0f, vadd(vsub(last, vscale(2.0f, c1)), c2));
    const float conc = rmax(vlength(b), vlength(vadd(a, b)));
    return __fsqrt_rn(__fdiv_rn(__fmul_rn(__fsqrt_rn(8.0f), TOLERANCE), conc));
}
// Number of iterations of `while t < 1 { t = min(t + dt, 1) }`, capped.
__device__ __forceinline__ uint32_t flatten_steps(float dt, bool* capped) {
    float t = 0.0f;
    uint32_t n = 0;
    while (t < 1.0f) {
        t = rmin(__fadd_rn(t, dt), 1.0f);
        if (++n >= FLATTEN_CAP) { *capped = true; break; }
    }
    return n;
}
__device__ __forceinline__ V2 quad_point(float t, V2 last, V2 c, V2 p) {
    return vlerp(t, vlerp(t, last, c), vlerp(t, c, p));
}
__device__ __forceinline__ V2 cubic_point(float t, V2 last, V2 c1, V2 c2, V2 p) {
    const V2 p01 = vlerp(t, last, c1), p12 = vlerp(t, c1, c2), p23 = vlerp(t, c2, p);
    return vlerp(t, vlerp(t, p01, p12), vlerp(t, p12, p23));
}

// Conic subdivision (path.rs:76-101) as an explicit depth-first stack.
// `emit(point)` is called for every line_to target in the reference's order.
struct ConicFrame { float t0, t1; V2 p0, p1; int depth; };
template <class Emit>
__device__ void conic_flatten(V2 last, V2 control, V2 point, float w, bool* capped, Emit emit) {
    ConicFrame stack[CONIC_DEPTH_CAP + 2];
    int sp = 0;
    stack[sp++] = ConicFrame{0.0f, 1.0f, last, point, 0};
    const V2 wc = vscale(w, control);
    while (sp > 0) {
        const ConicFrame f = stack[--sp];
        const float t = __fmul_rn(0.5f, __fadd_rn(f.t0, f.t1));
        const V2 p01 = vlerp(t, last, wc);
        const V2 p12 = vlerp(t, wc, point);
        const float u = __fsub_rn(1.0f, t);
        // (1-t)*(1-t) + 2*t*(1-t)*w + t*t, left to right
        const float denom = __fadd_rn(__fadd_rn(__fmul_rn(u, u), __fmul_rn(__fmul_rn(__fmul_rn(2.0f, t), u), w)),
                                      __fmul_rn(t, t));
        const V2 mid = vscale(__fdiv_rn(1.0f, denom), vlerp(t, p01, p12));
        const float err = vlength(vsub(mid, vscale(0.5f, vadd(f.p0, f.p1))));
        if (err > TOLERANCE) {
            if (f.depth >= CONIC_DEPTH_CAP) { *capped = true; return; }
            stack[sp++] = ConicFrame{t, f.t1, mid, f.p1, f.depth + 1};   // right half, after
            stack[sp++] = ConicFrame{f.t0, t, f.p0, mid, f.depth + 1};   // left half, first
        } else {
            emit(mid);
            emit(f.p1);
        }
    }
}

// The same subdivision, reporting with every emitted point its parameter t
// on the conic (the midpoint of a leaf, then the leaf's end): the adjoint
// needs t to differentiate the emitted points.
template <class Emit>
__device__ void conic_flatten_t(V2 last, V2 control, V2 point, float w, bool* capped, Emit emit) {
    ConicFrame stack[CONIC_DEPTH_CAP + 2];
    int sp = 0;
    stack[sp++] = ConicFrame{0.0f, 1.0f, last, point, 0};
    const V2 wc = vscale(w, control);
    while (sp > 0) {
        const ConicFrame f = stack[--sp];
        const float t = __fmul_rn(0.5f, __fadd_rn(f.t0, f.t1));
        const V2 p01 = vlerp(t, last, wc);
        const V2 p12 = vlerp(t, wc, point);
        const float u = __fsub_rn(1.0f, t);
        const float denom = __fadd_rn(__fadd_rn(__fmul_rn(u, u), __fmul_rn(__fmul_rn(__fmul_rn(2.0f, t), u), w)),
                                      __fmul_rn(t, t));
        const V2 mid = vscale(__fdiv_rn(1.0f, denom), vlerp(t, p01, p12));
        const float err = vlength(vsub(mid, vscale(0.5f, vadd(f.p0, f.p1))));
        if (err > TOLERANCE) {
            if (f.depth >= CONIC_DEPTH_CAP) { *capped = true; return; }
            stack[sp++] = ConicFrame{t, f.t1, mid, f.p1, f.depth + 1};
            stack[sp++] = ConicFrame{f.t0, t, f.p0, mid, f.depth + 1};
        } else {
            emit(mid, t);
            emit(f.p1, f.t1);
        }
    }
}

// ---------------------------------------------------------------------
// The pixel DDA of rasterizer.rs:72-136.
// ---------------------------------------------------------------------
struct Walk {
    V2 a, p;                 // self.last, point
    int x_dir, y_dir;        // signum as i16
    float x_step, y_step;    // |dtdx|, |dtdy|
    int end_x, end_y;        // floor(point) as i16 (the snap target)
};
struct WalkState {
    int x, y;                // current cell (i16 values)
    float row_t0, row_t1, col_t0, col_t1;
};

// Setup (rasterizer.rs:74-95).  Caller ensures a != p.
__device__ __forceinline__ void walk_setup(V2 a, V2 p, Walk& w, WalkState& s) {
    w.a = a;
    w.p = p;
    w.x_dir = signum_i16(__fsub_rn(p.x, a.x));
    w.y_dir = signum_i16(__fsub_rn(p.y, a.y));
    const float dtdx = __fdiv_rn(1.0f, __fsub_rn(p.x, a.x));
    const float dtdy = __fdiv_rn(1.0f, __fsub_rn(p.y, a.y));
    s.x = f2i16(floorf(a.x));
    s.y = f2i16(floorf(a.y));
    s.row_t0 = 0.0f;
    s.col_t0 = 0.0f;
    if (a.y == p.y) {
        s.row_t1 = __int_as_float(0x7f800000);
    } else {
        const float next_y = p.y > a.y ? (float)wrap16(s.y + 1) : (float)s.y;
        s.row_t1 = rmin(__fmul_rn(dtdy, __fsub_rn(next_y, a.y)), 1.0f);
    }
    if (a.x == p.x) {
        s.col_t1 = __int_as_float(0x7f800000);
    } else {
        const float next_x = p.x > a.x ? (float)wrap16(s.x + 1) : (float)s.x;
        s.col_t1 = rmin(__fmul_rn(dtdx, __fsub_rn(next_x, a.x)), 1.0f);
    }
    w.x_step = fabsf(dtdx);
    w.y_step = fabsf(dtdy);
    w.end_x = f2i16(floorf(p.x));
    w.end_y = f2i16(floorf(p.y));
}

// The increment pushed for the current cell (rasterizer.rs:98-106).
__device__ __forceinline__ void walk_increment(const Walk& w, const WalkState& s, float& area, float& height) {
    const float t0 = rmax(s.row_t0, s.col_t0);
    const float t1 = rmin(s.row_t1, s.col_t1);
    const V2 p0 = vlerp(t0, w.a, w.p);
    const V2 p1 = vlerp(t1, w.a, w.p);
    height = __fsub_rn(p1.y, p0.y);
    const float right = (float)wrap16(s.x + 1);
    area = __fmul_rn(__fmul_rn(0.5f, height), __fadd_rn(__fsub_rn(right, p0.x), __fsub_rn(right, p1.x)));
}

// One step (rasterizer.rs:108-121).  Returns true when the walk ends; the
// cell is then the snapped end cell, which receives no increment.
__device__ __forceinline__ bool walk_step(const Walk& w, WalkState& s) {
    if (s.row_t1 < s.col_t1) {
        s.row_t0 = s.row_t1;
        s.row_t1 = rmin(__fadd_rn(s.row_t1, w.y_step), 1.0f);
        s.y = wrap16(s.y + w.y_dir);
    } else {
        s.col_t0 = s.col_t1;
        s.col_t1 = rmin(__fadd_rn(s.col_t1, w.x_step), 1.0f);
        s.x = wrap16(s.x + w.x_dir);
    }
    const bool done = s.row_t0 == 1.0f || s.col_t0 == 1.0f;
    if (done) {
        s.x = w.end_x;
        s.y = w.end_y;
    }
    return done;
}

// Full walk of one line.  For every increment cell: on_cell(state);
// for every tile-row crossing (rasterizer.rs:123-131):
// on_cross(tile_x, tile_y, sign); for every visited cell including the
// snapped end cell: on_visit(x, y).  Returns false if the walk cap was hit.
template <class OnCell, class OnCross, class OnVisit>
__device__ __forceinline__ bool walk_line(V2 a, V2 p, OnCell on_cell, OnCross on_cross, OnVisit on_visit) {
    Walk w;
    WalkState s;
    walk_setup(a, p, w, s);
    int tile_y_prev = div8(s.y);   // == div8(floor(last.y) as i16), see the invariant in dda.cu
    on_visit(s.x, s.y);
    for (uint32_t it = 0;; ++it) {
        on_cell(w, s);
        const bool done = walk_step(w, s);
        on_visit(s.x, s.y);
        const int tile_y = div8(s.y);
        if (tile_y != tile_y_prev) {
            on_cross(div8(s.x), min(tile_y_prev, tile_y), (int)(int8_t)(int16_t)(tile_y - tile_y_prev));
            tile_y_prev = tile_y;
        }
        if (done) return true;
        if (it + 1 >= WALK_CAP) return false;
    }
}

// Pixel cells a line's walk visits, about: its start cell and one per row
// or column step (the reference's walk may add a cell at a corner tie).
__device__ __forceinline__ uint32_t walk_cells(const float4& l) {
    const float dx = fabsf(floorf(l.z) - floorf(l.x)), dy = fabsf(floorf(l.w) - floorf(l.y));
    const float c = 1.0f + dx + dy;
    return c < 65535.0f ? (uint32_t)c : 65535u;   // also NaN -> 65535 (bucketed last)
}

// ---------------------------------------------------------------------
// Memory-order helpers for single-pass look-back chains.
// ---------------------------------------------------------------------
__device__ __forceinline__ uint32_t ld_acquire(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(uint32_t* p, uint32_t v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed(uint32_t* p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint64_t ld_relaxed64(const uint64_t* p) {
    uint64_t v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed64(uint64_t* p, uint64_t v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
// ---------------------------------------------------------------------
// Bounded waits with a run-wide abort.
// ---------------------------------------------------------------------
// A wait polls at most spin_limit(err) times.  The first wait that gives up
// sets ERR_TIMEOUT in the run's error word; every other wait of the run sees
// that bit within a few polls and gives up too, so a run whose waits cannot
// finish ends after about one wait's limit, not one limit per wait.
__device__ __forceinline__ long long spin_limit(const uint32_t* err) {
    const uint32_t k = ld_relaxed(err + SPIN_LOG2_WORD);
    return k == 0u ? SPIN_LIMIT : (1ll << min(k, 40u));
}
// One more poll by a single thread; true when it must stop waiting.
__device__ __forceinline__ bool wait_give_up(long long& spins, long long limit, uint32_t* err) {
    ++spins;
    if ((spins & 7) == 0 && (ld_relaxed(err) & ERR_TIMEOUT) != 0u) return true;
    if (spins > limit) {
        atomicOr(err, ERR_TIMEOUT);
        return true;
    }
    return false;
}
// The same for a wait a whole warp makes together: the answer is the same in
// every lane (every lane calls it with the same spins and limit).
__device__ __forceinline__ bool wait_give_up_warp(long long& spins, long long limit, uint32_t* err) {
    ++spins;
    const bool aborted = (spins & 7) == 0 && (ld_relaxed(err) & ERR_TIMEOUT) != 0u;
    if (__any_sync(0xffffffffu, aborted)) return true;
    if (spins > limit) {
        if ((threadIdx.x & 31) == 0) atomicOr(err, ERR_TIMEOUT);
        return true;
    }
    return false;
}
// A kernel that consumes the results of earlier waiting kernels of its run
// returns at once when one of them gave up (their outputs are not valid).
__device__ __forceinline__ bool run_aborted(const uint32_t* err) { return (ld_relaxed(err) & ERR_TIMEOUT) != 0u; }

// Look-back slots whose flag is a word of its own (the block-form coverage's
// row sums) publish data with relaxed stores followed by a release store of
// the flag; readers acquire the flag, then read the data relaxed.  The
// release/acquire pair orders the data, so no separate fence is needed.  (The
// scans, the radix sort and the fused kernel keep a flag in every word
// instead: one relaxed round reads flags and values together.)
// Word-wise read of a trivially copyable T through relaxed accesses.
template <class T>
__device__ __forceinline__ T ld_words(const T* src) {
    T v;
    uint32_t* d = reinterpret_cast<uint32_t*>(&v);
    const uint32_t* s = reinterpret_cast<const uint32_t*>(src);
#pragma unroll
    for (int i = 0; i < (int)(sizeof(T) / 4); i++) d[i] = ld_relaxed(s + i);
    return v;
}

// Shuffle of a trivially copyable T, word by word.
template <class T>
__device__ __forceinline__ T shfl_up_T(T v, int delta) {
    static_assert(sizeof(T) % 4 == 0, "T must be a multiple of 4 bytes");
    T r;
    const uint32_t* s = reinterpret_cast<const uint32_t*>(&v);
    uint32_t* d = reinterpret_cast<uint32_t*>(&r);
#pragma unroll
    for (int i = 0; i < (int)(sizeof(T) / 4); i++) d[i] = __shfl_up_sync(0xffffffffu, s[i], delta);
    return r;
}
template <class T>
__device__ __forceinline__ T shfl_down_T(T v, int delta) {
    static_assert(sizeof(T) % 4 == 0, "T must be a multiple of 4 bytes");
    T r;
    const uint32_t* s = reinterpret_cast<const uint32_t*>(&v);
    uint32_t* d = reinterpret_cast<uint32_t*>(&r);
#pragma unroll
    for (int i = 0; i < (int)(sizeof(T) / 4); i++) d[i] = __shfl_down_sync(0xffffffffu, s[i], delta);
    return r;
}
template <class T>
__device__ __forceinline__ T shfl_idx_T(T v, int lane) {
    T r;
    const uint32_t* s = reinterpret_cast<const uint32_t*>(&v);
    uint32_t* d = reinterpret_cast<uint32_t*>(&r);
#pragma unroll
    for (int i = 0; i < (int)(sizeof(T) / 4); i++) d[i] = __shfl_sync(0xffffffffu, s[i], lane);
    return r;
}

// Binary search: index of the last element <= v in sorted a[0..n).
__device__ __forceinline__ uint32_t upper_bound_u32(const uint32_t* a, uint32_t n, uint32_t v) {
    uint32_t lo = 0, hi = n;   // first index with a[i] > v
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(a + mid) <= v) lo = mid + 1; else hi = mid;
    }
    return lo;
}

}  // namespace ochre
