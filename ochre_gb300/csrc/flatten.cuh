// Command context shared by the flattening stage and the backward pass:
// everything one command's flattening depends on (its transformed points,
// the rasterizer's `last` and `first` before it, and whether it ends its
// raster), reconstructed from the command scan (float offset, most recent
// Move, most recent non-Close command).
#pragma once

#include "common.cuh"
#include "internal.h"

namespace ochre {

struct BatchView {
    const uint8_t* verbs;
    const float* pts;
    const uint32_t* fill_off;
    const float* fill_xf;
    const uint8_t* fill_flags;
    const uint32_t* raster_off;
    uint32_t n_fills, n_rasters;
    uint64_t n_cmds;
    const uint32_t* cmd_foff;
    const uint32_t* cmd_mv;
    const uint32_t* cmd_ep;
    uint64_t n_floats;   // floats in pts: a command whose points lie beyond is invalid
};

// Command j's floats lie inside the point array.
__device__ __forceinline__ bool cmd_in_bounds(const BatchView& b, uint32_t j) {
    return (uint64_t)__ldg(b.cmd_foff + j) + floats_per_verb(__ldg(b.verbs + j)) <= b.n_floats;
}

// Everything a command's flattening depends on.
struct CmdCtx {
    uint8_t verb;
    uint32_t raster;
    bool last_of_raster;
    V2 last, first;   // rasterizer state before the command
    V2 pt[3];         // transformed points of the command
    float w;          // conic weight
    bool ok;
    int64_t last_ref;   // command whose end point is `last`, or -1 for (0,0)
    int64_t first_ref;  // Move command whose point is `first`, or -1 for (0,0)
    uint32_t fill;
};

// Command scan: float offset, most recent Move, most recent non-Close
// command, per command (exclusive), in one pass.
struct CmdScan {
    uint32_t foff;   // exclusive sum of floats consumed
    uint32_t mv;     // 1 + index of the most recent Move (0: none)
    uint32_t ep;     // 1 + index of the most recent non-Close command (0: none)
};
struct OpCmd {
    __device__ __forceinline__ CmdScan operator()(CmdScan a, CmdScan b) const {
        return CmdScan{a.foff + b.foff, max(a.mv, b.mv), max(a.ep, b.ep)};
    }
};
struct CmdIn {
    const uint8_t* verbs;
    uint32_t* err;
    __device__ __forceinline__ CmdScan operator()(uint64_t i) const {
        const uint8_t v = verbs[i];
        if (v > V_CLOSE) atomicOr(err, ERR_INVALID);
        const uint32_t id = (uint32_t)i + 1u;
        return CmdScan{floats_per_verb(v), v == V_MOVE ? id : 0u, v <= V_CONIC ? id : 0u};
    }
};
struct CmdOut {
    uint32_t* foff;
    uint32_t* mv;
    uint32_t* ep;
    __device__ __forceinline__ void operator()(uint64_t i, CmdScan ex, CmdScan) const {
        foff[i] = ex.foff;
        mv[i] = ex.mv;
        ep[i] = ex.ep;
    }
};

__device__ __forceinline__ uint32_t fill_of(const BatchView& b, uint32_t c) {
    return upper_bound_u32(b.fill_off, b.n_fills + 1, c) - 1u;
}

// The transformed end point of command j (a non-Close command).
__device__ __forceinline__ V2 endpoint_of(const BatchView& b, uint32_t j, uint32_t f_hint) {
    const uint32_t f = j >= __ldg(b.fill_off + f_hint) ? f_hint : fill_of(b, j);
    const uint8_t v = __ldg(b.verbs + j);
    const float* fp = b.pts + __ldg(b.cmd_foff + j) + endpoint_float(v);
    V2 p = v2(__ldg(fp), __ldg(fp + 1));
    const bool raw = b.fill_flags != nullptr && (__ldg(b.fill_flags + f) & OCHRE_FILL_RAW);
    if (!raw) p = xf_apply(b.fill_xf + 6 * (size_t)f, p);
    return p;
}

__device__ inline CmdCtx load_cmd(const BatchView& b, uint32_t c) {
    CmdCtx k;
    k.ok = true;
    k.verb = __ldg(b.verbs + c);
    const uint32_t f = fill_of(b, c);
    uint32_t r, rf0, rf1;
    if (b.raster_off != nullptr) {
        r = upper_bound_u32(b.raster_off, b.n_rasters + 1, f) - 1u;
        rf0 = __ldg(b.raster_off + r);
        rf1 = __ldg(b.raster_off + r + 1);
    } else {
        r = f;
        rf0 = f;
        rf1 = f + 1;
    }
    k.raster = r;
    const uint32_t rc0 = __ldg(b.fill_off + rf0), rc1 = __ldg(b.fill_off + rf1);
    k.last_of_raster = c + 1 == rc1;
    const uint32_t ep = __ldg(b.cmd_ep + c), mv = __ldg(b.cmd_mv + c);
    k.fill = f;
    k.last_ref = ep > rc0 ? (int64_t)(ep - 1u) : -1;
    k.first_ref = mv > rc0 ? (int64_t)(mv - 1u) : -1;
    // every command read below must lie inside the point array
    if (!cmd_in_bounds(b, c) || (ep > rc0 && !cmd_in_bounds(b, ep - 1u)) || (mv > rc0 && !cmd_in_bounds(b, mv - 1u))) {
        k.ok = false;
        k.last = k.first = k.pt[0] = k.pt[1] = k.pt[2] = v2(0.0f, 0.0f);
        k.w = 0.0f;
        return k;
    }
    k.last = ep > rc0 ? endpoint_of(b, ep - 1u, f) : v2(0.0f, 0.0f);
    if (mv > rc0) {
        const uint32_t m = mv - 1u;
        const uint32_t fm = m >= __ldg(b.fill_off + f) ? f : fill_of(b, m);
        const float* fp = b.pts + __ldg(b.cmd_foff + m);
        V2 p = v2(__ldg(fp), __ldg(fp + 1));
        const bool raw = b.fill_flags != nullptr && (__ldg(b.fill_flags + fm) & OCHRE_FILL_RAW);
        k.first = raw ? p : xf_apply(b.fill_xf + 6 * (size_t)fm, p);
    } else {
        k.first = v2(0.0f, 0.0f);
    }
    const bool raw = b.fill_flags != nullptr && (__ldg(b.fill_flags + f) & OCHRE_FILL_RAW);
    const float* xf = b.fill_xf + 6 * (size_t)f;
    const float* fp = b.pts + __ldg(b.cmd_foff + c);
    const int np = k.verb == V_MOVE || k.verb == V_LINE ? 1 : k.verb == V_QUAD || k.verb == V_CONIC ? 2
                 : k.verb == V_CUBIC ? 3 : 0;
    for (int q = 0; q < 3; q++) {
        if (q < np) {
            V2 p = v2(__ldg(fp + 2 * q), __ldg(fp + 2 * q + 1));
            if (!raw) p = xf_apply(xf, p);   // PathCmd::transform (path.rs:16-37)
            if (!finite2(p)) k.ok = false;
            k.pt[q] = p;
        } else {
            k.pt[q] = v2(0.0f, 0.0f);
        }
    }
    k.w = k.verb == V_CONIC ? __ldg(fp + 4) : 0.0f;
    if (k.verb == V_CONIC && !isfinite(k.w)) k.ok = false;
    return k;
}

}  // namespace ochre
