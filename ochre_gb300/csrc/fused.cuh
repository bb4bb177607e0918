// Shared by the two fused small-raster kernels (fused.cu: one CTA per
// raster; fused_warp.cu: one warp per raster): their launch arguments and the
// per-raster look-back that places each raster's tiles and spans in the
// output, in raster order.
#pragma once

#include "common.cuh"
#include "internal.h"

namespace ochre {

// Per-raster look-back slot: one 64-bit word holding a flag (bits 62-63: 0
// none, 1 aggregate, 2 inclusive) and two 30-bit counts (tiles in bits 0-29,
// spans in bits 30-59).  One naturally aligned 64-bit access reads or writes
// flag and counts together, so readers need no acquire/release pairing.
// Counts saturate at 2^30 - 1, above every output capacity.
constexpr uint64_t CH_AGG = 1ull << 62, CH_INC = 2ull << 62;
constexpr uint32_t CH_MAX = (1u << 30) - 1u;
__device__ __forceinline__ uint64_t ch_pack(uint64_t flag, uint32_t a0, uint32_t a1) {
    return flag | ((uint64_t)min(a1, CH_MAX) << 30) | min(a0, CH_MAX);
}
constexpr int CH_PER_LANE = 4;   // predecessors one lane reads per look-back round

// Publish raster r's counts: its aggregate, or, for raster 0, its inclusive
// value.  One thread.
__device__ __forceinline__ void chain_publish(uint64_t* slots, uint32_t r, uint32_t a0, uint32_t a1) {
    st_relaxed64(slots + r, ch_pack(r == 0 ? CH_INC : CH_AGG, a0, a1));
}

// Resolve raster r's exclusive prefix (its aggregate a0, a1 already
// published) by a warp-cooperative decoupled look-back over 32 x CH_PER_LANE
// predecessors per round (independent loads, one latency per round), and
// publish its inclusive value.  Predecessor q of a round (q = k * 32 + lane,
// nearest first) is raster top - q.  Called by one full warp; returns the
// prefix in every lane.  Every wait is bounded.
__device__ __forceinline__ void chain_lookback(uint64_t* slots, uint32_t r, uint32_t a0, uint32_t a1, uint32_t* err,
                                               uint32_t& p0, uint32_t& p1) {
    const int lane = threadIdx.x & 31;
    p0 = 0;
    p1 = 0;
    if (r == 0) return;
    int64_t top = (int64_t)r - 1;   // nearest predecessor not yet summed
    long long spins = 0;
    const long long poll_limit = spin_limit(err);
    while (top >= 0) {
        uint64_t w[CH_PER_LANE];
#pragma unroll
        for (int k = 0; k < CH_PER_LANE; k++) {
            const int64_t j = top - (k * 32 + lane);
            w[k] = j >= 0 ? ld_relaxed64(slots + j) : CH_INC;   // before raster 0: an inclusive zero
        }
        // nearest inclusive predecessor of the round: q_inc (32 * CH_PER_LANE if none)
        int q_inc = 32 * CH_PER_LANE;
#pragma unroll
        for (int k = CH_PER_LANE - 1; k >= 0; k--) {
            const uint32_t m2 = __ballot_sync(0xffffffffu, (w[k] >> 62) == 2u);
            if (m2) q_inc = k * 32 + __ffs(m2) - 1;
        }
        // every predecessor up to it must have published
        bool missing = false;
#pragma unroll
        for (int k = 0; k < CH_PER_LANE; k++) {
            const bool need = k * 32 + lane <= q_inc;
            if (__ballot_sync(0xffffffffu, need && (w[k] >> 62) == 0u)) missing = true;
        }
        if (missing) {
            if (wait_give_up_warp(spins, poll_limit, err)) break;
            if (spins > 16) __nanosleep(64);
            continue;
        }
        uint32_t v0 = 0, v1 = 0;
#pragma unroll
        for (int k = 0; k < CH_PER_LANE; k++) {
            if (k * 32 + lane <= q_inc) {
                v0 += (uint32_t)(w[k] & CH_MAX);
                v1 += (uint32_t)((w[k] >> 30) & CH_MAX);
            }
        }
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) {
            v0 += __shfl_xor_sync(0xffffffffu, v0, d);
            v1 += __shfl_xor_sync(0xffffffffu, v1, d);
        }
        p0 += v0;
        p1 += v1;
        if (q_inc < 32 * CH_PER_LANE) break;
        top -= 32 * CH_PER_LANE;
    }
    p0 = min(p0, CH_MAX);
    p1 = min(p1, CH_MAX);
    if (lane == 0) st_relaxed64(slots + r, ch_pack(CH_INC, p0 + a0, p1 + a1));
}

struct FusedArgs {
    const uint8_t* verbs;
    const float* pts;
    const uint32_t* cmd_foff;   // float offset of every command (exclusive scan of floats per verb)
    const uint32_t* fill_off;
    const float* fill_xf;
    const uint8_t* fill_flags;
    const uint32_t* raster_off;
    uint32_t n_fills, n_rasters;
    uint64_t n_floats;
    uint64_t* co;            // look-back slots of the output tiles / spans
    uint32_t* ticket;
    uint32_t* fallback;      // any raster did not fit
    uint32_t* err;
    uint32_t* totals;        // [0] tiles, [1] spans
    uint32_t tile_cap, span_cap;
    uint32_t* out_xy;
    uint8_t* out_alpha;
    float* out_cov;
    uint32_t* span_xy;
    uint16_t* span_w;
    uint32_t* span_tile;
    uint32_t* raster_tile_off;
    uint32_t* raster_span_off;
    uint8_t* stage_alpha;    // per CTA (or warp): its raster's staged alpha (and coverage when out_cov)
    float* stage_cov;
    uint32_t* frontier;      // warp form: every slot below it holds an inclusive value
    uint16_t* spill_id;      // warp form: per warp, increments past its shared-memory slots
    float2* spill_ah;
};

__device__ __forceinline__ V2 load_pt(const float* p) { return v2(__ldg(p), __ldg(p + 1)); }

// Helping the inclusive values along (warp form).  `frontier` is a raster
// index below which every slot holds its inclusive value.  A warp that has
// published its own aggregate reads the 128 slots from the frontier on (4
// consecutive slots per lane), turns the leading run of published slots into
// inclusive values (a segmented scan: an inclusive slot restarts the sum, an
// aggregate adds to it, seeded by the inclusive value just below the
// frontier) and moves the frontier past the run.  Never waits: with no
// published slot at the frontier it returns at once.  Inclusive values are a
// function of the published counts alone, so warps that help at the same
// time, and the owners' own look-backs, all write the same values.
// Called by one full warp.
__device__ __forceinline__ void frontier_help(uint64_t* slots, uint32_t* frontier, uint32_t n_rasters) {
    const int lane = threadIdx.x & 31;
    uint32_t f = 0;
    if (lane == 0) f = ld_acquire(frontier);
    f = __shfl_sync(0xffffffffu, f, 0);
    if (f >= n_rasters) return;
    uint32_t s0 = 0, s1 = 0;   // inclusive counts of slot f - 1
    if (f > 0) {
        const uint64_t v = ld_relaxed64(slots + f - 1);
        s0 = (uint32_t)(v & CH_MAX);
        s1 = (uint32_t)((v >> 30) & CH_MAX);
    }
    uint64_t w[4];
    int first_missing = 4;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const uint32_t j = f + 4u * (uint32_t)lane + (uint32_t)k;
        w[k] = j < n_rasters ? ld_relaxed64(slots + j) : 0ull;
        if ((w[k] >> 62) == 0u && first_missing == 4) first_missing = k;
    }
    const uint32_t mb = __ballot_sync(0xffffffffu, first_missing < 4);
    const int L = mb ? __ffs(mb) - 1 : 31;
    const int fm_L = __shfl_sync(0xffffffffu, first_missing, L);
    const int m = mb ? 4 * L + fm_L : 128;   // leading run of published slots
    if (m == 0) return;
    const int mine = max(0, min(4, m - 4 * lane));   // this lane's slots in the run
    // lane aggregate of its slots: (restarts, counts)
    bool rs = false;
    uint32_t a0 = 0, a1 = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        if (k < mine) {
            const uint32_t c0 = (uint32_t)(w[k] & CH_MAX), c1 = (uint32_t)((w[k] >> 30) & CH_MAX);
            if ((w[k] >> 62) == 2u) { rs = true; a0 = c0; a1 = c1; }
            else { a0 += c0; a1 += c1; }
        }
    }
    // segmented inclusive scan over lanes (an inclusive slot restarts the sum)
    bool irs = rs;
    uint32_t i0 = a0, i1 = a1;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const bool o_rs = __shfl_up_sync(0xffffffffu, irs ? 1 : 0, d) != 0;
        const uint32_t o0 = __shfl_up_sync(0xffffffffu, i0, d), o1 = __shfl_up_sync(0xffffffffu, i1, d);
        if (lane >= d && !irs) {
            i0 += o0;
            i1 += o1;
            irs = o_rs;
        }
    }
    // exclusive: the lanes before this one, seeded by slot f - 1
    bool e_rs = __shfl_up_sync(0xffffffffu, irs ? 1 : 0, 1) != 0;
    uint32_t e0 = __shfl_up_sync(0xffffffffu, i0, 1), e1 = __shfl_up_sync(0xffffffffu, i1, 1);
    if (lane == 0) { e_rs = false; e0 = 0; e1 = 0; }
    uint32_t run0 = e_rs ? e0 : s0 + e0, run1 = e_rs ? e1 : s1 + e1;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        if (k < mine) {
            const uint32_t c0 = (uint32_t)(w[k] & CH_MAX), c1 = (uint32_t)((w[k] >> 30) & CH_MAX);
            if ((w[k] >> 62) == 2u) {
                run0 = c0;
                run1 = c1;
            } else {
                run0 += c0;
                run1 += c1;
                st_relaxed64(slots + f + 4u * (uint32_t)lane + (uint32_t)k, ch_pack(CH_INC, run0, run1));
            }
        }
    }
    // the run's inclusive values before the frontier move: the warp barrier
    // orders every lane's stores before lane 0's release (cumulative)
    __syncwarp();
    if (lane == 0) {
        uint32_t old;
        asm volatile("atom.release.gpu.global.max.u32 %0, [%1], %2;"
                     : "=r"(old) : "l"(frontier), "r"(f + (uint32_t)m) : "memory");
    }
}

}  // namespace ochre
