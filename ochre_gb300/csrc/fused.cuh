// The fused small-raster kernel's launch arguments and the two-level
// look-back that places each raster's tiles and spans in the output, in
// raster order.
#pragma once

#include "common.cuh"
#include "internal.h"

namespace ochre {

// Look-back words: one 64-bit word holding a flag (bits 62-63: 0 none, 1
// aggregate, 2 inclusive) and two 30-bit counts (tiles in bits 0-29, spans
// in bits 30-59).  One naturally aligned 64-bit access reads or writes flag
// and counts together, so a reader trusts a value by its flag alone and no
// fence is needed anywhere.  Counts saturate at 2^30 - 1, above every output
// capacity.
constexpr uint64_t CH_AGG = 1ull << 62, CH_INC = 2ull << 62;
constexpr uint32_t CH_MAX = (1u << 30) - 1u;
__device__ __forceinline__ uint64_t ch_pack(uint64_t flag, uint32_t a0, uint32_t a1) {
    return flag | ((uint64_t)min(a1, CH_MAX) << 30) | min(a0, CH_MAX);
}
__device__ __forceinline__ uint32_t ch_t(uint64_t w) { return (uint32_t)(w & CH_MAX); }
__device__ __forceinline__ uint32_t ch_s(uint64_t w) { return (uint32_t)((w >> 30) & CH_MAX); }
__device__ __forceinline__ uint32_t ch_flag(uint64_t w) { return (uint32_t)(w >> 62); }

// Rasters are grouped in blocks of LB_BLOCK (in ticket order).  Per raster
// an aggregate word (its counts, written once) and an inclusive word (its
// prefix through itself, written when it has placed itself); per block the
// same two words, the block's aggregate written by whichever of its rasters
// publishes last (a per-block counter tells), its inclusive word by its last
// raster when that one has placed itself.  A raster then finds its prefix in
// about two rounds of loads: back through its own block's rasters to the
// nearest placed one (or the block's start), then back through whole blocks
// to the nearest placed block, instead of one round per 128 rasters of the
// ~2,000 in flight.
constexpr uint32_t LB_BLOCK = 128;
constexpr int LB_PER_LANE = LB_BLOCK / 32;

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
    // look-back words: per raster (aggregate, inclusive), per block
    // (aggregate, inclusive, publish counter)
    uint64_t* r_agg;
    uint64_t* r_inc;
    uint64_t* b_agg;
    uint64_t* b_inc;
    uint32_t* b_cnt;
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
    uint8_t* stage_alpha;    // per CTA: F_TMAX tiles of alpha (and of coverage when out_cov)
    float* stage_cov;
};

__device__ __forceinline__ V2 load_pt(const float* p) { return v2(__ldg(p), __ldg(p + 1)); }

// Publishes raster r's counts (one warp); the raster that completes its
// block also publishes the block's aggregate.
__device__ __forceinline__ void lb_publish(const FusedArgs& A, uint32_t r, uint32_t a0, uint32_t a1) {
    const int lane = threadIdx.x & 31;
    const uint32_t b = r / LB_BLOCK, b0 = b * LB_BLOCK;
    const uint32_t bn = min(LB_BLOCK, A.n_rasters - b0);   // rasters in the block
    uint32_t c = 0;
    if (lane == 0) {
        st_relaxed64(A.r_agg + r, ch_pack(CH_AGG, a0, a1));
        c = atomicAdd(A.b_cnt + b, 1u);
    }
    c = __shfl_sync(0xffffffffu, c, 0);
    if (c + 1 != bn) return;
    // every raster of the block has published (or is about to: its store
    // came before its count): sum the block, waiting for a word only while
    // its store is on the way
    long long spins = 0;
    const long long poll_limit = spin_limit(A.err);
    uint32_t s0 = 0, s1 = 0;
    for (;;) {
        uint64_t w[LB_PER_LANE];
        bool missing = false;
#pragma unroll
        for (int k = 0; k < LB_PER_LANE; k++) {
            const uint32_t i = (uint32_t)(k * 32 + lane);
            w[k] = i < bn ? ld_relaxed64(A.r_agg + b0 + i) : CH_AGG;
            missing = missing || ch_flag(w[k]) == 0u;
        }
        if (__any_sync(0xffffffffu, missing)) {
            if (wait_give_up_warp(spins, poll_limit, A.err)) break;
            continue;
        }
        s0 = 0;
        s1 = 0;
#pragma unroll
        for (int k = 0; k < LB_PER_LANE; k++) {
            s0 += ch_t(w[k]);
            s1 += ch_s(w[k]);
        }
        s0 = __reduce_add_sync(0xffffffffu, s0);
        s1 = __reduce_add_sync(0xffffffffu, s1);
        break;
    }
    if (lane == 0) st_relaxed64(A.b_agg + b, ch_pack(CH_AGG, s0, s1));
}

// Raster r's exclusive prefix (tiles, spans), then its inclusive word (and
// its block's, when r ends the block).  One full warp; every wait bounded.
__device__ __forceinline__ void lb_resolve(const FusedArgs& A, uint32_t r, uint32_t a0, uint32_t a1, uint32_t& p0,
                                           uint32_t& p1) {
    const int lane = threadIdx.x & 31;
    const uint32_t b = r / LB_BLOCK, b0 = b * LB_BLOCK;
    long long spins = 0;
    const long long poll_limit = spin_limit(A.err);
    p0 = 0;
    p1 = 0;
    // level 1: the rasters of this block before r, nearest first (q = k * 32 + lane)
    bool done = false;
    for (;;) {
        uint64_t wa[LB_PER_LANE], wi[LB_PER_LANE];
#pragma unroll
        for (int k = 0; k < LB_PER_LANE; k++) {
            const int64_t j = (int64_t)r - 1 - (k * 32 + lane);
            const bool in = j >= (int64_t)b0;
            wi[k] = in ? ld_relaxed64(A.r_inc + j) : 0ull;
            wa[k] = in ? ld_relaxed64(A.r_agg + j) : CH_AGG;
        }
        int q_inc = LB_BLOCK;   // nearest predecessor of the block already placed
#pragma unroll
        for (int k = LB_PER_LANE - 1; k >= 0; k--) {
            const uint32_t m = __ballot_sync(0xffffffffu, ch_flag(wi[k]) == 2u);
            if (m) q_inc = k * 32 + __ffs(m) - 1;
        }
        bool missing = false;
#pragma unroll
        for (int k = 0; k < LB_PER_LANE; k++)
            if (k * 32 + lane < q_inc && ch_flag(wa[k]) == 0u) missing = true;
        if (__any_sync(0xffffffffu, missing)) {
            if (wait_give_up_warp(spins, poll_limit, A.err)) return;
            if (spins > 16) __nanosleep(64);
            continue;
        }
        uint32_t v0 = 0, v1 = 0;
#pragma unroll
        for (int k = 0; k < LB_PER_LANE; k++) {
            const int q = k * 32 + lane;
            if (q < q_inc) {
                v0 += ch_t(wa[k]);
                v1 += ch_s(wa[k]);
            } else if (q == q_inc) {
                v0 += ch_t(wi[k]);
                v1 += ch_s(wi[k]);
            }
        }
        p0 = __reduce_add_sync(0xffffffffu, v0);
        p1 = __reduce_add_sync(0xffffffffu, v1);
        done = q_inc < LB_BLOCK;
        break;
    }
    // level 2: whole blocks before this one, nearest first, 32 per round
    int64_t top = (int64_t)b - 1;
    while (!done && top >= 0) {
        const int64_t j = top - lane;
        uint64_t bi = 0, ba = CH_AGG;
        if (j >= 0) {
            bi = ld_relaxed64(A.b_inc + j);
            ba = ld_relaxed64(A.b_agg + j);
        } else {
            bi = CH_INC;   // before block 0: an inclusive zero
        }
        const uint32_t m = __ballot_sync(0xffffffffu, ch_flag(bi) == 2u);
        const int q_inc = m ? __ffs(m) - 1 : 32;
        if (__any_sync(0xffffffffu, lane < q_inc && ch_flag(ba) == 0u)) {
            if (wait_give_up_warp(spins, poll_limit, A.err)) return;
            if (spins > 16) __nanosleep(64);
            continue;
        }
        uint32_t v0 = 0, v1 = 0;
        if (lane < q_inc) {
            v0 = ch_t(ba);
            v1 = ch_s(ba);
        } else if (lane == q_inc) {
            v0 = ch_t(bi);
            v1 = ch_s(bi);
        }
        p0 += __reduce_add_sync(0xffffffffu, v0);
        p1 += __reduce_add_sync(0xffffffffu, v1);
        if (m) break;
        top -= 32;
    }
    p0 = min(p0, CH_MAX);
    p1 = min(p1, CH_MAX);
    if (lane == 0) {
        const uint64_t w = ch_pack(CH_INC, p0 + a0, p1 + a1);
        st_relaxed64(A.r_inc + r, w);
        if (r + 1 == A.n_rasters || (r + 1) % LB_BLOCK == 0) st_relaxed64(A.b_inc + b, w);
    }
}

}  // namespace ochre
