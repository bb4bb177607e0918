// The fused small-raster kernel's launch arguments.
#pragma once

#include "common.cuh"
#include "internal.h"

namespace ochre {

// Output chunks: each CTA takes the output space of its rasters from a
// chunk of this many tiles (spans) that it claims from a device-wide cursor.
constexpr uint32_t U_CHUNK_TILES = 512;
constexpr uint32_t U_CHUNK_SPANS = 256;

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
    uint32_t* ticket;
    uint32_t* fallback;      // any raster did not fit
    uint32_t* err;
    // unordered output: chunk cursors (tiles, spans), capacities, arrays
    uint32_t* u_cursor;
    uint32_t u_tile_cap, u_span_cap;
    uint32_t* u_xy;
    uint8_t* u_alpha;
    float* u_cov;            // or nullptr
    uint32_t* u_span_xy;
    uint16_t* u_span_w;
    uint16_t* u_span_t;      // the tile a span follows, as an index within its raster
    // per raster: tile and span counts, first unordered tile and span
    uint32_t* r_count;
    uint32_t* r_start;
};

__device__ __forceinline__ V2 load_pt(const float* p) { return v2(__ldg(p), __ldg(p + 1)); }

}  // namespace ochre
