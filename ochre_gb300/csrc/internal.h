// Host-side internals shared by the translation units of libochre_gpu.so.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <vector>

#include "../../include/ochre_gpu.h"

namespace ochre {

// Bump region that DevBufs in arena mode carve from instead of cudaMalloc.
struct Arena {
    char* base = nullptr;
    size_t size = 0;
    size_t used = 0;
    bool overflow = false;   // a request did not fit
};

// Grow-only device buffer.  With `arena` set it never calls cudaMalloc: it
// carves from the arena; with `fixed` set it only accepts requests that fit
// the preset storage.
struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
    Arena* arena = nullptr;
    bool fixed = false;
    cudaError_t ensure(size_t bytes);
    void release();
    template <class T> T* as() const { return static_cast<T*>(p); }
};

// Grow-only pinned host buffer.
struct HostBuf {
    void* p = nullptr;
    size_t cap = 0;
    void* dev = nullptr;   // device view of the memory (mapped allocations), or nullptr
    cudaError_t ensure(size_t bytes);
    // like ensure(), but the memory is mapped into the device address space
    // (kernels can write results into it directly)
    cudaError_t ensure_mapped(size_t bytes);
    void release();
    template <class T> T* as() const { return static_cast<T*>(p); }
};

// Device-resident scalars of one run (read back with one copy).
struct DevScalars {
    uint32_t err;          // ERR_* bits
    uint32_t ticket;       // ticket counter for ticketed kernels
    uint32_t n_floats;     // floats the verbs consume (command scan total .foff)
    uint32_t cmd_mv_tot;   // unused totals of the command scan
    uint32_t cmd_ep_tot;
    uint32_t n_lines;      // total lines
    uint32_t n_line_ent;   // entries produced by lines
    uint32_t n_entries;    // all sort entries: n_line_ent + n_empty
    uint64_t keyspace;     // total key space (raster scan .ks)
    uint32_t n_empty;      // rasters without increments (raster scan .ne)
    uint32_t pad1;
    uint32_t n_tiles;      // tile-head scan total .heads   }
    uint32_t n_bins;       // tile-head scan total .bins    } (HeadScan layout)
    int32_t head_wind;     // sum of all crossing signs     }
    uint32_t pad2;         //                               }
    uint32_t n_spans;
    uint32_t sort_ticket;
    uint32_t fused_fallback;  // fused path: some raster did not fit
    uint32_t fused_tiles;     // fused path totals
    uint32_t fused_spans;
    uint32_t n_rows;          // tile rows (raster, tile_y) of the general chain
    uint32_t spin_log2;       // poll limit of the run's bounded waits, log2 (0: SPIN_LIMIT)
    uint32_t pad3;
    uint32_t line_ent_total;  // chain: sort entries the lines produce   } (line scan
    uint32_t n_incs;          // chain: pixel-cell increments of the lines } pair total)
    uint64_t inc_total;       // the same increment count summed in 64 bits (the pair
                              // total wraps above 2^32; this one says when it did)
    uint32_t walk_ticket[2];  // long-line pools handed out in the count and emit walks
    uint32_t n_long;          // lines queued for the long-line walkers (flatten)
    uint32_t pad4;
    uint32_t line_ticket;     // line windows handed out in the count walk
    uint32_t pad5;
};
// The waits find spin_log2 from the error word's address (common.cuh).
static_assert(offsetof(DevScalars, spin_log2) - offsetof(DevScalars, err) == 4 * 22,
              "spin_log2 must sit SPIN_LOG2_WORD words after err");

// Canvas sides of the differentiable entries: beyond the i16 tile
// coordinate range there is no pixel a tile can reach.
constexpr uint32_t MAX_CANVAS = 32768;

// The buffers of one differentiable step captured into a CUDA graph
// (ochre_graph_create_diff): coverage render, L2 loss, backward.
struct DiffStep {
    uint32_t w, h;
    const float* target;
    float* cov;
    float* dl_dcov;
    double* loss;
    float* dl_dpts;
    float* dl_dxf;
};

// Capacities of a launch chain captured into a CUDA graph.  Every buffer is
// sized from them once; the counts stay on the device, each kernel reads its
// count there and its grid covers the capacity.  A check kernel at every
// sizing point flags a count above its capacity (ERR_CAPACITY) and zeroes it,
// so that no later kernel works past a buffer.
struct GraphPlan {
    bool fused;          // the batch is one fused launch (else the general chain)
    uint32_t lines;      // general chain: lines, sort entries, tiles
    uint32_t entries;
    uint32_t tiles;      // (fused: output tiles and spans)
    uint32_t key_bits;   // sort key bits; keys are 64-bit above 32
    uint32_t incs;       // general chain: stored pixel-cell increments
    uint32_t rows;       // tile rows of the planning run (coverage form and grid)
    // Stroked fills (planned on the general chain): polyline commands and
    // floats, output commands and floats of the stroke stage.  Its units
    // never outnumber the polyline commands.  The output is padded to
    // stroke_cmds with Close commands (no lines) on the batch's last fill,
    // so the chain after it runs on fixed command and float counts.
    bool stroke;
    uint32_t stroke_poly, stroke_poly_floats;
    uint32_t stroke_cmds, stroke_floats;
    // a differentiable step: after the chain (signed coverage), its render,
    // loss and backward, their counts on the device
    const DiffStep* diff;
};

// Entry value tag for tile-row crossings: 1 | raster (23 bits) | sign byte.
constexpr uint32_t CROSS_TAG = 0x80000000u;
constexpr uint32_t MAX_RASTERS = 1u << 23;
constexpr uint64_t MAX_COUNT = (1ull << 30) - 1;   // lines, entries, tiles
constexpr uint64_t MAX_INCS = 0xffffffffull;        // stored increments (32-bit offsets)

// A bin: a run of consecutive pixel cells of one line's walk that share one
// tile (16 bytes).  Its cells' increments (area, height) were stored by the
// walk at inc .. inc + n - 1; the cells themselves follow from the first cell
// and the walk's steps (bit k of `steps`: the step from cell k to cell k + 1
// moved in x, else in y; `dirs` bit 0 / 1: the x / y step is -1).
struct alignas(16) BinRec {
    uint32_t inc;        // first increment of the run
    uint32_t raster;
    int16_t x, y;        // first cell of the run (i16 cell coordinates)
    uint16_t steps;
    uint8_t n;           // cells in the run (0 for the empty-raster tile)
    uint8_t dirs;
};
static_assert(sizeof(BinRec) == 16, "BinRec must be 16 bytes");
constexpr uint32_t BIN_MAX_CELLS = 16;   // a run longer than this is split (it never is: 15 at most)

// Look-back state of one block of tiles (block-form coverage kernel): the row
// sums (8 pixel rows) of the block's last row segment.
struct TileBlockState {
    uint32_t flag;       // 0: none, 1: aggregate (block continues one row), 2: inclusive
    uint32_t pad;
    float agg[8];
    float inc[8];
};

struct TileInfo {
    int32_t raster;
    int32_t tx, ty;
    uint32_t head;       // first bin entry of the tile in the sorted entries
    uint32_t nbins;
    int32_t wind;        // tile-row crossing winding at this tile (inclusive, per raster)
    uint32_t row_head;   // 1 if the tile starts its (raster, tile_y) row
    uint32_t pad;
};


}  // namespace ochre

struct ochre_gpu_ctx {
    int device = 0;
    uint32_t flags = 0;
    cudaStream_t own_stream = nullptr;

    // device copies of a host batch (ochre_gpu_rasterize)
    ochre::DevBuf in_verbs, in_pts, in_fill_off, in_fill_xf, in_fill_flags, in_raster_off;
    // per command
    ochre::DevBuf cmd_foff, cmd_mv, cmd_ep, cmd_line_off;
    // per line (line_inc_off: first stored increment of the line's walk)
    ochre::DevBuf lines, line_raster, line_ent_off, line_inc_off;
    ochre::DevBuf long_lines;   // indices of the lines walked by the long-line walkers
    // stored pixel-cell increments (area, height) of every walk, line by line
    ochre::DevBuf incs;
    // per raster
    ochre::DevBuf raster_bbox, raster_keybase, raster_empty;
    // per raster: sum of its tile-row crossing signs, and the sum over earlier rasters
    ochre::DevBuf raster_wsum, raster_wbase;
    // sort entries
    ochre::DevBuf keys, vals, keys_alt, vals_alt, bins;
    ochre::DevBuf sort_hist, sort_lookback;
    // tiles
    ochre::DevBuf tile_head, tile_info, tile_row_start, tile_state, span_flag, span_val;   // tile_state: TileBlockState
    // per tile: bins and crossing-sign sum of all entries before its head
    ochre::DevBuf tile_head_bins, tile_head_wind;
    // scan workspace
    ochre::DevBuf scan_status;
    ochre::DevBuf scalars;   // DevScalars
    ochre::DevBuf fused_chain;   // fused path: the rasters' and blocks' look-back words
    ochre::DevBuf fused_stage;   // fused path: per-CTA staged alpha (and coverage) of its raster
    uint32_t fused_max_ctas = 0; // fused path: at most this many persistent CTAs (0: no limit)
    uint32_t fused_tile_cap = 0; // fused path: output capacity guess (tiles)
    // The last batch of the device entry that did not fit the fused kernel
    // (its arrays and counts): while the same batch comes back, it goes to
    // the general chain without a fused attempt.
    ochre_batch fused_miss{};
    bool fused_miss_valid = false;
    // device outputs
    ochre::DevBuf out_tile_xy, out_tile_alpha, out_tile_cov, out_span_xy, out_span_w, out_span_tile,
        out_raster_tile_off, out_raster_span_off;
    // pinned host
    ochre::HostBuf h_scalars;
    // h_scalars as seen from the device when it is mapped host memory: the
    // read-back is then a kernel store, not a copy queued behind bulk copies
    void* h_scalars_dev = nullptr;
    ochre::HostBuf h_tile_xy, h_tile_alpha, h_tile_cov, h_span_xy, h_span_w, h_span_tile, h_raster_tile_off,
        h_raster_span_off;

    ochre_stats stats{};
    int keys64 = 0;          // last run used 64-bit keys

    bool cov_signed = false;   // tile_cov holds accum + area (signed) instead of |accum + area|
    // differentiable path scratch
    ochre::DevBuf grad_g, grad_gs, grad_left, grad_line, grad_pts;
    // Bumped by every call that rewrites the chain's buffers (run_device,
    // compositing).  The chain structure left by ochre_gpu_render_coverage
    // (lines, per-command line offsets, tiles with signed coverage) stays
    // valid while it is unchanged, and the backward of the same batch reuses it.
    uint64_t epoch = 0;
    struct SavedForward {
        bool valid;
        uint64_t epoch;
        ochre_batch in;
        ochre_result res;
        uint32_t n_lines;
    } saved{};
    // stroke stage: input command scan, polyline, units, output batch
    ochre::DevBuf sk_cmd_foff, sk_cmd_mv, sk_cmd_ep, sk_poly_off, sk_poly_foff, sk_pverbs, sk_ppts, sk_pfoff,
        sk_pfill_off, sk_first_close, sk_unit_start, sk_out_off, sk_out_foff, sk_unit_fill, sk_overbs, sk_opts,
        sk_ofill_off, sk_oflags, in_fill_width;
    // the last eager stroke stage's counts (polyline commands and floats,
    // output commands and floats): a CUDA graph's plan sizes from them
    uint32_t stroke_counts[4] = {0, 0, 0, 0};

    // Test hooks (ochre_gpu_set_tunable "test_*"), used by the next run only:
    // the poll limit of its bounded waits (log2; 0: the default), and, on the
    // fused path, a command scan whose first tile is never taken, so that
    // the waits of the tiles after it cannot finish.
    uint32_t test_spin_log2 = 0;
    uint32_t test_skip_first_ticket = 0;

    // Launch-shape tunables (ochre_gpu_set_tunable; chosen by the autotuner).
    int tune_fused_threads = 64;
    int tune_fused_chunk = 16;
    int tune_chain_tiles_per_warp = 8;
    int tune_chain_coverage_form = 0;   // 0: by row count, 1: block form, 2: row form
    int tune_sort_digit_bits = 8;       // radix sort digit width: 8 or 11
    int tune_chain_long_cells = 192;    // lines of more (estimated) cells go to the long-line walkers; 0: none
    int tune_chain_walk_refill = 8;     // idle lanes of a long-line warp that trigger a refill (1..32)

    // Host-batch entry: a large point array is copied on copy_stream while
    // the first stages run; pts_pending until a stage that reads points has
    // made the run's stream wait for ev_pts (wait_inputs).
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_prior = nullptr, ev_pts = nullptr;
    bool pts_pending = false;
    // The chain's long-line walkers run on walk_stream beside the per-line
    // walks (forked from and joined to the run's stream by the two events),
    // or on the run's stream itself when no_side_stream is set.
    cudaStream_t walk_stream = nullptr;
    cudaEvent_t ev_walk_fork = nullptr, ev_walk_join = nullptr;
    bool no_side_stream = false;

    // Set while the chain is planned for (and captured into) a CUDA graph:
    // stages size buffers from it and never read counts back to the host.
    const ochre::GraphPlan* plan = nullptr;


    // Tracing: every kernel launch of a run is counted; with OCHRE_CTX_PROFILE
    // each one is also bracketed by a pair of CUDA events on its stream.
    struct Prof {
        const char* name;
        cudaEvent_t a, b;
    };
    std::vector<Prof> prof;
    uint32_t prof_used = 0;
    uint32_t launches = 0;
    std::vector<ochre_kernel_time> timings;
};

namespace ochre {

// Stage launchers (each returns an ochre_status).
int stage_flatten(ochre_gpu_ctx* ctx, const ochre_batch* in, cudaStream_t s, uint32_t* n_lines);
int stage_bin(ochre_gpu_ctx* ctx, const ochre_batch* in, uint32_t n_lines, cudaStream_t s, uint64_t* n_entries,
              uint32_t* key_bits);
int stage_sort(ochre_gpu_ctx* ctx, uint64_t n_entries, uint32_t key_bits, cudaStream_t s, uint32_t* passes);
int stage_tiles(ochre_gpu_ctx* ctx, const ochre_batch* in, uint64_t n_entries, cudaStream_t s, uint32_t* n_tiles,
                uint32_t* n_spans);
// Rewrites stroked fills into plain fills (stroke.cu); *out views device memory.
int stage_stroke(ochre_gpu_ctx* ctx, const ochre_batch* in, cudaStream_t s, ochre_batch* out);
// After a planned chain with signed coverage: the coverage render, the L2
// loss and the backward of one differentiable step, every count read on the
// device (CUDA graphs; grad.cu).
int stage_diff_tail(ochre_gpu_ctx* ctx, const ochre_batch* in, const DiffStep& d, cudaStream_t s);
int stage_fused(ochre_gpu_ctx* ctx, const ochre_batch* in, cudaStream_t s, bool* handled, uint32_t* n_tiles,
                uint32_t* n_spans);


// The same arrays and counts.
inline bool same_batch(const ochre_batch& a, const ochre_batch& b) {
    return a.verbs == b.verbs && a.n_cmds == b.n_cmds && a.pts == b.pts && a.n_floats == b.n_floats &&
           a.fill_cmd_off == b.fill_cmd_off && a.fill_xf == b.fill_xf && a.fill_flags == b.fill_flags &&
           a.n_fills == b.n_fills && a.raster_fill_off == b.raster_fill_off && a.n_rasters == b.n_rasters &&
           a.fill_width == b.fill_width;
}

// The whole chain for one batch (device pointers), results in ctx buffers.
// With remember_miss, a batch that did not fit the fused kernel is noted in
// the context, and the same batch then skips the fused attempt.
int run_device(ochre_gpu_ctx* ctx, const ochre_batch* in, ochre_result* out, cudaStream_t s,
               bool remember_miss = false);

// Graph replays: device checks of counts against the plan (api.cu).  The
// entry check sets n_entries = line_ent_total + n_empty and zeroes it, and the
// line count, when it, the key space or the stored increments exceed the
// plan; the other zeroes *count above cap.  Both flag ERR_CAPACITY.
cudaError_t launch_plan_entries(ochre_gpu_ctx* ctx, uint32_t cap, uint32_t key_bits, uint32_t inc_cap,
                                cudaStream_t s);
cudaError_t launch_plan_cap(ochre_gpu_ctx* ctx, uint32_t* count, uint32_t cap, cudaStream_t s);

// Makes stream s wait for the batch's points if they are still being copied
// (host-batch entry); every stage calls it before its first read of points.
void wait_inputs(ochre_gpu_ctx* ctx, cudaStream_t s);

// Zeroes the device scalars of a run (and applies the poll-limit test hook).
cudaError_t reset_scalars(ochre_gpu_ctx* ctx, cudaStream_t s);
// Read the device scalars into ctx->h_scalars (synchronises the stream).
int read_scalars(ochre_gpu_ctx* ctx, cudaStream_t s);
// The same copy, enqueued only.
int copy_scalars_async(ochre_gpu_ctx* ctx, cudaStream_t s);
// Every device buffer of a context (release on destroy; a graph capture
// checks that none of them moved).
std::vector<DevBuf*> device_buffers(ochre_gpu_ctx* ctx);
inline DevScalars* dev_scalars(ochre_gpu_ctx* ctx) { return ctx->scalars.as<DevScalars>(); }
inline DevScalars* host_scalars(ochre_gpu_ctx* ctx) { return ctx->h_scalars.as<DevScalars>(); }
int check_device_error(ochre_gpu_ctx* ctx);
void prof_begin(ochre_gpu_ctx* ctx, const char* name, cudaStream_t s);
void prof_end(ochre_gpu_ctx* ctx, cudaStream_t s);
// Converts the event pairs recorded since the last reset into ctx->timings.
void collect_timings(ochre_gpu_ctx* ctx, cudaStream_t s);

// Counts (and, when profiling, times) one launch site: the statements in
// `...` must enqueue exactly the work to attribute to `name`.
#define OCHRE_LAUNCH(ctx, name, s, ...)      \
    do {                                      \
        ::ochre::prof_begin(ctx, name, s);    \
        __VA_ARGS__;                          \
        ::ochre::prof_end(ctx, s);            \
    } while (0)

#define OCHRE_CUDA_TRY(expr)                                   \
    do {                                                       \
        cudaError_t e_ = (expr);                               \
        if (e_ != cudaSuccess) {                               \
            return e_ == cudaErrorMemoryAllocation ? OCHRE_E_NOMEM : OCHRE_E_CUDA; \
        }                                                      \
    } while (0)

}  // namespace ochre
