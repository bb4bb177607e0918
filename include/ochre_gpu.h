/*
 * ochre_gpu.h — C ABI of the GB300 (sm_103a) implementation of ochre's
 * path-rasterization hot path (glowcoil/ochre 0.2.0).
 *
 * The reference API is Rust (src/rasterizer.rs):
 *     Rasterizer::new() -> Rasterizer                       rasterizer.rs:50
 *     Rasterizer::move_to(&mut self, Vec2)                  rasterizer.rs:61
 *     Rasterizer::line_to(&mut self, Vec2)                  rasterizer.rs:72
 *     Rasterizer::command(&mut self, PathCmd)               rasterizer.rs:145
 *     Rasterizer::fill(&mut self, &[PathCmd], Transform)    rasterizer.rs:161
 *     Rasterizer::finish<B: TileBuilder>(self, &mut B)      rasterizer.rs:180
 *     trait TileBuilder { tile(x, y, [u8; 64]); span(x, y, width) }  rasterizer.rs:12-22
 * Rust enums and traits cannot cross a C ABI, so:
 *   - PathCmd (path.rs:5-12) becomes a verb byte plus a float stream
 *     (see ochre_verb and the table below);
 *   - Transform (geom.rs:204-207) becomes 6 floats m0 m1 m2 m3 ox oy, the
 *     row-major Mat2x2 followed by the offset;
 *   - TileBuilder becomes two callbacks plus a user pointer;
 *   - errors, which the Rust API cannot report (it is infallible), are
 *     returned as an int status (ochre_status).
 *
 * Every function returns OCHRE_OK (0) or an ochre_status code.  A context is
 * bound to one CUDA device and one stream; use one context per host thread.
 * Output buffers returned in ochre_result are owned by the context and stay
 * valid until the next rasterize/finish call on it or ochre_gpu_destroy.
 */
#ifndef OCHRE_GPU_H
#define OCHRE_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OCHRE_TILE_SIZE 8      /* TILE_SIZE, rasterizer.rs:4 (not configurable) */
#define OCHRE_TOLERANCE 0.1f   /* TOLERANCE, rasterizer.rs:6 (device pixels) */

typedef enum ochre_status {
    OCHRE_OK = 0,
    OCHRE_E_INVALID = 1,   /* malformed input (bad verb, short point stream, bad offsets, non-finite point) */
    OCHRE_E_CAPACITY = 2,  /* a size limit of this implementation was exceeded (counts >= 2^30) */
    OCHRE_E_CUDA = 3,      /* a CUDA runtime call failed */
    OCHRE_E_TIMEOUT = 4,   /* a bounded device-side wait gave up (results are not valid) */
    OCHRE_E_NOMEM = 5,     /* device or host allocation failed */
    OCHRE_E_LIMIT = 6      /* a per-segment/per-line iteration cap was hit: the reference would not terminate */
} ochre_status;

/* PathCmd discriminants (path.rs:5-12).  Floats consumed per verb:
 *   MOVE x y | LINE x y | QUADRATIC cx cy x y | CUBIC c1x c1y c2x c2y x y |
 *   CONIC cx cy x y w | CLOSE (none) */
typedef enum ochre_verb {
    OCHRE_MOVE = 0,
    OCHRE_LINE = 1,
    OCHRE_QUADRATIC = 2,
    OCHRE_CUBIC = 3,
    OCHRE_CONIC = 4,
    OCHRE_CLOSE = 5
} ochre_verb;

/* fill_flags bit: the fill's commands are already in device space and are
 * not transformed (Rasterizer::command/move_to/line_to, rasterizer.rs:61-157). */
#define OCHRE_FILL_RAW 1u
/* fill_flags bit: the fill is stroked (Rasterizer::stroke, rasterizer.rs:169-171)
 * with width fill_width[f]: flattened in its own space, offset by width / 2 on
 * both sides with miter joins and butt caps (path.rs:113-274), then filled
 * with its transform. */
#define OCHRE_FILL_STROKE 2u

/* A batch of independent rasterizers.  Raster r owns fills
 * [raster_fill_off[r], raster_fill_off[r+1]) (one fill per raster when
 * raster_fill_off is NULL); fill f owns commands
 * [fill_cmd_off[f], fill_cmd_off[f+1]) and transform fill_xf[6f .. 6f+5].
 * Equivalent to, per raster: Rasterizer::new(); fill(cmds_f, xf_f) for each
 * of its fills in order; finish(builder).  Pointers are host pointers for
 * ochre_gpu_rasterize and device pointers for ochre_gpu_rasterize_device. */
typedef struct ochre_batch {
    const uint8_t *verbs;
    uint64_t n_cmds;
    const float *pts;
    uint64_t n_floats;
    const uint32_t *fill_cmd_off;    /* n_fills + 1 */
    const float *fill_xf;            /* 6 * n_fills */
    const uint8_t *fill_flags;       /* n_fills, or NULL (all transformed) */
    uint32_t n_fills;
    const uint32_t *raster_fill_off; /* n_rasters + 1, or NULL */
    uint32_t n_rasters;
    const float *fill_width;         /* n_fills stroke widths, or NULL (no stroked fills) */
} ochre_batch;

/* Output, in TileBuilder callback order per raster (rasterizer.rs:241, 263):
 * tiles ascending by (y, x); a span follows the tile with index span_tile. */
typedef struct ochre_result {
    uint32_t n_tiles;
    uint32_t n_spans;
    const int16_t *tile_xy;          /* 2 per tile: x, y in pixels (multiples of 8) */
    const uint8_t *tile_alpha;       /* 64 per tile, row-major 8x8 alpha mask */
    const float *tile_cov;           /* 64 per tile: |accum + area| before quantisation, or NULL */
    const int16_t *span_xy;          /* 2 per span */
    const uint16_t *span_width;      /* 1 per span, pixels; height is always 8 */
    const uint32_t *span_tile;       /* 1 per span: index of the tile it follows */
    const uint32_t *raster_tile_off; /* n_rasters + 1 */
    const uint32_t *raster_span_off; /* n_rasters + 1 */
} ochre_result;

/* Intermediate counts of the last run (for tests and profiling). */
typedef struct ochre_stats {
    uint64_t n_lines;      /* flattened line segments, including implicit closes */
    uint64_t n_entries;    /* sort entries: tile bins + tile-row crossings */
    uint64_t n_tiles;
    uint64_t n_spans;
    uint32_t key_bits;     /* significant bits of the tile sort key */
    uint32_t sort_passes;
    uint32_t n_launches;   /* kernels launched by the run */
    uint32_t pad;
    uint64_t n_bins;       /* sort entries that are tile bins (runs of cells in one tile) */
    uint32_t fused;        /* 1: the fused small-raster kernel handled the batch, 0: the general chain */
    uint32_t n_incs;       /* general chain: pixel-cell increments the lines stored (at most 2^32 - 1) */
} ochre_stats;

/* Device time of one kernel launch of the last run (OCHRE_CTX_PROFILE). */
typedef struct ochre_kernel_time {
    const char *name;      /* static string naming the kernel */
    float ms;
} ochre_kernel_time;

typedef struct ochre_gpu_ctx ochre_gpu_ctx;

#define OCHRE_CTX_WANT_COV 1u   /* also produce tile_cov */
#define OCHRE_CTX_PROFILE 2u    /* time every kernel launch with CUDA events */
#define OCHRE_CTX_CHAIN_ONLY 4u /* always use the general kernel chain (no fused small-raster path) */

/* Create a context on `device` (CUDA ordinal).  flags: OCHRE_CTX_*. */
int ochre_gpu_create(ochre_gpu_ctx **out, int device, uint32_t flags);
void ochre_gpu_destroy(ochre_gpu_ctx *ctx);
int ochre_gpu_set_flags(ochre_gpu_ctx *ctx, uint32_t flags);

/* Batched fill+finish of many independent rasterizers (device pointers in
 * `in`, results left in device memory owned by ctx).  `stream` is a
 * cudaStream_t, or NULL for the context's own stream.  Replaces, per raster,
 * Rasterizer::new/fill/finish (rasterizer.rs:50, 161-165, 180-268).
 * A batch with a raster beyond the fused kernel's limits runs on the general
 * chain; the context remembers the last such batch (its arrays and counts)
 * and runs it on the chain without a fused attempt while the same arrays and
 * counts come back.  Both forms give the same tiles and spans (alpha within
 * 1 LSB). */
int ochre_gpu_rasterize_device(ochre_gpu_ctx *ctx, const ochre_batch *in, ochre_result *out, void *stream);

/* Same with host buffers: copies the batch to the device, rasterizes and
 * copies the result back into pinned host buffers owned by ctx.  Checks the
 * batch with ochre_validate_batch first. */
int ochre_gpu_rasterize(ochre_gpu_ctx *ctx, const ochre_batch *in, ochre_result *out);

/* Structural check of a batch in host memory, without a GPU: pointers present
 * for nonzero counts, counts within the limits (OCHRE_E_CAPACITY), and
 * fill_cmd_off / raster_fill_off starting at 0, non-decreasing and ending at
 * n_cmds / n_fills (else OCHRE_E_INVALID).  Point values and verb codes are
 * checked by the kernels that read them. */
int ochre_validate_batch(const ochre_batch *in);

int ochre_gpu_last_stats(const ochre_gpu_ctx *ctx, ochre_stats *out);

/* Per-launch device times of the last run (needs OCHRE_CTX_PROFILE): writes
 * up to `cap` entries and the total count to *n. */
int ochre_gpu_last_timings(const ochre_gpu_ctx *ctx, ochre_kernel_time *out, uint32_t cap, uint32_t *n);

/* ---- CUDA-graph execution -------------------------------------------------
 * The whole fill -> finish launch chain of ochre_gpu_rasterize_device,
 * captured once into a CUDA graph and replayed by one graph launch per call
 * (no host read-backs between stages, one synchronisation per call).  For
 * batches rasterized over and over with the same structure: animation
 * frames (new transforms), optimisation loops (new points).  No counterpart
 * in the reference, which rasterizes one path per call on the CPU.
 *   - `in` holds device pointers; they and every count in `in` are fixed for
 *     the graph's life.  The values behind them may change between launches
 *     (points, transforms, verbs of the same float layout, stroke widths).
 *   - Stroked fills (fill_width) are captured too: the stroke stage runs in
 *     the graph with its counts on the device, and its output is padded
 *     with Close commands to the planned size; such a graph always runs the
 *     general chain (results are identical to the fused kernel's).
 *   - Creation runs the batch once eagerly and plans every internal buffer at
 *     `headroom` (1 to 16) times its count.  A launch whose counts outgrow the
 *     plan (or, for a batch planned on the fused kernel, a raster that no
 *     longer fits it) re-plans from an eager run and replays once.
 *   - The graph owns its buffers (a private context created on ctx's device
 *     with ctx's flags and tunables).  Results of a launch are device
 *     pointers into them, valid until the next launch or destroy.
 *   - `stream` is a cudaStream_t, or NULL for the graph's own stream; the
 *     launch returns when the replay has finished. */
typedef struct ochre_graph ochre_graph;
int ochre_graph_create(ochre_gpu_ctx *ctx, const ochre_batch *in, float headroom, ochre_graph **out);
int ochre_graph_launch(ochre_graph *g, ochre_result *out, void *stream);
/* Counts of the last launch (n_launches = kernels in the graph). */
int ochre_graph_last_stats(const ochre_graph *g, ochre_stats *out);
/* Kernels captured, re-plans so far, and 1 when the plan is the fused kernel. */
int ochre_graph_info(const ochre_graph *g, uint32_t *kernels, uint32_t *replans, uint32_t *fused);
void ochre_graph_destroy(ochre_graph *g);
/* One whole differentiable step captured the same way (no counterpart in the
 * reference): the forward with signed coverage, ochre_gpu_render_coverage
 * into `cov`, ochre_gpu_l2_loss against `target` (loss and dl_dcov) and
 * ochre_gpu_fill_backward into dl_dpts / dl_dxf, on the buffers given here
 * (device pointers, fixed for the graph's life; layouts as in the
 * differentiable entries below).  ochre_graph_launch replays the step (its
 * result is the forward's tiles with signed coverage); the values behind the
 * batch and the target may change between launches.  Stroked fills are not
 * differentiated (OCHRE_E_INVALID). */
int ochre_graph_create_diff(ochre_gpu_ctx *ctx, const ochre_batch *in, uint32_t w, uint32_t h, const float *target,
                            float *cov, float *dl_dcov, double *loss, float *dl_dpts, float *dl_dxf, float headroom,
                            ochre_graph **out);

/* ---- Differentiable fill -------------------------------------------------
 * Extends the reference's forward model (rasterizer.rs:180-268) with dense
 * coverage images and a hand-written backward pass.  Raster r renders into a
 * w x h canvas (origin (0,0)) at offset r*w*h of the image buffers; pixel
 * coverage is min(|accum + area|, 1) inside boundary tiles (the value the
 * reference quantises, rasterizer.rs:235), 1 inside spans, 0 elsewhere.
 * All pointers are device pointers; `stream` is a cudaStream_t or NULL. */
int ochre_gpu_render_coverage(ochre_gpu_ctx *ctx, const ochre_batch *in, uint32_t w, uint32_t h, float *cov,
                              void *stream);

/* loss = sum (cov - target)^2 (written as one double), dl_dcov = 2 (cov - target)
 * (may be NULL). */
int ochre_gpu_l2_loss(ochre_gpu_ctx *ctx, const float *cov, const float *target, uint64_t n, double *loss,
                      float *dl_dcov, void *stream);

/* Backward of ochre_gpu_render_coverage: from dL/d(coverage) (same layout),
 * writes dL/d(pts) (one value per input float, in the input (pre-transform)
 * space; a conic weight gets its own derivative) and dL/d(transform) (6 per fill: m0 m1 m2 m3
 * ox oy).  When the context's last call that ran the chain was
 * ochre_gpu_render_coverage of the same batch (the same arrays and counts),
 * the tile and line lists that call left are reused; the arrays must then
 * still hold the values they had in that call.  Otherwise (any rasterization
 * or compositing on the context in between, or another batch) they are
 * recomputed.  Segment counts, visited cells and tiles are held fixed (they
 * are piecewise constant in the inputs). */
int ochre_gpu_fill_backward(ochre_gpu_ctx *ctx, const ochre_batch *in, uint32_t w, uint32_t h,
                            const float *dl_dcov, float *dl_dpts, float *dl_dxf, void *stream);

/* ---- Rasterization without device allocation --------------------------
 * No counterpart in the reference (which allocates freely on the CPU).
 * For callers that may not allocate GPU memory once they are running:
 * hosts that reserve all device memory at start-up (cudaMalloc/cudaFree
 * synchronise the device and can stall a frame), or that run next to another
 * allocator owning the device memory.  Same chain and results as
 * ochre_gpu_rasterize_device (device pointers in `in`), but every
 * intermediate buffer comes from one static device array of
 * OCHRE_NOALLOC_SCRATCH_BYTES held by each GPU that loads the library, and
 * results go to the caller's buffers.  Calls no cudaMalloc/cudaFree.
 *   - Returns OCHRE_E_CAPACITY when the batch's intermediates do not fit the
 *     array (roughly up to ~100k lines / ~150k tiles) or a caller buffer is
 *     too small; span_capacity must be >= the tile count (a span follows at
 *     most one tile), raster offsets need n_rasters + 1 entries.
 *   - Every call looks up the array's device address (cudaGetSymbolAddress)
 *     with the calling device current; the first call on a device also loads
 *     the library's device code there, which places the array.  Make that
 *     first call before any stream capture.
 *   - All calls share the array: calls that overlap on the GPU race (host
 *     threads are serialised; a call that fails waits for the work it queued
 *     before returning).  `stream` is a cudaStream_t (NULL: default). */
#define OCHRE_NOALLOC_SCRATCH_BYTES (32u << 20)

typedef struct ochre_output_buffers {  /* device pointers; tile_alpha 8-byte aligned, tile_xy,
                                          span_xy and span_tile 4-byte aligned (else OCHRE_E_INVALID) */
    int16_t *tile_xy;           /* 2 * tile_capacity */
    uint8_t *tile_alpha;        /* 64 * tile_capacity */
    uint32_t tile_capacity;
    int16_t *span_xy;           /* 2 * span_capacity */
    uint16_t *span_width;       /* span_capacity */
    uint32_t *span_tile;        /* span_capacity */
    uint32_t span_capacity;
    uint32_t *raster_tile_off;  /* n_rasters + 1 */
    uint32_t *raster_span_off;  /* n_rasters + 1 */
    uint32_t n_tiles;           /* written on success */
    uint32_t n_spans;           /* written on success */
} ochre_output_buffers;

int ochre_gpu_rasterize_noalloc(const ochre_batch *in, ochre_output_buffers *out, void *stream);

/* Launch-shape tunables, chosen per GPU by the project's autotuner
 * (ochre_gb300/autotune.py) and applied per context:
 *   "fused_threads"          threads per raster in the fused kernel: 64 | 96 | 128
 *   "fused_chunk"            tiles accumulated per pass in the fused kernel: 8 | 16 | 32
 *                            (shapes built: 64x8, 64x16, 64x32, 96x8, 96x16, 128x16, 128x32)
 *   "chain_tiles_per_warp"   tiles per warp in the chain's coverage kernel: 4 | 8 | 16
 *   "chain_coverage_form"    coverage kernel form: 0 by tile-row count (default), 1 one warp
 *                            per block of tiles with a look-back carry, 2 one warp per tile row
 *   "sort_digit_bits"        radix digit width of the chain's sort: 8 (default) | 11
 *   "chain_long_cells"       lines of more estimated cells than this are walked by the
 *                            refilling long-line walkers beside the per-line kernels:
 *                            0 (none) | 16 .. 65535 (default 192)
 *   "chain_walk_refill"      idle lanes a long-line warp waits for before it refills: 1 .. 32
 *                            (default 8)
 * Results do not depend on them (beyond the 1 LSB alpha bound). */
int ochre_gpu_set_tunable(ochre_gpu_ctx *ctx, const char *name, int value);
int ochre_gpu_get_tunable(const ochre_gpu_ctx *ctx, const char *name, int *value);

/* Headless compositing (the reference example's GL path, examples/svg.rs,
 * restated): the rasters of a device result (ochre_gpu_rasterize_device),
 * each coloured with colors[4r .. 4r+3] (RGBA8), drawn in raster order onto
 * the RGBA8 canvas (w * h * 4 bytes, device, row-major, read and written):
 * fragment = colour * (1, 1, 1, mask / 255), blended SRC_ALPHA,
 * ONE_MINUS_SRC_ALPHA on all channels and quantised to 8 bits after every
 * quad.  colors and canvas are 4-byte aligned device pointers. */
int ochre_gpu_composite(ochre_gpu_ctx *ctx, const ochre_result *res, uint32_t n_rasters, const uint8_t *colors,
                        uint32_t w, uint32_t h, uint8_t *canvas, void *stream);

/* Status text for a code. */
const char *ochre_gpu_status_string(int status);

/* ---- Single-rasterizer mirror of the Rust API -------------------------- */

typedef struct ochre_rasterizer ochre_rasterizer;

/* TileBuilder::tile / TileBuilder::span (rasterizer.rs:14, 21). */
typedef void (*ochre_tile_fn)(void *user, int16_t x, int16_t y, const uint8_t data[64]);
typedef void (*ochre_span_fn)(void *user, int16_t x, int16_t y, uint16_t width);

/* Rasterizer::new (rasterizer.rs:50).  The rasterizer renders through ctx. */
int ochre_rasterizer_new(ochre_gpu_ctx *ctx, ochre_rasterizer **out);
/* Rasterizer::move_to / line_to (rasterizer.rs:61, 72): device-space points. */
int ochre_rasterizer_move_to(ochre_rasterizer *r, float x, float y);
int ochre_rasterizer_line_to(ochre_rasterizer *r, float x, float y);
/* Rasterizer::command (rasterizer.rs:145): one PathCmd, device space. */
int ochre_rasterizer_command(ochre_rasterizer *r, uint8_t verb, const float *floats);
/* Rasterizer::fill (rasterizer.rs:161): a path under a transform (6 floats). */
int ochre_rasterizer_fill(ochre_rasterizer *r, const uint8_t *verbs, size_t n_verbs,
                          const float *pts, size_t n_floats, const float xf[6]);

/* Rasterizer::stroke (rasterizer.rs:169-171): the path is stroked with the
 * given width in its own space, then filled with the transform. */
int ochre_rasterizer_stroke(ochre_rasterizer *r, const uint8_t *verbs, size_t n_verbs, const float *pts,
                            size_t n_floats, float width, const float xf[6]);
/* Rasterizer::finish (rasterizer.rs:180): rasterizes on the GPU, then calls
 * tile/span in the reference's order.  Consumes (frees) the rasterizer, even
 * on error. */
int ochre_rasterizer_finish(ochre_rasterizer *r, ochre_tile_fn tile, ochre_span_fn span, void *user);
/* Drop a rasterizer without finishing it. */
void ochre_rasterizer_free(ochre_rasterizer *r);

#ifdef __cplusplus
}
#endif
#endif /* OCHRE_GPU_H */
