/*
 * ORACLE — test infrastructure only (CPU restatement of ochre 0.2.0's
 * rasterizer; see ochre_oracle.c).  Parity with the reference: unpinned
 * (the Rust reference cannot be built here and ships no golden vectors).
 */
#ifndef OCHRE_ORACLE_H
#define OCHRE_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* PathCmd discriminants (path.rs:5-12); same numbering as the C-ABI. */
enum {
    OCHRE_ORACLE_MOVE = 0,
    OCHRE_ORACLE_LINE = 1,
    OCHRE_ORACLE_QUADRATIC = 2,
    OCHRE_ORACLE_CUBIC = 3,
    OCHRE_ORACLE_CONIC = 4,
    OCHRE_ORACLE_CLOSE = 5,
};

enum {
    OCHRE_ORACLE_E_INVALID = 1,
    OCHRE_ORACLE_E_NOMEM = 5,
    OCHRE_ORACLE_E_LIMIT = 6,
};

enum {
    OCHRE_ORACLE_WANT_COV = 1,      /* also return |accum + area| per tile pixel */
    OCHRE_ORACLE_CAPTURE_LINES = 2, /* also return every line_to segment */
    OCHRE_ORACLE_SIGNED_COV = 4,    /* with WANT_COV: accum + area before |.| */
};

/* Same layout as the product's ochre_batch (host pointers). */
typedef struct ochre_oracle_batch {
    const uint8_t *verbs;
    uint64_t n_cmds;
    const float *pts;
    uint64_t n_floats;
    const uint32_t *fill_cmd_off;    /* n_fills + 1 */
    const float *fill_xf;            /* 6 per fill */
    const uint8_t *fill_flags;       /* bit0: commands are not transformed; may be NULL */
    uint32_t n_fills;
    const uint32_t *raster_fill_off; /* n_rasters + 1; NULL means one fill per raster */
    uint32_t n_rasters;
    const float *fill_width;         /* n_fills, or NULL: stroke width of fills whose flags have bit1 */
} ochre_oracle_batch;

typedef struct ochre_oracle_result {
    uint32_t n_rasters;
    uint64_t n_tiles, n_spans, n_lines;
    int16_t *tile_xy;        /* 2 per tile */
    uint8_t *tile_alpha;     /* 64 per tile */
    float *tile_cov;         /* 64 per tile, or NULL */
    int16_t *span_xy;        /* 2 per span */
    uint16_t *span_w;
    uint32_t *span_tile;     /* global index of the tile the span follows */
    uint64_t *raster_tile_off, *raster_span_off, *raster_line_off; /* n_rasters + 1 */
    uint64_t *raster_stats;  /* 3 per raster: walked lines, increments, tile increments */
    float *lines;            /* 4 per captured line (x0, y0, x1, y1), or NULL */
    uint32_t *line_ninc;     /* increments per captured line */
    uint32_t error_raster;
} ochre_oracle_result;

int ochre_oracle_run(const ochre_oracle_batch *batch, int threads, int flags, ochre_oracle_result **out);

/* FP64 analytic coverage |sum| of the given f32 lines (4 floats each),
 * rasters delimited by raster_line_off, over one pixel rectangle per raster
 * (x0, y0, w, h); images are concatenated row-major into `out`. */
int ochre_oracle_cov64(const float *lines, const uint64_t *raster_line_off, uint32_t n_rasters,
                       const int32_t *rect, double *out);
void ochre_oracle_free(ochre_oracle_result *r);

/* Rasterizer::stroke's path preprocessing (path.rs:113-274): the path
 * flattened at the reference tolerance in its own space, then offset by
 * width / 2 on both sides with the reference's joins and caps.  Output:
 * Move / Line / Close commands (2 floats for Move and Line); the caller
 * frees *out_verbs and *out_pts with free(). */
int ochre_oracle_stroke(const uint8_t *verbs, uint64_t n_cmds, const float *pts, float width,
                        uint8_t **out_verbs, uint64_t *out_n_cmds, float **out_pts, uint64_t *out_n_floats);

/* Headless compositing of results (see ochre_oracle.c): rasters drawn in
 * order with their RGBA8 colours onto an RGBA8 w x h canvas (in place). */
void ochre_oracle_composite(uint32_t n_rasters, const int16_t *tile_xy, const uint8_t *tile_alpha,
                            const uint64_t *raster_tile_off, const int16_t *span_xy, const uint16_t *span_w,
                            const uint64_t *raster_span_off, const uint8_t *colors, uint32_t w, uint32_t h,
                            uint8_t *canvas);

/* Differentiable model in double (see ochre_oracle.c): per-command line
 * counts of the f32 flattening, then loss and gradients for a w x h canvas
 * per raster against `target` (n_rasters * w * h).  dpts / dxf may be NULL. */
int ochre_oracle_seg_counts(const ochre_oracle_batch *batch, uint32_t *counts);
int ochre_oracle_diff64(const ochre_oracle_batch *batch, const uint32_t *counts, int w, int h, const double *target,
                        double *loss, double *dpts, double *dxf);
/* The same backward from a given dL/dS per pixel (S = accum + area before
 * |.| and the clamp), n_rasters * w * h values. */
int ochre_oracle_backward64(const ochre_oracle_batch *batch, const uint32_t *counts, int w, int h, const double *dl_ds,
                            double *dpts, double *dxf);
/* The FP64 model's signed sums S = accum + area of every pixel ([R, H, W],
 * spans included as their running sums), target 0 and no gradient. */
int ochre_oracle_forward64(const ochre_oracle_batch *bt, const uint32_t *counts, int W, int H, double *s_out);

#ifdef __cplusplus
}
#endif
#endif
