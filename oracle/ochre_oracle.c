/*
 * ORACLE — test infrastructure only.
 *
 * A CPU restatement, in strict IEEE-754 single precision, of ochre 0.2.0's
 * path rasterizer (glowcoil/ochre).  It is the checker for the CUDA path in
 * ochre_gb300/csrc and the timed CPU baseline in bench.py ("kind": "port").
 * Nothing in the product links or calls it.
 *
 * Parity status: UNPINNED by the reference itself.  The reference is Rust
 * (no rustc/cargo on these machines) and ships no tests, golden vectors or
 * recorded outputs (its only executable example, examples/basic.rs, prints
 * and asserts nothing).  The restatement is cross-checked against an
 * independent pure-Python restatement (tests/oracle_py.py) and against
 * hand-derived known answers (tests/test_oracle.py).
 *
 * Build: oracle/__init__.py build() (gcc -O3 -ffp-contract=off -fno-fast-math
 * -fexcess-precision=standard): Rust never contracts a*b+c into an FMA, and
 * aarch64 gcc does by default, so contraction must be off for bit parity.
 *
 * Line-by-line sources (paths inside the ochre crate):
 *   geom.rs:19-21   dot            geom.rs:38-40  length
 *   geom.rs:50-52   lerp           geom.rs:170-178 Mat2x2 * Vec2
 *   geom.rs:260-262 Transform::apply
 *   path.rs:16-37   PathCmd::transform   path.rs:41-109 PathCmd::flatten
 *   rasterizer.rs:61-69  move_to   rasterizer.rs:72-140 line_to
 *   rasterizer.rs:145-157 command  rasterizer.rs:161-165 fill
 *   rasterizer.rs:180-268 finish
 */
#include "ochre_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ */
/* Rust scalar semantics (the casts and min/max used by the reference) */
/* ------------------------------------------------------------------ */

/* `f as i16`: truncate toward zero, saturate, NaN -> 0. */
static int16_t f2i16(float v) {
    if (v != v) return 0;
    if (v <= -32768.0f) return -32768;
    if (v >= 32767.0f) return 32767;
    return (int16_t)v;
}

/* `f as u8`: truncate toward zero, saturate, NaN -> 0. */
static uint8_t f2u8(float v) {
    if (v != v) return 0;
    if (v <= 0.0f) return 0;
    if (v >= 255.0f) return 255;
    return (uint8_t)v;
}

/* `f32::signum(v) as i16`: +0 and +inf give 1, -0 and -inf give -1,
 * NaN gives NaN which casts to 0. */
static int16_t signum_i16(float v) {
    if (v != v) return 0;
    return signbit(v) ? -1 : 1;
}

/* i16::wrapping_div_euclid(8): floor division for a positive divisor. */
static int16_t div8(int16_t v) {
    int q = (int)v / 8;
    if ((int)v % 8 < 0) q -= 1;
    return (int16_t)q;
}

/* f32::min / f32::max return the non-NaN operand, as fminf / fmaxf do. */
static float rmin(float a, float b) { return fminf(a, b); }
static float rmax(float a, float b) { return fmaxf(a, b); }

/* ------------------------------------------------------------------ */
/* geom.rs                                                             */
/* ------------------------------------------------------------------ */
typedef struct { float x, y; } vec2;

static vec2 v2(float x, float y) { vec2 r = {x, y}; return r; }
static vec2 vadd(vec2 a, vec2 b) { return v2(a.x + b.x, a.y + b.y); }
static vec2 vsub(vec2 a, vec2 b) { return v2(a.x - b.x, a.y - b.y); }
static vec2 vscale(float s, vec2 a) { return v2(s * a.x, s * a.y); }
static int veq(vec2 a, vec2 b) { return a.x == b.x && a.y == b.y; }
static float vlength(vec2 a) { return sqrtf(a.x * a.x + a.y * a.y); }
static float vdot(vec2 a, vec2 b) { return a.x * b.x + a.y * b.y; }
/* Vec2 * f32 (geom.rs:108-117) */
static vec2 vmul(vec2 a, float s) { return v2(a.x * s, a.y * s); }
/* lerp(t, a, b) = (1 - t) * a + t * b */
static vec2 vlerp(float t, vec2 a, vec2 b) {
    return vadd(vscale(1.0f - t, a), vscale(t, b));
}
/* Transform::apply: matrix * v + offset, matrix row-major [m0 m1; m2 m3]. */
static vec2 xf_apply(const float *xf, vec2 v) {
    vec2 m = v2(xf[0] * v.x + xf[1] * v.y, xf[2] * v.x + xf[3] * v.y);
    return vadd(m, v2(xf[4], xf[5]));
}

/* ------------------------------------------------------------------ */
/* rasterizer.rs                                                       */
/* ------------------------------------------------------------------ */
#define TILE 8
#define TOLERANCE 0.1f

typedef struct { int16_t x, y; float area, height; } increment;
typedef struct { int16_t tile_x, tile_y; int8_t sign; } tile_increment;

typedef struct {
    increment *inc; size_t n_inc, cap_inc;
    tile_increment *tinc; size_t n_tinc, cap_tinc;
    vec2 first, last;
    int16_t tile_y_prev;
    /* statistics and safety */
    uint64_t n_lines;        /* line_to calls that walked (point != last) */
    int error;               /* nonzero: an iteration cap was hit */
    /* optional line capture (intermediate parity) */
    float *lines; size_t n_lines_cap_used, cap_lines;
    uint32_t *line_ninc;
    int capture_lines;
} rasterizer;

/* Iteration caps: the reference would loop (or allocate) without bound on
 * such inputs; the oracle stops and reports instead. */
#define WALK_CAP (1u << 20)
#define FLATTEN_CAP (1u << 20)
#define CONIC_DEPTH_CAP 64

static int push_inc(rasterizer *r, increment v) {
    if (r->n_inc == r->cap_inc) {
        size_t c = r->cap_inc ? r->cap_inc * 2 : 256;
        increment *p = (increment *)realloc(r->inc, c * sizeof *p);
        if (!p) { r->error = OCHRE_ORACLE_E_NOMEM; return 0; }
        r->inc = p; r->cap_inc = c;
    }
    r->inc[r->n_inc++] = v;
    return 1;
}

static int push_tinc(rasterizer *r, tile_increment v) {
    if (r->n_tinc == r->cap_tinc) {
        size_t c = r->cap_tinc ? r->cap_tinc * 2 : 64;
        tile_increment *p = (tile_increment *)realloc(r->tinc, c * sizeof *p);
        if (!p) { r->error = OCHRE_ORACLE_E_NOMEM; return 0; }
        r->tinc = p; r->cap_tinc = c;
    }
    r->tinc[r->n_tinc++] = v;
    return 1;
}

static void capture_line(rasterizer *r, vec2 a, vec2 b, uint32_t ninc) {
    if (!r->capture_lines) return;
    if (r->n_lines_cap_used == r->cap_lines) {
        size_t c = r->cap_lines ? r->cap_lines * 2 : 256;
        float *p = (float *)realloc(r->lines, c * 4 * sizeof(float));
        uint32_t *q = (uint32_t *)realloc(r->line_ninc, c * sizeof(uint32_t));
        if (!p || !q) { r->error = OCHRE_ORACLE_E_NOMEM; free(p); return; }
        r->lines = p; r->line_ninc = q; r->cap_lines = c;
    }
    float *d = r->lines + 4 * r->n_lines_cap_used;
    d[0] = a.x; d[1] = a.y; d[2] = b.x; d[3] = b.y;
    r->line_ninc[r->n_lines_cap_used++] = ninc;
}

static void rasterizer_init(rasterizer *r) {
    memset(r, 0, sizeof *r);
    r->first = v2(0.0f, 0.0f);
    r->last = v2(0.0f, 0.0f);
    r->tile_y_prev = 0;
}

static void rasterizer_free(rasterizer *r) {
    free(r->inc); free(r->tinc); free(r->lines); free(r->line_ninc);
}

static void line_to(rasterizer *r, vec2 point);

/* rasterizer.rs:61-69 */
static void move_to(rasterizer *r, vec2 point) {
    if (!veq(r->last, r->first)) line_to(r, r->first);
    r->first = point;
    r->last = point;
    r->tile_y_prev = div8(f2i16(floorf(point.y)));
}

/* rasterizer.rs:72-140: the pixel DDA. */
static void line_to(rasterizer *r, vec2 point) {
    vec2 last = r->last;
    size_t inc_before = r->n_inc;
    int walked = 0;
    if (!veq(point, last)) {
        walked = 1;
        int16_t x_dir = signum_i16(point.x - last.x);
        int16_t y_dir = signum_i16(point.y - last.y);
        float dtdx = 1.0f / (point.x - last.x);
        float dtdy = 1.0f / (point.y - last.y);
        int16_t x = f2i16(floorf(last.x));
        int16_t y = f2i16(floorf(last.y));
        float row_t0 = 0.0f, col_t0 = 0.0f;
        float row_t1, col_t1;
        if (last.y == point.y) {
            row_t1 = INFINITY;
        } else {
            float next_y = point.y > last.y ? (float)(int16_t)(y + 1) : (float)y;
            row_t1 = rmin(dtdy * (next_y - last.y), 1.0f);
        }
        if (last.x == point.x) {
            col_t1 = INFINITY;
        } else {
            float next_x = point.x > last.x ? (float)(int16_t)(x + 1) : (float)x;
            col_t1 = rmin(dtdx * (next_x - last.x), 1.0f);
        }
        float x_step = fabsf(dtdx);
        float y_step = fabsf(dtdy);

        uint32_t iters = 0;
        for (;;) {
            float t0 = rmax(row_t0, col_t0);
            float t1 = rmin(row_t1, col_t1);
            vec2 p0 = vadd(vscale(1.0f - t0, last), vscale(t0, point));
            vec2 p1 = vadd(vscale(1.0f - t1, last), vscale(t1, point));
            float height = p1.y - p0.y;
            float right = (float)(int16_t)(x + 1);
            float area = 0.5f * height * ((right - p0.x) + (right - p1.x));
            increment inc = {x, y, area, height};
            if (!push_inc(r, inc)) return;

            if (row_t1 < col_t1) {
                row_t0 = row_t1;
                row_t1 = rmin(row_t1 + y_step, 1.0f);
                y = (int16_t)(y + y_dir);
            } else {
                col_t0 = col_t1;
                col_t1 = rmin(col_t1 + x_step, 1.0f);
                x = (int16_t)(x + x_dir);
            }

            int done = row_t0 == 1.0f || col_t0 == 1.0f;
            if (done) {
                x = f2i16(floorf(point.x));
                y = f2i16(floorf(point.y));
            }

            int16_t tile_y = div8(y);
            if (tile_y != r->tile_y_prev) {
                tile_increment ti;
                ti.tile_x = div8(x);
                ti.tile_y = r->tile_y_prev < tile_y ? r->tile_y_prev : tile_y;
                ti.sign = (int8_t)(int16_t)(tile_y - r->tile_y_prev);
                if (!push_tinc(r, ti)) return;
                r->tile_y_prev = tile_y;
            }

            if (done) break;
            if (++iters >= WALK_CAP) { r->error = OCHRE_ORACLE_E_LIMIT; break; }
        }
        r->n_lines++;
    }
    capture_line(r, last, point, walked ? (uint32_t)(r->n_inc - inc_before) : 0u);
    r->last = point;
}

/* path.rs:76-101 */
static void flatten_conic(rasterizer *r, vec2 last, vec2 control, vec2 point, float weight,
                          float t0, float t1, vec2 p0, vec2 p1, int depth) {
    float t = 0.5f * (t0 + t1);
    vec2 wc = vscale(weight, control);
    vec2 p01 = vlerp(t, last, wc);
    vec2 p12 = vlerp(t, wc, point);
    float denom = (1.0f - t) * (1.0f - t) + 2.0f * t * (1.0f - t) * weight + t * t;
    vec2 midpoint = vscale(1.0f / denom, vlerp(t, p01, p12));
    float err = vlength(vsub(midpoint, vscale(0.5f, vadd(p0, p1))));
    if (err > TOLERANCE) {
        if (depth >= CONIC_DEPTH_CAP) { r->error = OCHRE_ORACLE_E_LIMIT; return; }
        flatten_conic(r, last, control, point, weight, t0, t, p0, midpoint, depth + 1);
        flatten_conic(r, last, control, point, weight, t, t1, midpoint, p1, depth + 1);
    } else {
        line_to(r, midpoint);
        line_to(r, p1);
    }
}

/* rasterizer.rs:145-157 with path.rs:41-109 inlined (the callback only
 * dispatches Move and Line; Close is ignored). `last` is the rasterizer's
 * last point at the time of the call. */
static void command(rasterizer *r, uint8_t verb, const vec2 *p, float weight) {
    vec2 last = r->last;
    switch (verb) {
    case OCHRE_ORACLE_MOVE:
        move_to(r, p[0]);
        break;
    case OCHRE_ORACLE_LINE:
        line_to(r, p[0]);
        break;
    case OCHRE_ORACLE_QUADRATIC: {
        vec2 control = p[0], point = p[1];
        float dt = sqrtf((4.0f * TOLERANCE) / vlength(vadd(vsub(last, vscale(2.0f, control)), point)));
        float t = 0.0f;
        uint32_t n = 0;
        while (t < 1.0f) {
            t = rmin(t + dt, 1.0f);
            vec2 p01 = vlerp(t, last, control);
            vec2 p12 = vlerp(t, control, point);
            line_to(r, vlerp(t, p01, p12));
            if (++n >= FLATTEN_CAP) { r->error = OCHRE_ORACLE_E_LIMIT; break; }
        }
        break;
    }
    case OCHRE_ORACLE_CUBIC: {
        vec2 c1 = p[0], c2 = p[1], point = p[2];
        vec2 a = vadd(vsub(vadd(vscale(-1.0f, last), vscale(3.0f, c1)), vscale(3.0f, c2)), point);
        vec2 b = vscale(3.0f, vadd(vsub(last, vscale(2.0f, c1)), c2));
        float conc = rmax(vlength(b), vlength(vadd(a, b)));
        float dt = sqrtf((sqrtf(8.0f) * TOLERANCE) / conc);
        float t = 0.0f;
        uint32_t n = 0;
        while (t < 1.0f) {
            t = rmin(t + dt, 1.0f);
            vec2 p01 = vlerp(t, last, c1);
            vec2 p12 = vlerp(t, c1, c2);
            vec2 p23 = vlerp(t, c2, point);
            vec2 p012 = vlerp(t, p01, p12);
            vec2 p123 = vlerp(t, p12, p23);
            line_to(r, vlerp(t, p012, p123));
            if (++n >= FLATTEN_CAP) { r->error = OCHRE_ORACLE_E_LIMIT; break; }
        }
        break;
    }
    case OCHRE_ORACLE_CONIC:
        flatten_conic(r, last, p[0], p[1], weight, 0.0f, 1.0f, last, p[1], 0);
        break;
    default: /* Close */
        break;
    }
}

/* ------------------------------------------------------------------ */
/* finish (rasterizer.rs:180-268) into a collecting builder            */
/* ------------------------------------------------------------------ */
typedef struct { int16_t tile_x, tile_y; size_t start, end; } bin;

static int cmp_bin(const void *a, const void *b) {
    const bin *x = (const bin *)a, *y = (const bin *)b;
    if (x->tile_y != y->tile_y) return x->tile_y < y->tile_y ? -1 : 1;
    if (x->tile_x != y->tile_x) return x->tile_x < y->tile_x ? -1 : 1;
    /* Any order is a valid outcome of the reference's unstable sort; take
     * emission order so the oracle is deterministic. */
    return x->start < y->start ? -1 : (x->start > y->start);
}

typedef struct { tile_increment t; size_t idx; } tinc_ix;
static int cmp_tinc(const void *a, const void *b) {
    const tinc_ix *x = (const tinc_ix *)a, *y = (const tinc_ix *)b;
    if (x->t.tile_y != y->t.tile_y) return x->t.tile_y < y->t.tile_y ? -1 : 1;
    if (x->t.tile_x != y->t.tile_x) return x->t.tile_x < y->t.tile_x ? -1 : 1;
    return x->idx < y->idx ? -1 : (x->idx > y->idx);
}

typedef struct {
    int16_t *tile_xy; uint8_t *tile_alpha; float *tile_cov;
    size_t n_tiles, cap_tiles;
    int16_t *span_xy; uint16_t *span_w; uint32_t *span_tile;
    size_t n_spans, cap_spans;
    int want_cov;
    int error;
} collector;

static void coll_tile(collector *c, int16_t x, int16_t y, const uint8_t *data, const float *cov) {
    if (c->n_tiles == c->cap_tiles) {
        size_t n = c->cap_tiles ? c->cap_tiles * 2 : 64;
        int16_t *a = (int16_t *)realloc(c->tile_xy, n * 2 * sizeof(int16_t));
        if (a) c->tile_xy = a;
        uint8_t *b = (uint8_t *)realloc(c->tile_alpha, n * 64);
        if (b) c->tile_alpha = b;
        if (!a || !b) { c->error = OCHRE_ORACLE_E_NOMEM; return; }
        if (c->want_cov) {
            float *f = (float *)realloc(c->tile_cov, n * 64 * sizeof(float));
            if (!f) { c->error = OCHRE_ORACLE_E_NOMEM; return; }
            c->tile_cov = f;
        }
        c->cap_tiles = n;
    }
    c->tile_xy[2 * c->n_tiles] = x;
    c->tile_xy[2 * c->n_tiles + 1] = y;
    memcpy(c->tile_alpha + 64 * c->n_tiles, data, 64);
    if (c->want_cov) memcpy(c->tile_cov + 64 * c->n_tiles, cov, 64 * sizeof(float));
    c->n_tiles++;
}

static void coll_span(collector *c, int16_t x, int16_t y, uint16_t w) {
    if (c->n_spans == c->cap_spans) {
        size_t n = c->cap_spans ? c->cap_spans * 2 : 16;
        int16_t *a = (int16_t *)realloc(c->span_xy, n * 2 * sizeof(int16_t));
        if (a) c->span_xy = a;
        uint16_t *b = (uint16_t *)realloc(c->span_w, n * sizeof(uint16_t));
        if (b) c->span_w = b;
        uint32_t *d = (uint32_t *)realloc(c->span_tile, n * sizeof(uint32_t));
        if (d) c->span_tile = d;
        if (!a || !b || !d) { c->error = OCHRE_ORACLE_E_NOMEM; return; }
        c->cap_spans = n;
    }
    c->span_xy[2 * c->n_spans] = x;
    c->span_xy[2 * c->n_spans + 1] = y;
    c->span_w[c->n_spans] = w;
    c->span_tile[c->n_spans] = (uint32_t)(c->n_tiles - 1); /* follows the last tile */
    c->n_spans++;
}

static void finish(rasterizer *r, collector *out) {
    if (!veq(r->last, r->first)) line_to(r, r->first);

    size_t cap = 16, nb = 0;
    bin *bins = (bin *)malloc(cap * sizeof(bin));
    if (!bins) { out->error = OCHRE_ORACLE_E_NOMEM; return; }
    bin b = {0, 0, 0, 0};
    if (r->n_inc > 0) {
        b.tile_x = div8(r->inc[0].x);
        b.tile_y = div8(r->inc[0].y);
    }
    for (size_t i = 0; i < r->n_inc; i++) {
        int16_t tx = div8(r->inc[i].x), ty = div8(r->inc[i].y);
        if (tx != b.tile_x || ty != b.tile_y) {
            if (nb == cap) { cap *= 2; bin *p = (bin *)realloc(bins, cap * sizeof(bin)); if (!p) { free(bins); out->error = OCHRE_ORACLE_E_NOMEM; return; } bins = p; }
            bins[nb++] = b;
            b.tile_x = tx; b.tile_y = ty; b.start = i; b.end = i;
        }
        b.end += 1;
    }
    if (nb == cap) { cap *= 2; bin *p = (bin *)realloc(bins, cap * sizeof(bin)); if (!p) { free(bins); out->error = OCHRE_ORACLE_E_NOMEM; return; } bins = p; }
    bins[nb++] = b;
    qsort(bins, nb, sizeof(bin), cmp_bin);

    tinc_ix *ti = (tinc_ix *)malloc((r->n_tinc ? r->n_tinc : 1) * sizeof(tinc_ix));
    if (!ti) { free(bins); out->error = OCHRE_ORACLE_E_NOMEM; return; }
    for (size_t i = 0; i < r->n_tinc; i++) { ti[i].t = r->tinc[i]; ti[i].idx = i; }
    qsort(ti, r->n_tinc, sizeof(tinc_ix), cmp_tinc);

    float areas[64] = {0}, heights[64] = {0}, prev[8] = {0}, next[8] = {0};
    size_t tinc_i = 0;
    long long winding = 0;

    for (size_t i = 0; i < nb; i++) {
        bin bn = bins[i];
        for (size_t k = bn.start; k < bn.end; k++) {
            const increment *inc = &r->inc[k];
            unsigned x = (unsigned)(uint16_t)inc->x & 7u; /* (x as usize).rem_euclid(8) */
            unsigned y = (unsigned)(uint16_t)inc->y & 7u;
            areas[y * 8 + x] += inc->area;
            heights[y * 8 + x] += inc->height;
        }
        if (i + 1 == nb || bins[i + 1].tile_x != bn.tile_x || bins[i + 1].tile_y != bn.tile_y) {
            uint8_t tile[64];
            float cov[64];
            for (int y = 0; y < 8; y++) {
                float accum = prev[y];
                for (int x = 0; x < 8; x++) {
                    const float sum = accum + areas[y * 8 + x];
                    float c = fabsf(sum);
                    cov[y * 8 + x] = out->want_cov == 2 ? sum : c;
                    tile[y * 8 + x] = f2u8(rmin(c * 256.0f, 255.0f));
                    accum += heights[y * 8 + x];
                }
                next[y] = accum;
            }
            coll_tile(out, (int16_t)(bn.tile_x * 8), (int16_t)(bn.tile_y * 8), tile, cov);

            memset(areas, 0, sizeof areas);
            memset(heights, 0, sizeof heights);
            if (i + 1 < nb && bins[i + 1].tile_y == bn.tile_y) memcpy(prev, next, sizeof prev);
            else memset(prev, 0, sizeof prev);
            memset(next, 0, sizeof next);

            if (i + 1 < nb && bins[i + 1].tile_y == bn.tile_y && bins[i + 1].tile_x > bn.tile_x + 1) {
                while (tinc_i < r->n_tinc) {
                    tile_increment t = ti[tinc_i].t;
                    if (t.tile_y > bn.tile_y || (t.tile_y == bn.tile_y && t.tile_x > bn.tile_x)) break;
                    winding += t.sign;
                    tinc_i++;
                }
                if (winding != 0) {
                    int16_t width = (int16_t)(bins[i + 1].tile_x - bn.tile_x - 1);
                    coll_span(out, (int16_t)((bn.tile_x + 1) * 8), (int16_t)(bn.tile_y * 8),
                              (uint16_t)((uint16_t)width * 8u));
                }
            }
        }
    }
    free(bins);
    free(ti);
}

/* ------------------------------------------------------------------ */
/* Batch entry: each raster is Rasterizer::new -> fill* -> finish       */
/* ------------------------------------------------------------------ */
static const int FLOATS_PER_VERB[6] = {2, 2, 4, 6, 5, 0};

typedef struct {
    collector c;
    uint64_t n_lines, n_inc, n_tinc;
    float *lines; uint32_t *line_ninc; size_t n_cap_lines;
    int error;
} raster_out;

/* ------------------------------------------------------------------ */
/* path.rs:113-274: flatten() and stroke()                             */
/* ------------------------------------------------------------------ */
typedef struct {
    uint8_t *verbs;
    float *pts;          /* 2 per command (Close: unused zeros) */
    size_t n, cap;
    int error;
} pbuf;

static void pb_push(pbuf *b, uint8_t verb, vec2 p) {
    if (b->error) return;
    if (b->n == b->cap) {
        size_t c = b->cap ? b->cap * 2 : 64;
        uint8_t *v = (uint8_t *)realloc(b->verbs, c);
        float *q = (float *)realloc(b->pts, c * 2 * sizeof(float));
        if (v) b->verbs = v;
        if (q) b->pts = q;
        if (!v || !q) { b->error = OCHRE_ORACLE_E_NOMEM; return; }
        b->cap = c;
    }
    b->verbs[b->n] = verb;
    b->pts[2 * b->n] = p.x;
    b->pts[2 * b->n + 1] = p.y;
    b->n++;
}

static vec2 pb_point(const pbuf *b, size_t i) { return v2(b->pts[2 * i], b->pts[2 * i + 1]); }

/* path.rs:76-101, emitting Line commands */
static void pb_flatten_conic(pbuf *b, vec2 last, vec2 control, vec2 point, float weight, float t0, float t1,
                             vec2 p0, vec2 p1, int depth) {
    float t = 0.5f * (t0 + t1);
    vec2 wc = vscale(weight, control);
    vec2 p01 = vlerp(t, last, wc);
    vec2 p12 = vlerp(t, wc, point);
    float denom = (1.0f - t) * (1.0f - t) + 2.0f * t * (1.0f - t) * weight + t * t;
    vec2 midpoint = vscale(1.0f / denom, vlerp(t, p01, p12));
    float err = vlength(vsub(midpoint, vscale(0.5f, vadd(p0, p1))));
    if (err > TOLERANCE) {
        if (depth >= CONIC_DEPTH_CAP) { b->error = OCHRE_ORACLE_E_LIMIT; return; }
        pb_flatten_conic(b, last, control, point, weight, t0, t, p0, midpoint, depth + 1);
        pb_flatten_conic(b, last, control, point, weight, t, t1, midpoint, p1, depth + 1);
    } else {
        pb_push(b, OCHRE_ORACLE_LINE, midpoint);
        pb_push(b, OCHRE_ORACLE_LINE, p1);
    }
}

/* path.rs:113-142: `last` starts at the origin and follows every command's
 * end point (Close leaves it). */
static void path_flatten(const uint8_t *verbs, uint64_t n, const float *pts, pbuf *out) {
    vec2 last = v2(0.0f, 0.0f);
    uint64_t fo = 0;
    for (uint64_t c = 0; c < n && !out->error; c++) {
        const float *fp = pts + fo;
        fo += FLOATS_PER_VERB[verbs[c]];
        switch (verbs[c]) {
        case OCHRE_ORACLE_MOVE:
            pb_push(out, OCHRE_ORACLE_MOVE, v2(fp[0], fp[1]));
            last = v2(fp[0], fp[1]);
            break;
        case OCHRE_ORACLE_LINE:
            pb_push(out, OCHRE_ORACLE_LINE, v2(fp[0], fp[1]));
            last = v2(fp[0], fp[1]);
            break;
        case OCHRE_ORACLE_QUADRATIC: {
            vec2 control = v2(fp[0], fp[1]), point = v2(fp[2], fp[3]);
            float dt = sqrtf((4.0f * TOLERANCE) / vlength(vadd(vsub(last, vscale(2.0f, control)), point)));
            float t = 0.0f;
            uint32_t k = 0;
            while (t < 1.0f) {
                t = rmin(t + dt, 1.0f);
                pb_push(out, OCHRE_ORACLE_LINE, vlerp(t, vlerp(t, last, control), vlerp(t, control, point)));
                if (++k >= FLATTEN_CAP) { out->error = OCHRE_ORACLE_E_LIMIT; break; }
            }
            last = point;
            break;
        }
        case OCHRE_ORACLE_CUBIC: {
            vec2 c1 = v2(fp[0], fp[1]), c2 = v2(fp[2], fp[3]), point = v2(fp[4], fp[5]);
            vec2 a = vadd(vsub(vadd(vscale(-1.0f, last), vscale(3.0f, c1)), vscale(3.0f, c2)), point);
            vec2 bb = vscale(3.0f, vadd(vsub(last, vscale(2.0f, c1)), c2));
            float conc = rmax(vlength(bb), vlength(vadd(a, bb)));
            float dt = sqrtf((sqrtf(8.0f) * TOLERANCE) / conc);
            float t = 0.0f;
            uint32_t k = 0;
            while (t < 1.0f) {
                t = rmin(t + dt, 1.0f);
                vec2 p01 = vlerp(t, last, c1), p12 = vlerp(t, c1, c2), p23 = vlerp(t, c2, point);
                pb_push(out, OCHRE_ORACLE_LINE, vlerp(t, vlerp(t, p01, p12), vlerp(t, p12, p23)));
                if (++k >= FLATTEN_CAP) { out->error = OCHRE_ORACLE_E_LIMIT; break; }
            }
            last = point;
            break;
        }
        case OCHRE_ORACLE_CONIC: {
            vec2 control = v2(fp[0], fp[1]), point = v2(fp[2], fp[3]);
            pb_flatten_conic(out, last, control, point, fp[4], 0.0f, 1.0f, last, point, 0);
            last = point;
            break;
        }
        default:
            pb_push(out, OCHRE_ORACLE_CLOSE, v2(0.0f, 0.0f));
            break;
        }
    }
}

/* path.rs:160-168 */
static void stroke_join(pbuf *out, float width, vec2 prev_normal, vec2 next_normal, vec2 point) {
    const float offset = 1.0f / (1.0f + vdot(prev_normal, next_normal));
    if (fabsf(offset) > 2.0f) {
        pb_push(out, OCHRE_ORACLE_LINE, vadd(point, vscale(0.5f * width, prev_normal)));
        pb_push(out, OCHRE_ORACLE_LINE, vadd(point, vscale(0.5f * width, next_normal)));
    } else {
        pb_push(out, OCHRE_ORACLE_LINE, vadd(point, vscale(0.5f * width * offset, vadd(prev_normal, next_normal))));
    }
}

/* path.rs:170-212: one side of a contour (poly[c0, c1)) */
static void stroke_offset(pbuf *out, float width, const pbuf *poly, size_t c0, size_t c1, int closed, int reverse) {
    const size_t len = c1 - c0;
    const vec2 first_point = closed == reverse ? pb_point(poly, c0) : pb_point(poly, c1 - 1);
    vec2 prev_point = first_point;
    vec2 prev_normal = v2(0.0f, 0.0f);
    for (size_t i = 0;; i++) {
        vec2 next_point;
        if (i < len) next_point = reverse ? pb_point(poly, c0 + len - i - 1) : pb_point(poly, c0 + i);
        else next_point = first_point;
        if (!veq(next_point, prev_point) || i == len) {
            const vec2 next_tangent = vsub(next_point, prev_point);
            vec2 next_normal = v2(-next_tangent.y, next_tangent.x);
            const float next_normal_len = vlength(next_normal);
            next_normal = next_normal_len == 0.0f ? v2(0.0f, 0.0f) : vmul(next_normal, 1.0f / next_normal_len);
            stroke_join(out, width, prev_normal, next_normal, prev_point);
            prev_point = next_point;
            prev_normal = next_normal;
        }
        if (i + 1 > len) break;
    }
}

/* path.rs:214-274.  Contours run from a Move (or the command after a Close)
 * to the next Move / Close / end; `closed` becomes true at the first Close
 * and stays true for the rest of the path. */
static void stroke_path(const pbuf *poly, float width, pbuf *out) {
    size_t start = 0, end = 0;
    int closed = 0;
    for (size_t k = 0;; k++) {
        const int have = k < poly->n;
        const uint8_t verb = have ? poly->verbs[k] : 0xff;
        if (have && verb == OCHRE_ORACLE_CLOSE) closed = 1;
        if (!have || verb == OCHRE_ORACLE_MOVE || verb == OCHRE_ORACLE_CLOSE) {
            if (start != end) {
                size_t base = out->n;
                stroke_offset(out, width, poly, start, end, closed, 0);
                if (!out->error) out->verbs[base] = OCHRE_ORACLE_MOVE;
                if (closed) pb_push(out, OCHRE_ORACLE_CLOSE, v2(0.0f, 0.0f));
                base = out->n;
                stroke_offset(out, width, poly, start, end, closed, 1);
                if (closed && !out->error) out->verbs[base] = OCHRE_ORACLE_MOVE;
                pb_push(out, OCHRE_ORACLE_CLOSE, v2(0.0f, 0.0f));
            }
        }
        if (!have) break;
        if (verb == OCHRE_ORACLE_MOVE) {
            start = end;
            end = start + 1;
        } else if (verb == OCHRE_ORACLE_LINE) {
            end += 1;
        } else {   /* Close */
            start = end + 1;
            end = start;
            closed = 1;
        }
    }
}

int ochre_oracle_stroke(const uint8_t *verbs, uint64_t n_cmds, const float *pts, float width,
                        uint8_t **out_verbs, uint64_t *out_n_cmds, float **out_pts, uint64_t *out_n_floats) {
    *out_verbs = NULL;
    *out_pts = NULL;
    *out_n_cmds = 0;
    *out_n_floats = 0;
    for (uint64_t c = 0; c < n_cmds; c++)
        if (verbs[c] > 5) return OCHRE_ORACLE_E_INVALID;
    pbuf poly = {0}, out = {0};
    path_flatten(verbs, n_cmds, pts, &poly);
    if (!poly.error) stroke_path(&poly, width, &out);
    int st = poly.error ? poly.error : out.error;
    free(poly.verbs);
    free(poly.pts);
    if (st) { free(out.verbs); free(out.pts); return st; }
    /* compact the float stream: Move/Line keep 2 floats, Close none */
    uint64_t nf = 0;
    for (size_t i = 0; i < out.n; i++)
        if (out.verbs[i] != OCHRE_ORACLE_CLOSE) {
            out.pts[nf] = out.pts[2 * i];
            out.pts[nf + 1] = out.pts[2 * i + 1];
            nf += 2;
        }
    *out_verbs = out.verbs;
    *out_pts = out.pts;
    *out_n_cmds = out.n;
    *out_n_floats = nf;
    return 0;
}

static void run_raster(const ochre_oracle_batch *bt, const uint64_t *cmd_float_off, uint32_t ri,
                       int want_cov, int capture, raster_out *ro) {
    rasterizer r;
    rasterizer_init(&r);
    r.capture_lines = capture;
    memset(&ro->c, 0, sizeof ro->c);
    ro->c.want_cov = want_cov;
    uint32_t f0 = bt->raster_fill_off ? bt->raster_fill_off[ri] : ri;
    uint32_t f1 = bt->raster_fill_off ? bt->raster_fill_off[ri + 1] : ri + 1;
    for (uint32_t f = f0; f < f1 && !r.error; f++) {
        const float *xf = bt->fill_xf + 6 * (size_t)f;
        int raw = bt->fill_flags ? (bt->fill_flags[f] & 1) : 0;
        if (bt->fill_flags && (bt->fill_flags[f] & 2) && bt->fill_width) {
            /* Rasterizer::stroke (rasterizer.rs:169-171): fill(stroke(flatten(path)), transform) */
            const uint32_t c0 = bt->fill_cmd_off[f], c1 = bt->fill_cmd_off[f + 1];
            uint8_t *sv;
            float *sp;
            uint64_t sn, snf;
            int e = ochre_oracle_stroke(bt->verbs + c0, c1 - c0, bt->pts + cmd_float_off[c0], bt->fill_width[f],
                                        &sv, &sn, &sp, &snf);
            if (e) { r.error = e; break; }
            uint64_t fo = 0;
            for (uint64_t k = 0; k < sn && !r.error; k++) {
                vec2 q[1] = {v2(0.0f, 0.0f)};
                if (sv[k] != OCHRE_ORACLE_CLOSE) {
                    q[0] = v2(sp[fo], sp[fo + 1]);
                    fo += 2;
                    if (!raw) q[0] = xf_apply(xf, q[0]);
                }
                command(&r, sv[k], q, 0.0f);
            }
            free(sv);
            free(sp);
            continue;
        }
        for (uint32_t c = bt->fill_cmd_off[f]; c < bt->fill_cmd_off[f + 1] && !r.error; c++) {
            uint8_t verb = bt->verbs[c];
            const float *fp = bt->pts + cmd_float_off[c];
            vec2 p[3];
            float w = 0.0f;
            int np = 0;
            switch (verb) {
            case OCHRE_ORACLE_MOVE: case OCHRE_ORACLE_LINE: np = 1; break;
            case OCHRE_ORACLE_QUADRATIC: np = 2; break;
            case OCHRE_ORACLE_CUBIC: np = 3; break;
            case OCHRE_ORACLE_CONIC: np = 2; w = fp[4]; break;
            default: np = 0; break;
            }
            for (int k = 0; k < np; k++) {
                p[k] = v2(fp[2 * k], fp[2 * k + 1]);
                if (!raw) p[k] = xf_apply(xf, p[k]); /* PathCmd::transform, path.rs:16-37 */
            }
            command(&r, verb, p, w);
        }
    }
    if (!r.error) finish(&r, &ro->c);
    ro->n_lines = r.n_lines;
    ro->n_inc = r.n_inc;
    ro->n_tinc = r.n_tinc;
    ro->error = r.error ? r.error : ro->c.error;
    if (capture) {
        ro->lines = r.lines; ro->line_ninc = r.line_ninc; ro->n_cap_lines = r.n_lines_cap_used;
        r.lines = NULL; r.line_ninc = NULL;
    }
    rasterizer_free(&r);
}

typedef struct {
    const ochre_oracle_batch *bt;
    const uint64_t *cmd_float_off;
    raster_out *outs;
    atomic_uint next;
    int want_cov, capture;
} pool_ctx;

static void *worker(void *arg) {
    pool_ctx *pc = (pool_ctx *)arg;
    for (;;) {
        unsigned ri = atomic_fetch_add(&pc->next, 1u);
        if (ri >= pc->bt->n_rasters) break;
        run_raster(pc->bt, pc->cmd_float_off, ri, pc->want_cov, pc->capture, &pc->outs[ri]);
    }
    return NULL;
}

static int validate(const ochre_oracle_batch *bt, uint64_t **off_out) {
    uint64_t *off = (uint64_t *)malloc((bt->n_cmds + 1) * sizeof(uint64_t));
    if (!off) return OCHRE_ORACLE_E_NOMEM;
    uint64_t acc = 0;
    for (uint64_t c = 0; c < bt->n_cmds; c++) {
        if (bt->verbs[c] > 5) { free(off); return OCHRE_ORACLE_E_INVALID; }
        off[c] = acc;
        acc += (uint64_t)FLOATS_PER_VERB[bt->verbs[c]];
    }
    off[bt->n_cmds] = acc;
    if (acc > bt->n_floats) { free(off); return OCHRE_ORACLE_E_INVALID; }
    if (bt->fill_cmd_off[0] != 0 || bt->fill_cmd_off[bt->n_fills] != bt->n_cmds) { free(off); return OCHRE_ORACLE_E_INVALID; }
    *off_out = off;
    return 0;
}

int ochre_oracle_run(const ochre_oracle_batch *bt, int threads, int flags, ochre_oracle_result **res_out) {
    *res_out = NULL;
    uint64_t *off = NULL;
    int st = validate(bt, &off);
    if (st) return st;
    raster_out *outs = (raster_out *)calloc(bt->n_rasters ? bt->n_rasters : 1, sizeof(raster_out));
    if (!outs) { free(off); return OCHRE_ORACLE_E_NOMEM; }
    int want_cov = (flags & OCHRE_ORACLE_WANT_COV) ? ((flags & OCHRE_ORACLE_SIGNED_COV) ? 2 : 1) : 0;
    int capture = (flags & OCHRE_ORACLE_CAPTURE_LINES) != 0;

    if (threads <= 1) {
        for (uint32_t ri = 0; ri < bt->n_rasters; ri++) run_raster(bt, off, ri, want_cov, capture, &outs[ri]);
    } else {
        pool_ctx pc;
        pc.bt = bt; pc.cmd_float_off = off; pc.outs = outs; pc.want_cov = want_cov; pc.capture = capture;
        atomic_init(&pc.next, 0u);
        pthread_t *th = (pthread_t *)malloc((size_t)threads * sizeof(pthread_t));
        int started = 0;
        for (int i = 0; th && i < threads; i++) {
            if (pthread_create(&th[i], NULL, worker, &pc) == 0) started++;
        }
        if (started == 0) worker(&pc);
        for (int i = 0; i < started; i++) pthread_join(th[i], NULL);
        free(th);
    }
    free(off);

    /* Concatenate per-raster outputs in raster order. */
    ochre_oracle_result *res = (ochre_oracle_result *)calloc(1, sizeof *res);
    if (!res) { st = OCHRE_ORACLE_E_NOMEM; goto cleanup; }
    res->n_rasters = bt->n_rasters;
    res->raster_tile_off = (uint64_t *)calloc(bt->n_rasters + 1, sizeof(uint64_t));
    res->raster_span_off = (uint64_t *)calloc(bt->n_rasters + 1, sizeof(uint64_t));
    res->raster_line_off = (uint64_t *)calloc(bt->n_rasters + 1, sizeof(uint64_t));
    res->raster_stats = (uint64_t *)calloc(3 * (size_t)bt->n_rasters + 1, sizeof(uint64_t));
    if (!res->raster_tile_off || !res->raster_span_off || !res->raster_line_off || !res->raster_stats) { st = OCHRE_ORACLE_E_NOMEM; goto cleanup; }
    uint64_t nt = 0, ns = 0, nl = 0;
    for (uint32_t ri = 0; ri < bt->n_rasters; ri++) {
        if (outs[ri].error && !st) { st = outs[ri].error; res->error_raster = ri; }
        res->raster_tile_off[ri] = nt; res->raster_span_off[ri] = ns; res->raster_line_off[ri] = nl;
        nt += outs[ri].c.n_tiles; ns += outs[ri].c.n_spans; nl += outs[ri].n_cap_lines;
        res->raster_stats[3 * ri] = outs[ri].n_lines;
        res->raster_stats[3 * ri + 1] = outs[ri].n_inc;
        res->raster_stats[3 * ri + 2] = outs[ri].n_tinc;
    }
    res->raster_tile_off[bt->n_rasters] = nt;
    res->raster_span_off[bt->n_rasters] = ns;
    res->raster_line_off[bt->n_rasters] = nl;
    res->n_tiles = nt; res->n_spans = ns; res->n_lines = nl;
    res->tile_xy = (int16_t *)malloc((nt ? nt : 1) * 2 * sizeof(int16_t));
    res->tile_alpha = (uint8_t *)malloc((nt ? nt : 1) * 64);
    res->tile_cov = want_cov ? (float *)malloc((nt ? nt : 1) * 64 * sizeof(float)) : NULL;
    res->span_xy = (int16_t *)malloc((ns ? ns : 1) * 2 * sizeof(int16_t));
    res->span_w = (uint16_t *)malloc((ns ? ns : 1) * sizeof(uint16_t));
    res->span_tile = (uint32_t *)malloc((ns ? ns : 1) * sizeof(uint32_t));
    res->lines = capture ? (float *)malloc((nl ? nl : 1) * 4 * sizeof(float)) : NULL;
    res->line_ninc = capture ? (uint32_t *)malloc((nl ? nl : 1) * sizeof(uint32_t)) : NULL;
    if (!res->tile_xy || !res->tile_alpha || (want_cov && !res->tile_cov) || !res->span_xy || !res->span_w ||
        !res->span_tile || (capture && (!res->lines || !res->line_ninc))) { st = OCHRE_ORACLE_E_NOMEM; goto cleanup; }
    for (uint32_t ri = 0; ri < bt->n_rasters; ri++) {
        collector *c = &outs[ri].c;
        uint64_t t0 = res->raster_tile_off[ri], s0 = res->raster_span_off[ri], l0 = res->raster_line_off[ri];
        if (c->n_tiles) {
            memcpy(res->tile_xy + 2 * t0, c->tile_xy, c->n_tiles * 2 * sizeof(int16_t));
            memcpy(res->tile_alpha + 64 * t0, c->tile_alpha, c->n_tiles * 64);
            if (want_cov) memcpy(res->tile_cov + 64 * t0, c->tile_cov, c->n_tiles * 64 * sizeof(float));
        }
        for (size_t s = 0; s < c->n_spans; s++) {
            res->span_xy[2 * (s0 + s)] = c->span_xy[2 * s];
            res->span_xy[2 * (s0 + s) + 1] = c->span_xy[2 * s + 1];
            res->span_w[s0 + s] = c->span_w[s];
            res->span_tile[s0 + s] = (uint32_t)(t0 + c->span_tile[s]);
        }
        if (capture && outs[ri].n_cap_lines) {
            memcpy(res->lines + 4 * l0, outs[ri].lines, outs[ri].n_cap_lines * 4 * sizeof(float));
            memcpy(res->line_ninc + l0, outs[ri].line_ninc, outs[ri].n_cap_lines * sizeof(uint32_t));
        }
    }
cleanup:
    for (uint32_t ri = 0; ri < bt->n_rasters; ri++) {
        free(outs[ri].c.tile_xy); free(outs[ri].c.tile_alpha); free(outs[ri].c.tile_cov);
        free(outs[ri].c.span_xy); free(outs[ri].c.span_w); free(outs[ri].c.span_tile);
        free(outs[ri].lines); free(outs[ri].line_ninc);
    }
    free(outs);
    if (st && st != OCHRE_ORACLE_E_LIMIT && res) { ochre_oracle_free(res); res = NULL; }
    *res_out = res;
    return st;
}

void ochre_oracle_free(ochre_oracle_result *r) {
    if (!r) return;
    free(r->tile_xy); free(r->tile_alpha); free(r->tile_cov);
    free(r->span_xy); free(r->span_w); free(r->span_tile);
    free(r->raster_tile_off); free(r->raster_span_off); free(r->raster_line_off); free(r->raster_stats);
    free(r->lines); free(r->line_ninc);
    free(r);
}


/* ------------------------------------------------------------------ */
/* FP64 analytic coverage of the f32 lines                             */
/* ------------------------------------------------------------------ */
/* For each raster: the same f32 line segments the reference rasterizes
 * (line_to calls, captured by ochre_oracle_run), clipped exactly against the
 * pixel grid in double precision.  Each piece inside cell (cx, cy) adds
 * area = 0.5*h*((cx+1-p0.x)+(cx+1-p1.x)) and height h = p1.y - p0.y, the
 * quantities rasterizer.rs:102-104 computes in f32 from the DDA's serial
 * crossing parameters; here every crossing parameter is computed directly.
 * Coverage before quantisation is |sum of heights left of the pixel on its
 * row + area of the pixel| (rasterizer.rs:232-239), written for the pixels
 * of the rectangle [x0, x0+w) x [y0, y0+h); heights of pieces left of the
 * rectangle are carried in. */
static int cmp_double(const void *a, const void *b) {
    double x = *(const double *)a, y = *(const double *)b;
    return x < y ? -1 : x > y;
}

int ochre_oracle_cov64(const float *lines, const uint64_t *raster_line_off, uint32_t n_rasters,
                       const int32_t *rect /* 4 per raster: x0 y0 w h */, double *out) {
    size_t base = 0;
    for (uint32_t r = 0; r < n_rasters; r++) {
        const int x0 = rect[4 * r], y0 = rect[4 * r + 1], w = rect[4 * r + 2], h = rect[4 * r + 3];
        double *img = out + base;
        size_t npx = (size_t)w * (size_t)h;
        double *hsum = (double *)calloc(npx ? npx : 1, sizeof(double));
        double *left = (double *)calloc(h ? (size_t)h : 1, sizeof(double));
        if (!hsum || !left) { free(hsum); free(left); return OCHRE_ORACLE_E_NOMEM; }
        for (size_t i = 0; i < npx; i++) img[i] = 0.0;
        for (uint64_t l = raster_line_off[r]; l < raster_line_off[r + 1]; l++) {
            const double ax = lines[4 * l], ay = lines[4 * l + 1], bx = lines[4 * l + 2], by = lines[4 * l + 3];
            if (ax == bx && ay == by) continue;
            const double dx = bx - ax, dy = by - ay;
            /* crossing parameters with every integer x and y between the ends */
            long fx0 = (long)floor(fmin(ax, bx)), fx1 = (long)floor(fmax(ax, bx));
            long fy0 = (long)floor(fmin(ay, by)), fy1 = (long)floor(fmax(ay, by));
            size_t cap = (size_t)(fx1 - fx0 + fy1 - fy0 + 4);
            double *ts = (double *)malloc(cap * sizeof(double));
            if (!ts) { free(hsum); free(left); return OCHRE_ORACLE_E_NOMEM; }
            size_t nt = 0;
            ts[nt++] = 0.0;
            if (dx != 0.0)
                for (long k = fx0 + 1; k <= fx1; k++) {
                    double t = ((double)k - ax) / dx;
                    if (t > 0.0 && t < 1.0) ts[nt++] = t;
                }
            if (dy != 0.0)
                for (long k = fy0 + 1; k <= fy1; k++) {
                    double t = ((double)k - ay) / dy;
                    if (t > 0.0 && t < 1.0) ts[nt++] = t;
                }
            ts[nt++] = 1.0;
            qsort(ts, nt, sizeof(double), cmp_double);
            for (size_t i = 0; i + 1 < nt; i++) {
                const double t0 = ts[i], t1 = ts[i + 1];
                if (t1 <= t0) continue;
                const double tm = 0.5 * (t0 + t1);
                const long cx = (long)floor(ax + tm * dx), cy = (long)floor(ay + tm * dy);
                const double p0x = ax + t0 * dx, p0y = ay + t0 * dy, p1x = ax + t1 * dx, p1y = ay + t1 * dy;
                const double hh = p1y - p0y;
                const double right = (double)(cx + 1);
                const double aa = 0.5 * hh * ((right - p0x) + (right - p1x));
                const long py = cy - y0, px = cx - x0;
                if (py < 0 || py >= h) continue;
                if (px < 0) { left[py] += hh; continue; }
                if (px >= w) continue;
                img[(size_t)py * w + px] += aa;
                hsum[(size_t)py * w + px] += hh;
            }
            free(ts);
        }
        for (int y = 0; y < h; y++) {
            double acc = left[y];
            for (int x = 0; x < w; x++) {
                double v = acc + img[(size_t)y * w + x];
                acc += hsum[(size_t)y * w + x];
                img[(size_t)y * w + x] = fabs(v);
            }
        }
        free(hsum);
        free(left);
        base += npx;
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* Differentiable model in double precision                           */
/* ------------------------------------------------------------------ */
/* The model of ochre_gb300's differentiable fill, restated in double:
 * coverage c = min(|S|, 1) on a w x h canvas per raster, S from the exact
 * clipping of the path's edges (as ochre_oracle_cov64), loss = sum (c - t)^2.
 * The discrete structure is held fixed: every curve keeps the number of
 * lines the f32 flattening gives it (path.rs:52-57, 65-73), with parameters
 * t_j = min(j dt, 1) (t_n = 1); closing lines (rasterizer.rs:62-64,
 * 181-183) are always present, zero-length when the contour is closed. */
typedef struct { double x, y; } dv2;
typedef struct { dv2 a, b; } dedge;
typedef struct { int64_t cmd; int pt; } pref;   /* a device-space point: command, point index; cmd < 0: constant */

static dv2 dxf_apply(const float *xf, dv2 v) {
    dv2 r = {(double)xf[0] * v.x + (double)xf[1] * v.y + (double)xf[4],
             (double)xf[2] * v.x + (double)xf[3] * v.y + (double)xf[5]};
    return r;
}
static int npts_of(uint8_t v) { return v == 0 || v == 1 ? 1 : v == 2 || v == 4 ? 2 : v == 3 ? 3 : 0; }
static int endpt_of(uint8_t v) { return v == 3 ? 2 : (v == 2 || v == 4) ? 1 : 0; }

int ochre_oracle_seg_counts(const ochre_oracle_batch *bt, uint32_t *counts) {
    uint64_t *off = NULL;
    int st = validate(bt, &off);
    if (st) return st;
    for (uint32_t ri = 0; ri < bt->n_rasters; ri++) {
        uint32_t f0 = bt->raster_fill_off ? bt->raster_fill_off[ri] : ri;
        uint32_t f1 = bt->raster_fill_off ? bt->raster_fill_off[ri + 1] : ri + 1;
        vec2 last = v2(0.0f, 0.0f);
        for (uint32_t f = f0; f < f1; f++) {
            const float *xf = bt->fill_xf + 6 * (size_t)f;
            int raw = bt->fill_flags ? (bt->fill_flags[f] & 1) : 0;
            for (uint32_t c = bt->fill_cmd_off[f]; c < bt->fill_cmd_off[f + 1]; c++) {
                uint8_t verb = bt->verbs[c];
                const float *fp = bt->pts + off[c];
                vec2 p[3];
                for (int k = 0; k < npts_of(verb); k++) {
                    p[k] = v2(fp[2 * k], fp[2 * k + 1]);
                    if (!raw) p[k] = xf_apply(xf, p[k]);
                }
                uint32_t n = 0;
                if (verb == 2 || verb == 3) {
                    float dt;
                    if (verb == 2) {
                        dt = sqrtf((4.0f * TOLERANCE) / vlength(vadd(vsub(last, vscale(2.0f, p[0])), p[1])));
                    } else {
                        vec2 a = vadd(vsub(vadd(vscale(-1.0f, last), vscale(3.0f, p[0])), vscale(3.0f, p[1])), p[2]);
                        vec2 b = vscale(3.0f, vadd(vsub(last, vscale(2.0f, p[0])), p[1]));
                        float conc = rmax(vlength(b), vlength(vadd(a, b)));
                        dt = sqrtf((sqrtf(8.0f) * TOLERANCE) / conc);
                    }
                    float t = 0.0f;
                    while (t < 1.0f && n < FLATTEN_CAP) { t = rmin(t + dt, 1.0f); n++; }
                }
                counts[c] = n;
                if (verb <= 4) last = p[endpt_of(verb)];
            }
        }
    }
    free(off);
    return 0;
}

/* exact clipping of one edge; calls piece(cx, cy, p0, p1, kind0, kind1, bnd0, bnd1)
 * where kind = 0 endpoint, 1 vertical boundary x = bnd, 2 horizontal y = bnd */
typedef void (*piece_fn)(void *u, long cx, long cy, dv2 p0, dv2 p1, int k0, double b0, int k1, double b1);

typedef struct { double t; int kind; double bnd; } tcross;

/* Pieces of the edge A -> B, one per pixel cell on its way, each with the
 * kinds of its two ends (start, end, or the pixel boundary crossed), in
 * exact arithmetic.  The cell sequence is that of the reference's walk
 * (rasterizer.rs:72-121) without rounding: it starts in floor(A), a crossing
 * of a vertical boundary moves one column, of a horizontal one one row,
 * simultaneous crossings take the column first (the walk's tie rule), and a
 * crossing exactly at B still moves into floor(B).  Pieces may have zero
 * length (an end point on a boundary, or a pass through a pixel corner). */
static int cmp_tcross_kind(const void *a, const void *b) {
    const tcross *x = (const tcross *)a, *y = (const tcross *)b;
    if (x->t != y->t) return x->t < y->t ? -1 : 1;
    return x->kind - y->kind;   /* vertical (1) before horizontal (2) */
}

static int clip_edge(dv2 A, dv2 B, piece_fn fn, void *u) {
    const double dx = B.x - A.x, dy = B.y - A.y;
    const long ax = (long)floor(A.x), ay = (long)floor(A.y), bx = (long)floor(B.x), by = (long)floor(B.y);
    const size_t cap = (size_t)(labs(bx - ax) + labs(by - ay) + 2);
    tcross *ts = (tcross *)malloc(cap * sizeof(tcross));
    if (!ts) return OCHRE_ORACLE_E_NOMEM;
    size_t n = 0;
    if (dx > 0.0)
        for (long k = ax + 1; k <= bx; k++) { ts[n].t = ((double)k - A.x) / dx; ts[n].kind = 1; ts[n].bnd = (double)k; n++; }
    else if (dx < 0.0)
        for (long k = ax; k > bx; k--) { ts[n].t = ((double)k - A.x) / dx; ts[n].kind = 1; ts[n].bnd = (double)k; n++; }
    if (dy > 0.0)
        for (long k = ay + 1; k <= by; k++) { ts[n].t = ((double)k - A.y) / dy; ts[n].kind = 2; ts[n].bnd = (double)k; n++; }
    else if (dy < 0.0)
        for (long k = ay; k > by; k--) { ts[n].t = ((double)k - A.y) / dy; ts[n].kind = 2; ts[n].bnd = (double)k; n++; }
    qsort(ts, n, sizeof(tcross), cmp_tcross_kind);
    long cx = ax, cy = ay;
    dv2 p0 = A;
    int k0 = 0;
    double b0 = 0.0;
    for (size_t i = 0; i <= n; i++) {
        dv2 p1 = B;
        int k1 = 0;
        double b1 = 0.0;
        if (i < n) {
            const double t = ts[i].t;
            p1.x = A.x + t * dx;
            p1.y = A.y + t * dy;
            k1 = ts[i].kind;
            b1 = ts[i].bnd;
            if (k1 == 1) p1.x = b1; else p1.y = b1;
        }
        fn(u, cx, cy, p0, p1, k0, b0, k1, b1);
        if (i < n) {
            if (k1 == 1) cx += dx > 0.0 ? 1 : -1;
            else cy += dy > 0.0 ? 1 : -1;
        }
        p0 = p1;
        k0 = k1;
        b0 = b1;
    }
    free(ts);
    return 0;
}

typedef struct {
    int W, H;
    double *area, *hgt, *left;   /* forward accumulation */
    const double *g, *G, *gleft; /* backward: dL/dS, suffix sums, row totals */
    dv2 A, B;                    /* current edge */
    dv2 dA, dB;
} diffctx;

static void fwd_piece(void *u, long cx, long cy, dv2 p0, dv2 p1, int k0, double b0, int k1, double b1) {
    (void)k0; (void)b0; (void)k1; (void)b1;
    diffctx *d = (diffctx *)u;
    if (cy < 0 || cy >= d->H) return;
    const double h = p1.y - p0.y;
    if (cx < 0) { d->left[cy] += h; return; }
    if (cx >= d->W) return;
    const double right = (double)(cx + 1);
    d->area[(size_t)cy * d->W + cx] += 0.5 * h * ((right - p0.x) + (right - p1.x));
    d->hgt[(size_t)cy * d->W + cx] += h;
}

static void lookup(const diffctx *d, long cx, long cy, double *g, double *G) {
    *g = 0.0; *G = 0.0;
    if (cy < 0 || cy >= d->H) return;
    if (cx < 0) { *G = d->gleft[cy]; return; }
    if (cx >= d->W) return;
    *g = d->g[(size_t)cy * d->W + cx];
    *G = d->G[(size_t)cy * d->W + cx];
}

/* dL/d(A, B) of a point on the edge given by its kind (see clip_edge) */
static void chain_point(diffctx *d, int kind, double bnd, int is_end, double gx, double gy) {
    const dv2 A = d->A, B = d->B;
    const double D = B.x - A.x, E = B.y - A.y;
    if (kind == 0) {
        if (is_end) { d->dB.x += gx; d->dB.y += gy; }
        else { d->dA.x += gx; d->dA.y += gy; }
    } else if (kind == 1) {
        const double s = (bnd - A.x) / D;
        d->dA.y += gy * (1.0 - s);
        d->dB.y += gy * s;
        d->dA.x += gy * E * (s - 1.0) / D;
        d->dB.x += gy * (-E * s / D);
    } else {
        const double u = (bnd - A.y) / E;
        d->dA.x += gx * (1.0 - u);
        d->dB.x += gx * u;
        d->dA.y += gx * D * (u - 1.0) / E;
        d->dB.y += gx * (-D * u / E);
    }
}

static void bwd_piece(void *u, long cx, long cy, dv2 p0, dv2 p1, int k0, double b0, int k1, double b1) {
    diffctx *d = (diffctx *)u;
    double g, G;
    lookup(d, cx, cy, &g, &G);
    if (g == 0.0 && G == 0.0) return;
    const double h = p1.y - p0.y;
    const double right = (double)(cx + 1);
    const double m = 0.5 * ((right - p0.x) + (right - p1.x));
    chain_point(d, k0, b0, 0, -0.5 * h * g, -m * g - G);
    chain_point(d, k1, b1, 1, -0.5 * h * g, m * g + G);
}

/* Edges of one raster in the model, with the points they depend on. */
typedef struct {
    dedge *e; size_t n, cap;
    pref *ra, *rb;          /* per edge: point refs of A and B when they are plain points (closing lines, lines) */
    double *tb;             /* per edge: conic parameter of B (conic edges), else -1 */
} edges_t;

/* Parameters t of the points a conic's subdivision emits, in order (path.rs:75-104
 * in f32 as the forward runs it: the midpoint of every leaf, then its end). */
typedef struct { double *t; size_t n, cap; int error; } tlist;
static void tl_push(tlist *l, double t) {
    if (l->n == l->cap) {
        size_t c = l->cap ? 2 * l->cap : 64;
        double *p = (double *)realloc(l->t, c * sizeof(double));
        if (!p) { l->error = OCHRE_ORACLE_E_NOMEM; return; }
        l->t = p; l->cap = c;
    }
    l->t[l->n++] = t;
}
static void conic_params(tlist *l, vec2 last, vec2 control, vec2 point, float weight, float t0, float t1, vec2 p0,
                         vec2 p1, int depth) {
    float t = 0.5f * (t0 + t1);
    vec2 wc = vscale(weight, control);
    vec2 p01 = vlerp(t, last, wc);
    vec2 p12 = vlerp(t, wc, point);
    float denom = (1.0f - t) * (1.0f - t) + 2.0f * t * (1.0f - t) * weight + t * t;
    vec2 midpoint = vscale(1.0f / denom, vlerp(t, p01, p12));
    float err = vlength(vsub(midpoint, vscale(0.5f, vadd(p0, p1))));
    if (err > TOLERANCE) {
        if (depth >= CONIC_DEPTH_CAP) { l->error = OCHRE_ORACLE_E_LIMIT; return; }
        conic_params(l, last, control, point, weight, t0, t, p0, midpoint, depth + 1);
        conic_params(l, last, control, point, weight, t, t1, midpoint, p1, depth + 1);
    } else {
        tl_push(l, t);
        tl_push(l, t1);
    }
}

static int push_edge_t(edges_t *E, dv2 a, dv2 b, pref ra, pref rb, double tb) {
    if (E->n == E->cap) {
        size_t c = E->cap ? E->cap * 2 : 256;
        dedge *p = (dedge *)realloc(E->e, c * sizeof(dedge));
        pref *qa = (pref *)realloc(E->ra, c * sizeof(pref));
        pref *qb = (pref *)realloc(E->rb, c * sizeof(pref));
        double *qt = (double *)realloc(E->tb, c * sizeof(double));
        if (p) E->e = p;
        if (qa) E->ra = qa;
        if (qb) E->rb = qb;
        if (qt) E->tb = qt;
        if (!p || !qa || !qb || !qt) return OCHRE_ORACLE_E_NOMEM;
        E->cap = c;
    }
    E->e[E->n].a = a; E->e[E->n].b = b;
    E->ra[E->n] = ra; E->rb[E->n] = rb;
    E->tb[E->n] = tb;
    E->n++;
    return 0;
}
static int push_edge(edges_t *E, dv2 a, dv2 b, pref ra, pref rb) { return push_edge_t(E, a, b, ra, rb, -1.0); }

static int diff64_impl(const ochre_oracle_batch *bt, const uint32_t *counts, int W, int H, const double *target,
                       const double *dl_ds, double *loss_out, double *dpts, double *dxf, double *s_out) {
    uint64_t *off = NULL;
    int st = validate(bt, &off);
    if (st) return st;
    const size_t npx = (size_t)W * (size_t)H;
    double *area = (double *)malloc(npx * sizeof(double));
    double *hgt = (double *)malloc(npx * sizeof(double));
    double *gimg = (double *)malloc(npx * sizeof(double));
    double *Gimg = (double *)malloc(npx * sizeof(double));
    double *left = (double *)malloc((size_t)H * sizeof(double));
    double *gleft = (double *)malloc((size_t)H * sizeof(double));
    double *dp = (double *)calloc(bt->n_floats ? bt->n_floats : 1, sizeof(double));   /* device-space point grads */
    if (!area || !hgt || !gimg || !Gimg || !left || !gleft || !dp) { st = OCHRE_ORACLE_E_NOMEM; goto done; }
    if (dpts) for (uint64_t i = 0; i < bt->n_floats; i++) dpts[i] = 0.0;
    if (dxf) for (uint32_t i = 0; i < 6 * bt->n_fills; i++) dxf[i] = 0.0;
    double loss = 0.0;
    for (uint32_t ri = 0; ri < bt->n_rasters && !st; ri++) {
        uint32_t f0 = bt->raster_fill_off ? bt->raster_fill_off[ri] : ri;
        uint32_t f1 = bt->raster_fill_off ? bt->raster_fill_off[ri + 1] : ri + 1;
        edges_t E = {0};
        /* per command: first own edge, own edge count */
        uint64_t c0 = bt->fill_cmd_off[f0], c1 = bt->fill_cmd_off[f1];
        size_t ncmd = (size_t)(c1 - c0);
        size_t *e_first = (size_t *)malloc((ncmd + 1) * sizeof(size_t));
        dv2 *cpts = (dv2 *)malloc((ncmd ? ncmd : 1) * 3 * sizeof(dv2));
        if (!e_first || !cpts) { free(e_first); free(cpts); st = OCHRE_ORACLE_E_NOMEM; break; }
        dv2 last = {0.0, 0.0}, first = {0.0, 0.0};
        vec2 last32 = v2(0.0f, 0.0f);   /* the f32 forward's last point (conic subdivision) */
        pref last_ref = {-1, 0}, first_ref = {-1, 0};
        /* ---- edges ---- */
        for (uint32_t f = f0; f < f1 && !st; f++) {
            const float *xf = bt->fill_xf + 6 * (size_t)f;
            int raw = bt->fill_flags ? (bt->fill_flags[f] & 1) : 0;
            for (uint64_t c = bt->fill_cmd_off[f]; c < bt->fill_cmd_off[f + 1]; c++) {
                const size_t li = (size_t)(c - c0);
                uint8_t verb = bt->verbs[c];
                const float *fp = bt->pts + off[c];
                dv2 *p = cpts + 3 * li;
                vec2 p32[3];
                for (int k = 0; k < npts_of(verb); k++) {
                    dv2 v = {fp[2 * k], fp[2 * k + 1]};
                    p[k] = raw ? v : dxf_apply(xf, v);
                    p32[k] = raw ? v2(fp[2 * k], fp[2 * k + 1]) : xf_apply(xf, v2(fp[2 * k], fp[2 * k + 1]));
                }
                e_first[li] = E.n;
                pref self0 = {(int64_t)c, 0}, none = {-1, 0};
                if (verb == 0) {
                    st = push_edge(&E, last, first, last_ref, first_ref);
                    first = p[0]; last = p[0];
                    first_ref = self0; last_ref = self0;
                    last32 = p32[0];
                } else if (verb == 1) {
                    st = push_edge(&E, last, p[0], last_ref, self0);
                    last = p[0]; last_ref = self0;
                    last32 = p32[0];
                } else if (verb == 2 || verb == 3) {
                    const uint32_t n = counts[c];
                    double dt;
                    if (verb == 2) {
                        dv2 v = {last.x - 2.0 * p[0].x + p[1].x, last.y - 2.0 * p[0].y + p[1].y};
                        dt = sqrt(0.4 / sqrt(v.x * v.x + v.y * v.y));
                    } else {
                        dv2 b = {3.0 * (last.x - 2.0 * p[0].x + p[1].x), 3.0 * (last.y - 2.0 * p[0].y + p[1].y)};
                        dv2 ab = {2.0 * last.x - 3.0 * p[0].x + p[2].x, 2.0 * last.y - 3.0 * p[0].y + p[2].y};
                        double conc = fmax(sqrt(b.x * b.x + b.y * b.y), sqrt(ab.x * ab.x + ab.y * ab.y));
                        dt = sqrt(sqrt(8.0) * 0.1 / conc);
                    }
                    dv2 prev = last;
                    for (uint32_t j = 1; j <= n && !st; j++) {
                        double t = j == n ? 1.0 : fmin((double)j * dt, 1.0), u = 1.0 - t;
                        dv2 q;
                        if (verb == 2) {
                            q.x = u * u * last.x + 2.0 * u * t * p[0].x + t * t * p[1].x;
                            q.y = u * u * last.y + 2.0 * u * t * p[0].y + t * t * p[1].y;
                        } else {
                            q.x = u * u * u * last.x + 3.0 * u * u * t * p[0].x + 3.0 * u * t * t * p[1].x + t * t * t * p[2].x;
                            q.y = u * u * u * last.y + 3.0 * u * u * t * p[0].y + 3.0 * u * t * t * p[1].y + t * t * t * p[2].y;
                        }
                        st = push_edge(&E, prev, q, none, none);
                        prev = q;
                    }
                    last = p[verb == 2 ? 1 : 2];
                    last_ref.cmd = (int64_t)c; last_ref.pt = verb == 2 ? 1 : 2;
                    last32 = p32[verb == 2 ? 1 : 2];
                } else if (verb == 4) {
                    /* the conic at the f32 subdivision's parameters, in double */
                    const double w = fp[4];
                    tlist tl = {0};
                    conic_params(&tl, last32, p32[0], p32[1], fp[4], 0.0f, 1.0f, last32, p32[1], 0);
                    if (tl.error) st = tl.error;
                    dv2 prev = last;
                    for (size_t j = 0; j < tl.n && !st; j++) {
                        const double t = tl.t[j], u = 1.0 - t;
                        const double D = u * u + 2.0 * t * u * w + t * t;
                        dv2 q = {(u * u * last.x + 2.0 * t * u * w * p[0].x + t * t * p[1].x) / D,
                                 (u * u * last.y + 2.0 * t * u * w * p[0].y + t * t * p[1].y) / D};
                        st = push_edge_t(&E, prev, q, none, none, t);
                        prev = q;
                    }
                    free(tl.t);
                    last = p[1];
                    last_ref.cmd = (int64_t)c; last_ref.pt = 1;
                    last32 = p32[1];
                }
            }
        }
        e_first[ncmd] = E.n;
        if (!st) st = push_edge(&E, last, first, last_ref, first_ref);   /* finish's closing line */
        /* ---- forward ---- */
        diffctx d;
        memset(&d, 0, sizeof d);
        d.W = W; d.H = H; d.area = area; d.hgt = hgt; d.left = left;
        for (size_t i = 0; i < npx; i++) { area[i] = 0.0; hgt[i] = 0.0; }
        for (int y = 0; y < H; y++) left[y] = 0.0;
        for (size_t e = 0; e < E.n && !st; e++)
            if (!(E.e[e].a.x == E.e[e].b.x && E.e[e].a.y == E.e[e].b.y)) st = clip_edge(E.e[e].a, E.e[e].b, fwd_piece, &d);
        const double *tgt = target ? target + (size_t)ri * npx : NULL;
        for (int y = 0; y < H && !tgt; y++)
            for (int x = 0; x < W; x++) gimg[(size_t)y * W + x] = dl_ds[(size_t)ri * npx + (size_t)y * W + x];
        for (int y = 0; y < H && tgt; y++) {
            double acc = left[y];
            for (int x = 0; x < W; x++) {
                const size_t i = (size_t)y * W + x;
                const double S = acc + area[i];
                acc += hgt[i];
                if (s_out) s_out[(size_t)ri * npx + i] = S;
                const double c = fmin(fabs(S), 1.0);
                loss += (c - tgt[i]) * (c - tgt[i]);
                const double gc = 2.0 * (c - tgt[i]);
                gimg[i] = fabs(S) < 1.0 ? (S > 0.0 ? gc : S < 0.0 ? -gc : 0.0) : 0.0;
            }
        }
        if (dpts || dxf) {
            /* suffix sums of dL/dS to the right of each pixel, and row totals */
            for (int y = 0; y < H; y++) {
                double s = 0.0;
                for (int x = W - 1; x >= 0; x--) {
                    Gimg[(size_t)y * W + x] = s;
                    s += gimg[(size_t)y * W + x];
                }
                gleft[y] = s;
            }
            d.g = gimg; d.G = Gimg; d.gleft = gleft;
            dv2 *gA = (dv2 *)calloc(E.n ? E.n : 1, sizeof(dv2));
            dv2 *gB = (dv2 *)calloc(E.n ? E.n : 1, sizeof(dv2));
            if (!gA || !gB) { free(gA); free(gB); st = OCHRE_ORACLE_E_NOMEM; }
            for (size_t e = 0; e < E.n && !st; e++) {
                d.A = E.e[e].a; d.B = E.e[e].b;
                d.dA.x = d.dA.y = d.dB.x = d.dB.y = 0.0;
                if (d.A.x == d.B.x && d.A.y == d.B.y) {
                    double g, G;
                    const long cx = (long)floor(d.B.x), cy = (long)floor(d.B.y);
                    lookup(&d, cx, cy, &g, &G);
                    const double dy = ((double)(cx + 1) - d.B.x) * g + G;
                    d.dA.y = -dy; d.dB.y = dy;
                } else {
                    st = clip_edge(d.A, d.B, bwd_piece, &d);
                }
                gA[e] = d.dA; gB[e] = d.dB;
            }
            /* flatten adjoint: edge end points back to device-space points */
#define ADDP(ref, vx, vy) do { if ((ref).cmd >= 0) { dp[off[(ref).cmd] + 2 * (ref).pt] += (vx); dp[off[(ref).cmd] + 2 * (ref).pt + 1] += (vy); } } while (0)
            last_ref.cmd = -1; first_ref.cmd = -1;
            dv2 lastp = {0.0, 0.0};
            for (size_t li = 0; li < ncmd && !st; li++) {
                const uint64_t c = c0 + li;
                const uint8_t verb = bt->verbs[c];
                const size_t e0 = e_first[li], e1 = e_first[li + 1];
                const dv2 *p = cpts + 3 * li;
                pref self0 = {(int64_t)c, 0};
                if (verb == 0) {
                    ADDP(E.ra[e0], gA[e0].x, gA[e0].y);
                    ADDP(E.rb[e0], gB[e0].x, gB[e0].y);
                    first_ref = self0; last_ref = self0; lastp = p[0];
                } else if (verb == 1) {
                    ADDP(E.ra[e0], gA[e0].x, gA[e0].y);
                    ADDP(E.rb[e0], gB[e0].x, gB[e0].y);
                    last_ref = self0; lastp = p[0];
                } else if (verb == 2 || verb == 3) {
                    const int cubic = verb == 3;
                    const size_t n = e1 - e0;
                    const dv2 P0 = lastp, P1 = p[0], P2 = p[1], P3 = cubic ? p[2] : p[1];
                    double dt, S = 0.0;
                    dv2 g[4] = {{gA[e0].x, gA[e0].y}, {0, 0}, {0, 0}, {0, 0}};
                    if (!cubic) {
                        dv2 v = {P0.x - 2.0 * P1.x + P2.x, P0.y - 2.0 * P1.y + P2.y};
                        dt = sqrt(0.4 / sqrt(v.x * v.x + v.y * v.y));
                    } else {
                        dv2 b = {3.0 * (P0.x - 2.0 * P1.x + P2.x), 3.0 * (P0.y - 2.0 * P1.y + P2.y)};
                        dv2 ab = {2.0 * P0.x - 3.0 * P1.x + P3.x, 2.0 * P0.y - 3.0 * P1.y + P3.y};
                        dt = sqrt(sqrt(8.0) * 0.1 / fmax(sqrt(b.x * b.x + b.y * b.y), sqrt(ab.x * ab.x + ab.y * ab.y)));
                    }
                    for (size_t j = 1; j <= n; j++) {
                        const double t = j == n ? 1.0 : fmin((double)j * dt, 1.0), u = 1.0 - t;
                        dv2 dq = gB[e0 + j - 1];
                        if (j < n) { dq.x += gA[e0 + j].x; dq.y += gA[e0 + j].y; }
                        dv2 dc;
                        if (cubic) {
                            const double b0 = u * u * u, b1 = 3 * u * u * t, b2 = 3 * u * t * t, b3 = t * t * t;
                            g[0].x += b0 * dq.x; g[0].y += b0 * dq.y; g[1].x += b1 * dq.x; g[1].y += b1 * dq.y;
                            g[2].x += b2 * dq.x; g[2].y += b2 * dq.y; g[3].x += b3 * dq.x; g[3].y += b3 * dq.y;
                            dc.x = 3 * u * u * (P1.x - P0.x) + 6 * u * t * (P2.x - P1.x) + 3 * t * t * (P3.x - P2.x);
                            dc.y = 3 * u * u * (P1.y - P0.y) + 6 * u * t * (P2.y - P1.y) + 3 * t * t * (P3.y - P2.y);
                        } else {
                            const double b0 = u * u, b1 = 2 * u * t, b2 = t * t;
                            g[0].x += b0 * dq.x; g[0].y += b0 * dq.y; g[1].x += b1 * dq.x; g[1].y += b1 * dq.y;
                            g[2].x += b2 * dq.x; g[2].y += b2 * dq.y;
                            dc.x = 2 * u * (P1.x - P0.x) + 2 * t * (P2.x - P1.x);
                            dc.y = 2 * u * (P1.y - P0.y) + 2 * t * (P2.y - P1.y);
                        }
                        if (j < n && (double)j * dt < 1.0) S += (double)j * (dc.x * dq.x + dc.y * dq.y);
                    }
                    if (S != 0.0 && isfinite(dt)) {
                        if (cubic) {
                            dv2 b = {3.0 * (P0.x - 2.0 * P1.x + P2.x), 3.0 * (P0.y - 2.0 * P1.y + P2.y)};
                            dv2 ab = {2.0 * P0.x - 3.0 * P1.x + P3.x, 2.0 * P0.y - 3.0 * P1.y + P3.y};
                            const double lb = sqrt(b.x * b.x + b.y * b.y), lab = sqrt(ab.x * ab.x + ab.y * ab.y);
                            const double conc = fmax(lb, lab), k1 = S * (-0.5 * dt / conc);
                            if (lb >= lab && lb > 0.0) {
                                const dv2 u1 = {k1 * b.x / lb, k1 * b.y / lb};
                                g[0].x += 3 * u1.x; g[0].y += 3 * u1.y; g[1].x -= 6 * u1.x; g[1].y -= 6 * u1.y;
                                g[2].x += 3 * u1.x; g[2].y += 3 * u1.y;
                            } else if (lab > 0.0) {
                                const dv2 u1 = {k1 * ab.x / lab, k1 * ab.y / lab};
                                g[0].x += 2 * u1.x; g[0].y += 2 * u1.y; g[1].x -= 3 * u1.x; g[1].y -= 3 * u1.y;
                                g[3].x += u1.x; g[3].y += u1.y;
                            }
                        } else {
                            const dv2 v = {P0.x - 2.0 * P1.x + P2.x, P0.y - 2.0 * P1.y + P2.y};
                            const double len2 = v.x * v.x + v.y * v.y;
                            if (len2 > 0.0) {
                                const double k1 = S * (-0.5 * dt / len2);
                                g[0].x += k1 * v.x; g[0].y += k1 * v.y; g[1].x -= 2 * k1 * v.x; g[1].y -= 2 * k1 * v.y;
                                g[2].x += k1 * v.x; g[2].y += k1 * v.y;
                            }
                        }
                    }
                    ADDP(last_ref, g[0].x, g[0].y);
                    pref r1 = {(int64_t)c, 0}, r2 = {(int64_t)c, 1}, r3 = {(int64_t)c, 2};
                    ADDP(r1, g[1].x, g[1].y);
                    ADDP(r2, g[2].x, g[2].y);
                    if (cubic) ADDP(r3, g[3].x, g[3].y);
                    last_ref.cmd = (int64_t)c; last_ref.pt = cubic ? 2 : 1; lastp = cubic ? p[2] : p[1];
                } else if (verb == 4) {
                    /* q_j = (u^2 P0 + 2tu w P1 + t^2 P2) / D at fixed t_j: linear in the
                     * points; dq/dw = 2tu (P1 - q) / D */
                    const size_t n = e1 - e0;
                    const dv2 P0 = lastp, P1 = p[0];
                    const double w = bt->pts[off[c] + 4];
                    dv2 g0 = gA[e0], g1 = {0, 0}, g2 = {0, 0};
                    double gw = 0.0;
                    for (size_t j = 1; j <= n; j++) {
                        const double t = E.tb[e0 + j - 1], u = 1.0 - t;
                        const double D = u * u + 2.0 * t * u * w + t * t;
                        const double A = u * u / D, B = 2.0 * t * u * w / D, C = t * t / D;
                        dv2 dq = gB[e0 + j - 1];
                        if (j < n) { dq.x += gA[e0 + j].x; dq.y += gA[e0 + j].y; }
                        g0.x += A * dq.x; g0.y += A * dq.y;
                        g1.x += B * dq.x; g1.y += B * dq.y;
                        g2.x += C * dq.x; g2.y += C * dq.y;
                        const dv2 q = E.e[e0 + j - 1].b;
                        gw += 2.0 * t * u / D * ((P1.x - q.x) * dq.x + (P1.y - q.y) * dq.y);
                    }
                    (void)P0;
                    ADDP(last_ref, g0.x, g0.y);
                    pref r1 = {(int64_t)c, 0}, r2 = {(int64_t)c, 1};
                    ADDP(r1, g1.x, g1.y);
                    ADDP(r2, g2.x, g2.y);
                    dp[off[c] + 4] += gw;   /* the weight, not transformed */
                    last_ref.cmd = (int64_t)c; last_ref.pt = 1; lastp = p[1];
                }
            }
            {
                const size_t e = E.n - 1;   /* finish's closing line */
                ADDP(E.ra[e], gA[e].x, gA[e].y);
                ADDP(E.rb[e], gB[e].x, gB[e].y);
            }
#undef ADDP
            free(gA); free(gB);
        }
        free(E.e); free(E.ra); free(E.rb); free(E.tb); free(e_first); free(cpts);
    }
    /* transform adjoint */
    if (!st && (dpts || dxf)) {
        for (uint32_t f = 0; f < bt->n_fills; f++) {
            const float *xf = bt->fill_xf + 6 * (size_t)f;
            int raw = bt->fill_flags ? (bt->fill_flags[f] & 1) : 0;
            for (uint64_t c = bt->fill_cmd_off[f]; c < bt->fill_cmd_off[f + 1]; c++) {
                const float *fp = bt->pts + off[c];
                for (int k = 0; k < npts_of(bt->verbs[c]); k++) {
                    const double gx = dp[off[c] + 2 * k], gy = dp[off[c] + 2 * k + 1];
                    const double vx = fp[2 * k], vy = fp[2 * k + 1];
                    if (dpts) {
                        if (raw) { dpts[off[c] + 2 * k] = gx; dpts[off[c] + 2 * k + 1] = gy; }
                        else {
                            dpts[off[c] + 2 * k] = xf[0] * gx + xf[2] * gy;
                            dpts[off[c] + 2 * k + 1] = xf[1] * gx + xf[3] * gy;
                        }
                    }
                    if (dxf && !raw) {
                        dxf[6 * f + 0] += gx * vx; dxf[6 * f + 1] += gx * vy;
                        dxf[6 * f + 2] += gy * vx; dxf[6 * f + 3] += gy * vy;
                        dxf[6 * f + 4] += gx; dxf[6 * f + 5] += gy;
                    }
                }
                if (dpts && bt->verbs[c] == 4) dpts[off[c] + 4] = dp[off[c] + 4];
            }
        }
    }
    *loss_out = 0.0;
    if (!st) *loss_out = loss;
done:
    free(area); free(hgt); free(gimg); free(Gimg); free(left); free(gleft); free(dp); free(off);
    return st;
}

int ochre_oracle_diff64(const ochre_oracle_batch *bt, const uint32_t *counts, int W, int H, const double *target,
                        double *loss_out, double *dpts, double *dxf) {
    return diff64_impl(bt, counts, W, H, target, NULL, loss_out, dpts, dxf, NULL);
}

int ochre_oracle_backward64(const ochre_oracle_batch *bt, const uint32_t *counts, int W, int H, const double *dl_ds,
                            double *dpts, double *dxf) {
    double loss;
    return diff64_impl(bt, counts, W, H, NULL, dl_ds, &loss, dpts, dxf, NULL);
}

/* The FP64 model's signed pre-quantisation sums S (accum + area) of every
 * pixel, [R, H, W]; target = 0, no gradient. */
int ochre_oracle_forward64(const ochre_oracle_batch *bt, const uint32_t *counts, int W, int H, double *s_out) {
    const size_t n = (size_t)bt->n_rasters * (size_t)W * (size_t)H;
    double *zero = (double *)calloc(n ? n : 1, sizeof(double));
    if (!zero) return OCHRE_ORACLE_E_NOMEM;
    double loss;
    const int st = diff64_impl(bt, counts, W, H, zero, NULL, &loss, NULL, NULL, s_out);
    free(zero);
    return st;
}

/* ------------------------------------------------------------------ */
/* Headless compositing (examples/svg.rs restated without GL)          */
/* ------------------------------------------------------------------ */
/* Every tile is an 8x8 quad textured with its alpha mask, every span an
 * n x 8 quad with mask 1 (the atlas texel at (0,0) is 255,
 * examples/svg.rs:33-38, 85-87), coloured with its raster's RGBA8 colour;
 * the fragment is colour * (1, 1, 1, mask) (:341-353) and blends with
 * SRC_ALPHA, ONE_MINUS_SRC_ALPHA on all four channels (:173-174) into an
 * RGBA8 target, quantised after every quad (f -> floor(f * 255 + 0.5)).
 * Rasters are drawn in order (:139-165); within a raster nothing overlaps. */
static uint8_t unorm8(float f) {
    float q = floorf(f * 255.0f + 0.5f);
    if (!(q >= 0.0f)) q = 0.0f;
    if (q > 255.0f) q = 255.0f;
    return (uint8_t)q;
}

static void blend_px(uint8_t *dst, const uint8_t *col, uint8_t mask) {
    const float a = ((float)col[3] / 255.0f) * ((float)mask / 255.0f);
    const float ia = 1.0f - a;
    for (int c = 0; c < 3; c++) {
        const float s = (float)col[c] / 255.0f;
        const float d = (float)dst[c] / 255.0f;
        dst[c] = unorm8(s * a + d * ia);
    }
    const float d = (float)dst[3] / 255.0f;
    dst[3] = unorm8(a * a + d * ia);
}

void ochre_oracle_composite(uint32_t n_rasters, const int16_t *tile_xy, const uint8_t *tile_alpha,
                            const uint64_t *raster_tile_off, const int16_t *span_xy, const uint16_t *span_w,
                            const uint64_t *raster_span_off, const uint8_t *colors, uint32_t w, uint32_t h,
                            uint8_t *canvas) {
    for (uint32_t r = 0; r < n_rasters; r++) {
        const uint8_t *col = colors + 4 * (size_t)r;
        for (uint64_t t = raster_tile_off[r]; t < raster_tile_off[r + 1]; t++) {
            const int x0 = tile_xy[2 * t], y0 = tile_xy[2 * t + 1];
            for (int py = 0; py < 8; py++)
                for (int px = 0; px < 8; px++) {
                    const int x = x0 + px, y = y0 + py;
                    if (x < 0 || y < 0 || x >= (int)w || y >= (int)h) continue;
                    blend_px(canvas + 4 * ((size_t)y * w + x), col, tile_alpha[64 * t + 8 * py + px]);
                }
        }
        for (uint64_t s = raster_span_off[r]; s < raster_span_off[r + 1]; s++) {
            const int x0 = span_xy[2 * s], y0 = span_xy[2 * s + 1];
            for (int py = 0; py < 8; py++)
                for (int px = 0; px < (int)span_w[s]; px++) {
                    const int x = x0 + px, y = y0 + py;
                    if (x < 0 || y < 0 || x >= (int)w || y >= (int)h) continue;
                    blend_px(canvas + 4 * ((size_t)y * w + x), col, 255);
                }
        }
    }
}
