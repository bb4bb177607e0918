// Differentiable fill: dense coverage images, an L2 loss, and the
// hand-written adjoint back to control points and transforms.
//
// The reference only renders (rasterizer.rs:180-268); this extends its
// forward model.  Coverage of pixel (x, y) of raster r's w x h canvas:
//   c = min(|S|, 1),  S = (sum of heights left of the pixel on its row) + area
// inside boundary tiles (S is the reference's accum + area before
// quantisation, rasterizer.rs:232-239), 1 inside spans, 0 elsewhere.
//
// Backward, with the discrete structure (line counts, visited cells, tiles)
// held fixed: the one the last render_coverage of the same batch left in the
// context while nothing has rewritten it since, else recomputed by running
// the forward chain again:
//   dL/dS   = dL/dc * sign(S) * [|S| < 1] at boundary-tile pixels, else 0;
//   an increment (cell x, y; area a, height h) adds a to S(x, y) and h to
//   S(x', y) for every x' > x, so dL/da = dL/dS(x, y) and dL/dh = the suffix
//   sum of dL/dS to the right of x on row y;
//   a = h * m, h = p1.y - p0.y, m = ((x+1 - p0.x) + (x+1 - p1.x)) / 2 where
//   p0 / p1 are where the line enters / leaves the cell: the line's start or
//   end, or its crossing with a pixel boundary x = X (p.y = A.y + s (B.y - A.y),
//   s = (X - A.x) / (B.x - A.x)) or y = Y (symmetric);
//   line end points q_j = curve(t_j), t_j = min(j * dt, 1) with dt the
//   reference's step (path.rs:50, 60-63), so dq_j/dtheta = basis_j + curve'(t_j)
//   * j * d(dt)/dtheta for unclamped t_j;
//   device-space points p = M v + o, so dv = M^T dp, dM = dp v^T, do = dp.
// Closing lines whose ends coincide are kept as zero-length edges (see
// degenerate_dy).  Conic points are the conic at the subdivision's
// parameters t (held fixed, like the curves' line counts): linear in the
// control points, with a weight derivative (path.rs:75-104).
#include <algorithm>

#include "common.cuh"
#include "flatten.cuh"
#include "internal.h"

namespace ochre {

__device__ __forceinline__ int tile_x_of(uint32_t xy) { return (int)(int16_t)(xy & 0xffffu); }
__device__ __forceinline__ int tile_y_of(uint32_t xy) { return (int)(int16_t)(xy >> 16); }

// ---- forward: tiles and spans onto dense canvases ----
// (t_dev / n_dev / l_dev below: a count held on the device, in CUDA-graph
// replays; the launch-time count is then its capacity, see dev_count)
__global__ void k_composite_tiles(const uint32_t* __restrict__ tile_xy, const float* __restrict__ tile_sum,
                                  uint32_t T, const uint32_t* t_dev, const uint32_t* __restrict__ raster_tile_off,
                                  uint32_t R, uint32_t W, uint32_t H, float* __restrict__ cov) {
    const uint64_t idx = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const uint32_t t = (uint32_t)(idx >> 6), c = (uint32_t)(idx & 63u);
    if (t >= dev_count(T, t_dev)) return;
    const uint32_t r = upper_bound_u32(raster_tile_off, R + 1, t) - 1u;
    const uint32_t xy = tile_xy[t];
    const int x = tile_x_of(xy) + (int)(c & 7u), y = tile_y_of(xy) + (int)(c >> 3);
    if (x < 0 || y < 0 || x >= (int)W || y >= (int)H) return;
    cov[(size_t)r * W * H + (size_t)y * W + x] = fminf(fabsf(tile_sum[(size_t)t * 64 + c]), 1.0f);
}

__global__ void k_composite_spans(const uint32_t* __restrict__ span_xy, const uint16_t* __restrict__ span_w,
                                  uint32_t N, const uint32_t* n_dev, const uint32_t* __restrict__ raster_span_off,
                                  uint32_t R, uint32_t W, uint32_t H, float* __restrict__ cov) {
    const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= dev_count(N, n_dev)) return;
    const uint32_t s = (uint32_t)warp;
    const uint32_t r = upper_bound_u32(raster_span_off, R + 1, s) - 1u;
    const int x0 = tile_x_of(span_xy[s]), y0 = tile_y_of(span_xy[s]);
    const int w = span_w[s];
    float* img = cov + (size_t)r * W * H;
    for (int i = lane; i < 8 * w; i += 32) {
        const int x = x0 + i % w, y = y0 + i / w;
        if (x >= 0 && y >= 0 && x < (int)W && y < (int)H) img[(size_t)y * W + x] = 1.0f;
    }
}

// ---- L2 loss ----
// Per thread a compensated (Kahan) float sum of (cov - target)^2 (its error
// does not grow with the count: FP64 arithmetic per pixel would bound this
// kernel by the GPU's FP64 rate instead of HBM), one double per thread into
// the block reduction.  16-byte accesses when all three arrays allow.
__global__ void k_l2(const float* __restrict__ cov, const float* __restrict__ target, uint64_t n,
                     double* __restrict__ loss, float* __restrict__ dl) {
    float sum = 0.0f, comp = 0.0f;
    auto add = [&](float d) {
        const float y = d * d - comp;
        const float t = sum + y;
        comp = (t - sum) - y;
        sum = t;
    };
    const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x, stride = (uint64_t)gridDim.x * blockDim.x;
    const bool vec = ((reinterpret_cast<uintptr_t>(cov) | reinterpret_cast<uintptr_t>(target) |
                       reinterpret_cast<uintptr_t>(dl)) & 15u) == 0;
    uint64_t done = 0;
    if (vec) {
        const uint64_t n4 = n / 4;
        const float4* c4 = reinterpret_cast<const float4*>(cov);
        const float4* t4 = reinterpret_cast<const float4*>(target);
        float4* d4 = reinterpret_cast<float4*>(dl);
        for (uint64_t i = tid; i < n4; i += stride) {
            const float4 c = c4[i], g = t4[i];
            const float4 d = make_float4(c.x - g.x, c.y - g.y, c.z - g.z, c.w - g.w);
            add(d.x);
            add(d.y);
            add(d.z);
            add(d.w);
            if (dl) d4[i] = make_float4(2.0f * d.x, 2.0f * d.y, 2.0f * d.z, 2.0f * d.w);
        }
        done = n4 * 4;
    }
    for (uint64_t i = done + tid; i < n; i += stride) {
        const float d = cov[i] - target[i];
        add(d);
        if (dl) dl[i] = 2.0f * d;
    }
    double acc = (double)sum - (double)comp;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    __shared__ double s[32];
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) t += s[k];
        atomicAdd(loss, t);
    }
}

// ---- backward 1: dL/dS at boundary-tile pixels ----
__global__ void k_gsigma(const uint32_t* __restrict__ tile_xy, const float* __restrict__ tile_sum, uint32_t T,
                         const uint32_t* t_dev, const uint32_t* __restrict__ raster_tile_off, uint32_t R, uint32_t W,
                         uint32_t H, const float* __restrict__ dl_dcov, float* __restrict__ gsig) {
    const uint64_t idx = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const uint32_t t = (uint32_t)(idx >> 6), c = (uint32_t)(idx & 63u);
    if (t >= dev_count(T, t_dev)) return;
    const uint32_t r = upper_bound_u32(raster_tile_off, R + 1, t) - 1u;
    const uint32_t xy = tile_xy[t];
    const int x = tile_x_of(xy) + (int)(c & 7u), y = tile_y_of(xy) + (int)(c >> 3);
    if (x < 0 || y < 0 || x >= (int)W || y >= (int)H) return;
    const size_t p = (size_t)r * W * H + (size_t)y * W + x;
    const float s = tile_sum[(size_t)t * 64 + c];
    const float g = dl_dcov[p];
    gsig[p] = fabsf(s) < 1.0f ? (s > 0.0f ? g : s < 0.0f ? -g : 0.0f) : 0.0f;
}

// ---- backward 2: exclusive suffix sums of dL/dS along every canvas row ----
__global__ void k_row_suffix(const float* __restrict__ gsig, uint64_t rows, uint32_t W, float* __restrict__ gs,
                             float* __restrict__ row_total) {
    const uint64_t row = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (row >= rows) return;
    const float* g = gsig + row * W;
    float* o = gs + row * W;
    float carry = 0.0f;
    for (int base = (int)((W - 1) / 32) * 32; base >= 0; base -= 32) {
        const int i = base + lane;
        const float v = i < (int)W ? g[i] : 0.0f;
        float suf = v;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const float u = __shfl_down_sync(0xffffffffu, suf, d);
            if (lane + d < 32) suf += u;
        }
        float ex = __shfl_down_sync(0xffffffffu, suf, 1);
        if (lane == 31) ex = 0.0f;
        if (i < (int)W) o[i] = ex + carry;
        carry += __shfl_sync(0xffffffffu, suf, 0);
    }
    if (lane == 0) row_total[row] = carry;
}

// ---- backward 3: per line, dL/d(start, end) along the reference's cells ----
struct LineGrad {
    float ax, ay, bx, by;
};

// A zero-length edge at P (a closing line whose ends coincide, or a line_to
// to the current point): moving its end B by d opens a piece of height d.y in
// cell floor(P), so dL/dB = (0, m g + G) with m = x + 1 - P.x, and
// dL/dA = -dL/dB.  The reference draws nothing for it, but the derivative of
// the closed outline needs it.
__device__ __forceinline__ float degenerate_dy(V2 P, uint32_t r, uint32_t W, uint32_t H, const float* gsig,
                                               const float* gs, const float* row_total) {
    const int x = (int)floorf(P.x), y = (int)floorf(P.y);
    if (y < 0 || y >= (int)H) return 0.0f;
    float g = 0.0f, G;
    if (x < 0) {
        G = row_total[(size_t)r * H + y];
    } else if (x < (int)W) {
        const size_t p = (size_t)r * W * H + (size_t)y * W + x;
        g = gsig[p];
        G = gs[p];
    } else {
        return 0.0f;
    }
    return ((float)(x + 1) - P.x) * g + G;
}

// Pixel-cell lookup of dL/dS (g) and its exclusive row suffix sum (G);
// cells left of the canvas see the whole row's sum, cells right of it or
// off its rows see nothing.
__device__ __forceinline__ void cell_grads(int x, int y, uint32_t r, uint32_t W, uint32_t H, const float* gsig,
                                           const float* gs, const float* row_total, float& g, float& G) {
    g = 0.0f;
    G = 0.0f;
    if (y < 0 || y >= (int)H) return;
    if (x < 0) {
        G = row_total[(size_t)r * H + y];
    } else if (x < (int)W) {
        const size_t p = (size_t)r * W * H + (size_t)y * W + x;
        g = gsig[p];
        G = gs[p];
    }
}

// Per line: dL/dA and dL/dB summed over the pieces the reference's walk
// cuts the line into (one per visited cell).  Every piece end is the line's
// start (first cell only), its end (last cell only), or a crossing of the
// pixel boundary the walk stepped across (a row step crosses y = Y, a column
// step x = X).  An end point lying on a pixel boundary belongs to the cell
// floor(point), like the start of the line that follows it: when the walk's
// last cell is not floor(B), the last piece ends on the boundary and a
// zero-length piece in floor(B) carries B.  (The coverage is continuous
// there; taking both sides of a shared point in the same cell keeps the
// suffix-sum terms of consecutive lines cancelling.)
__global__ void k_line_grad(const float4* __restrict__ lines, const uint32_t* __restrict__ line_raster, uint32_t L,
                            const uint32_t* l_dev, uint32_t W, uint32_t H, const float* __restrict__ gsig,
                            const float* __restrict__ gs, const float* __restrict__ row_total,
                            LineGrad* __restrict__ out) {
    const uint32_t l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= dev_count(L, l_dev)) return;
    const float4 ln = lines[l];
    const V2 A = v2(ln.x, ln.y), B = v2(ln.z, ln.w);
    const uint32_t r = line_raster[l];
    LineGrad d{0.0f, 0.0f, 0.0f, 0.0f};
    if (veq(A, B)) {
        const float dy = degenerate_dy(B, r, W, H, gsig, gs, row_total);
        d.ay = -dy;
        d.by = dy;
    } else {
        const float D = B.x - A.x, E = B.y - A.y;
        // p.y on the vertical pixel boundary x = X, as a function of A and B
        auto vertical = [&](float X, float gy) {
            const float s = (X - A.x) / D;
            d.ay += gy * (1.0f - s);
            d.by += gy * s;
            d.ax += gy * E * (s - 1.0f) / D;
            d.bx += gy * (-E * s / D);
        };
        // p.x on the horizontal pixel boundary y = Y
        auto horizontal = [&](float Y, float gx) {
            const float u = (Y - A.y) / E;
            d.ax += gx * (1.0f - u);
            d.bx += gx * u;
            d.ay += gx * D * (u - 1.0f) / E;
            d.by += gx * (-D * u / E);
        };
        // a piece end on a boundary crossed by a row step (horizontal) or a column step
        auto crossing = [&](bool row_step, int x, int y, bool leaving, const Walk& w, float gx, float gy) {
            if (row_step)
                horizontal((float)((w.y_dir > 0) == leaving ? y + 1 : y), gx);
            else
                vertical((float)((w.x_dir > 0) == leaving ? x + 1 : x), gy);
        };
        bool first = true, prev_row_step = false;
        walk_line(
            A, B,
            [&](const Walk& w, const WalkState& s) {
                const int x = s.x, y = s.y;
                const bool next_row_step = s.row_t1 < s.col_t1;   // the walk's own choice (ties step x)
                const float t0 = rmax(s.row_t0, s.col_t0), t1 = rmin(s.row_t1, s.col_t1);
                const bool last = t1 >= 1.0f;
                float g, G;
                cell_grads(x, y, r, W, H, gsig, gs, row_total, g, G);
                if (g != 0.0f || G != 0.0f) {
                    const V2 p0 = vlerp(t0, A, B), p1 = vlerp(t1, A, B);
                    const float h = p1.y - p0.y;
                    const float right = (float)(x + 1);
                    const float m = 0.5f * ((right - p0.x) + (right - p1.x));
                    // dL/dp0 and dL/dp1 of a = h m and h
                    const float d0x = -0.5f * h * g, d0y = -m * g - G;
                    const float d1x = -0.5f * h * g, d1y = m * g + G;
                    if (first) {
                        d.ax += d0x;
                        d.ay += d0y;
                    } else {
                        crossing(prev_row_step, x, y, false, w, d0x, d0y);
                    }
                    if (last && x == w.end_x && y == w.end_y) {
                        d.bx += d1x;
                        d.by += d1y;
                    } else {
                        crossing(next_row_step, x, y, true, w, d1x, d1y);
                    }
                }
                if (last && (x != w.end_x || y != w.end_y)) {
                    // zero-length pieces from the last cell into floor(B), the
                    // column first (the walk's tie rule); each holds the height
                    // term of its cell: dL/dp0 = (0, -q), dL/dp1 = (0, q)
                    int cx = x, cy = y;
                    bool row = next_row_step;
                    float bnd = row ? (float)(w.y_dir > 0 ? y + 1 : y) : (float)(w.x_dir > 0 ? x + 1 : x);
                    if (row) cy = w.y_dir > 0 ? cy + 1 : cy - 1; else cx = w.x_dir > 0 ? cx + 1 : cx - 1;
                    for (int k = 0; k < 4; k++) {
                        float gz, Gz;
                        cell_grads(cx, cy, r, W, H, gsig, gs, row_total, gz, Gz);
                        const float q = ((float)(cx + 1) - B.x) * gz + Gz;
                        if (!row) vertical(bnd, -q);   // a horizontal entry passes only dL/dp.x = 0
                        if (cx == w.end_x && cy == w.end_y) {
                            d.by += q;
                            break;
                        }
                        row = cx == w.end_x;
                        const int sx = w.end_x > cx ? 1 : -1, sy = w.end_y > cy ? 1 : -1;
                        bnd = row ? (float)(sy > 0 ? cy + 1 : cy) : (float)(sx > 0 ? cx + 1 : cx);
                        if (!row) vertical(bnd, q);
                        if (row) cy += sy; else cx += sx;
                    }
                }
                first = false;
                prev_row_step = next_row_step;
            },
            [&](int, int, int) {}, [&](int, int) {});
    }
    out[l] = d;
}

// ---- backward 4: per command, through the flattening to device-space points ----
__device__ __forceinline__ void add_point(float* gp, const BatchView& b, int64_t cmd, int q, V2 g) {
    if (cmd < 0) return;
    const uint32_t f = __ldg(b.cmd_foff + cmd) + 2u * (uint32_t)q;
    atomicAdd(gp + f, g.x);
    atomicAdd(gp + f + 1, g.y);
}
__device__ __forceinline__ int endpoint_index(uint8_t v) {
    return v == V_CUBIC ? 2 : (v == V_QUAD || v == V_CONIC) ? 1 : 0;
}
__device__ __forceinline__ V2 add2(V2 a, V2 b) { return v2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ V2 mul2(float s, V2 a) { return v2(s * a.x, s * a.y); }

// (`err`: a planned run's error word; when a count of the run outgrew its
// capacity the lines and offsets are not all there, and nothing is read)
__global__ void k_cmd_grad(BatchView b, const uint32_t* __restrict__ line_off, uint32_t L, const uint32_t* l_dev,
                           const uint32_t* err, const LineGrad* __restrict__ lg, float* __restrict__ gp, uint32_t W,
                           uint32_t H, const float* __restrict__ gsig, const float* __restrict__ gs,
                           const float* __restrict__ row_total) {
    const uint64_t c = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (c >= b.n_cmds) return;
    if (err != nullptr && (ld_relaxed(err) & ERR_CAPACITY)) return;
    L = (uint32_t)dev_count(L, l_dev);
    const CmdCtx k = load_cmd(b, (uint32_t)c);
    if (!k.ok) return;
    const uint32_t o0 = line_off[c];
    const uint32_t o1 = c + 1 < b.n_cmds ? line_off[c + 1] : L;
    const int64_t self = (int64_t)c;
    // the final closing line of finish (rasterizer.rs:181-183) is the raster's last line
    const V2 last_end = k.verb == V_CLOSE ? k.last : k.verb == V_CUBIC ? k.pt[2]
                      : k.verb == V_MOVE || k.verb == V_LINE ? k.pt[0] : k.pt[1];
    const V2 first_end = k.verb == V_MOVE ? k.pt[0] : k.first;
    const bool final_close = k.last_of_raster && !veq(last_end, first_end);
    const int n_own = (int)(o1 - o0) - (final_close ? 1 : 0);
    auto add_last = [&](V2 g) {
        if (k.last_ref >= 0) add_point(gp, b, k.last_ref, endpoint_index(__ldg(b.verbs + k.last_ref)), g);
    };
    auto add_first = [&](V2 g) { add_point(gp, b, k.first_ref, 0, g); };
    switch (k.verb) {
    case V_MOVE:
        if (n_own == 1) {
            const LineGrad g = lg[o0];
            add_last(v2(g.ax, g.ay));
            add_first(v2(g.bx, g.by));
        } else {
            // closing line last -> first of zero length
            const float dy = degenerate_dy(k.first, k.raster, W, H, gsig, gs, row_total);
            add_last(v2(0.0f, -dy));
            add_first(v2(0.0f, dy));
        }
        break;
    case V_LINE: {
        const LineGrad g = lg[o0];
        add_last(v2(g.ax, g.ay));
        add_point(gp, b, self, 0, v2(g.bx, g.by));
        break;
    }
    case V_QUAD:
    case V_CUBIC: {
        const bool cubic = k.verb == V_CUBIC;
        const V2 P0 = k.last, P1 = k.pt[0], P2 = k.pt[1], P3 = k.pt[2];
        const float dt = cubic ? cubic_dt(P0, P1, P2, P3) : quad_dt(P0, P1, P2);
        V2 g0 = v2(0, 0), g1 = v2(0, 0), g2 = v2(0, 0), g3 = v2(0, 0);
        float S = 0.0f;   // sum_j j * <curve'(t_j), dL/dq_j> over unclamped t_j
        const LineGrad first_line = lg[o0];
        g0 = v2(first_line.ax, first_line.ay);   // q_0 = last
        float t = 0.0f;
        for (int j = 1; j <= n_own; j++) {
            t = rmin(__fadd_rn(t, dt), 1.0f);
            const LineGrad gj = lg[o0 + j - 1];
            V2 dq = v2(gj.bx, gj.by);
            if (j < n_own) {
                const LineGrad gn = lg[o0 + j];
                dq = add2(dq, v2(gn.ax, gn.ay));
            }
            const float u = 1.0f - t;
            V2 dcurve;
            if (cubic) {
                const float b0 = u * u * u, b1 = 3.0f * u * u * t, b2 = 3.0f * u * t * t, b3 = t * t * t;
                g0 = add2(g0, mul2(b0, dq));
                g1 = add2(g1, mul2(b1, dq));
                g2 = add2(g2, mul2(b2, dq));
                g3 = add2(g3, mul2(b3, dq));
                dcurve = add2(add2(mul2(3.0f * u * u, vsub(P1, P0)), mul2(6.0f * u * t, vsub(P2, P1))),
                              mul2(3.0f * t * t, vsub(P3, P2)));
            } else {
                const float b0 = u * u, b1 = 2.0f * u * t, b2 = t * t;
                g0 = add2(g0, mul2(b0, dq));
                g1 = add2(g1, mul2(b1, dq));
                g2 = add2(g2, mul2(b2, dq));
                dcurve = add2(mul2(2.0f * u, vsub(P1, P0)), mul2(2.0f * t, vsub(P2, P1)));
            }
            if (t < 1.0f) S += (float)j * (dcurve.x * dq.x + dcurve.y * dq.y);
        }
        if (S != 0.0f && isfinite(dt)) {
            if (cubic) {
                // conc = max(|b|, |a + b|), b = 3(P0 - 2P1 + P2), a + b = 2P0 - 3P1 + P3
                const V2 bv = vscale(3.0f, vadd(vsub(P0, vscale(2.0f, P1)), P2));
                const V2 ab = v2(2.0f * P0.x - 3.0f * P1.x + P3.x, 2.0f * P0.y - 3.0f * P1.y + P3.y);
                const float lb = vlength(bv), lab = vlength(ab);
                const float conc = rmax(lb, lab);
                const float k1 = S * (-0.5f * dt / conc);   // dL/dconc
                if (lb >= lab && lb > 0.0f) {
                    const V2 u1 = mul2(k1 / lb, bv);
                    g0 = add2(g0, mul2(3.0f, u1));
                    g1 = add2(g1, mul2(-6.0f, u1));
                    g2 = add2(g2, mul2(3.0f, u1));
                } else if (lab > 0.0f) {
                    const V2 u1 = mul2(k1 / lab, ab);
                    g0 = add2(g0, mul2(2.0f, u1));
                    g1 = add2(g1, mul2(-3.0f, u1));
                    g3 = add2(g3, u1);
                }
            } else {
                const V2 vv = vadd(vsub(P0, vscale(2.0f, P1)), P2);
                const float len2 = vv.x * vv.x + vv.y * vv.y;
                if (len2 > 0.0f) {
                    const V2 u1 = mul2(S * (-0.5f * dt / len2), vv);   // dL/dv
                    g0 = add2(g0, u1);
                    g1 = add2(g1, mul2(-2.0f, u1));
                    g2 = add2(g2, u1);
                }
            }
        }
        add_last(g0);
        add_point(gp, b, self, 0, g1);
        add_point(gp, b, self, 1, g2);
        if (cubic) add_point(gp, b, self, 2, g3);
        break;
    }
    case V_CONIC: {
        // path.rs:75-104: every emitted point is the conic at a subdivision
        // parameter t, q = ((1-t)^2 P0 + 2t(1-t) w P1 + t^2 P2) / D, D =
        // (1-t)^2 + 2t(1-t) w + t^2; the subdivision (which t) is held fixed,
        // so q is linear in the control points, and dq/dw = 2t(1-t)(P1 - q)/D.
        const V2 P0 = k.last, P1 = k.pt[0], P2 = k.pt[1];
        const float w = k.w;
        const LineGrad first_line = lg[o0];
        V2 g0 = v2(first_line.ax, first_line.ay), g1 = v2(0, 0), g2 = v2(0, 0);
        float gw = 0.0f;
        int j = 0;
        bool capped = false;
        conic_flatten_t(P0, P1, P2, w, &capped, [&](V2 q, float t) {
            j++;
            if (j > n_own) return;
            const LineGrad gj = lg[o0 + j - 1];
            V2 dq = v2(gj.bx, gj.by);
            if (j < n_own) {
                const LineGrad gn = lg[o0 + j];
                dq = add2(dq, v2(gn.ax, gn.ay));
            }
            const float u = 1.0f - t;
            const float D = u * u + 2.0f * t * u * w + t * t;
            const float A = u * u / D, B = 2.0f * t * u * w / D, C = t * t / D;
            g0 = add2(g0, mul2(A, dq));
            g1 = add2(g1, mul2(B, dq));
            g2 = add2(g2, mul2(C, dq));
            const float dw = 2.0f * t * u / D;
            gw += dw * ((P1.x - q.x) * dq.x + (P1.y - q.y) * dq.y);
        });
        add_last(g0);
        add_point(gp, b, self, 0, g1);
        add_point(gp, b, self, 1, g2);
        atomicAdd(gp + __ldg(b.cmd_foff + c) + 4, gw);   // the weight (not transformed)
        break;
    }
    default:
        break;
    }
    if (k.last_of_raster) {
        V2 ga, gb;
        if (final_close) {
            const LineGrad g = lg[o1 - 1];
            ga = v2(g.ax, g.ay);
            gb = v2(g.bx, g.by);
        } else {
            // zero-length final closing line (the contour ends where it began)
            const float dy = degenerate_dy(first_end, k.raster, W, H, gsig, gs, row_total);
            ga = v2(0.0f, -dy);
            gb = v2(0.0f, dy);
        }
        if (k.verb == V_CLOSE) add_last(ga);
        else add_point(gp, b, self, endpoint_index(k.verb), ga);
        if (k.verb == V_MOVE) add_point(gp, b, self, 0, gb);
        else add_first(gb);
    }
}

// ---- backward 5: device-space point gradients -> input points and transforms ----
__global__ void k_fill_grad(BatchView b, const float* __restrict__ gp, float* __restrict__ dl_dpts,
                            float* __restrict__ dl_dxf) {
    const uint64_t c = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const bool valid = c < b.n_cmds;
    float acc[6] = {0, 0, 0, 0, 0, 0};
    uint32_t f = 0xffffffffu;
    if (valid) {
        f = fill_of(b, (uint32_t)c);
        const uint8_t v = __ldg(b.verbs + c);
        const uint32_t fo = __ldg(b.cmd_foff + c);
        const int np = v == V_MOVE || v == V_LINE ? 1 : v == V_QUAD || v == V_CONIC ? 2 : v == V_CUBIC ? 3 : 0;
        const bool raw = b.fill_flags != nullptr && (__ldg(b.fill_flags + f) & OCHRE_FILL_RAW);
        const float* m = b.fill_xf + 6 * (size_t)f;
        for (int q = 0; q < np; q++) {
            const float gx = gp[fo + 2 * q], gy = gp[fo + 2 * q + 1];
            if (raw) {
                dl_dpts[fo + 2 * q] = gx;
                dl_dpts[fo + 2 * q + 1] = gy;
            } else {
                const float vx = __ldg(b.pts + fo + 2 * q), vy = __ldg(b.pts + fo + 2 * q + 1);
                dl_dpts[fo + 2 * q] = __ldg(m + 0) * gx + __ldg(m + 2) * gy;
                dl_dpts[fo + 2 * q + 1] = __ldg(m + 1) * gx + __ldg(m + 3) * gy;
                acc[0] += gx * vx;
                acc[1] += gx * vy;
                acc[2] += gy * vx;
                acc[3] += gy * vy;
                acc[4] += gx;
                acc[5] += gy;
            }
        }
        if (v == V_CONIC) dl_dpts[fo + 4] = gp[fo + 4];   // the weight's gradient, as accumulated
    }
    // commands of a fill are contiguous: segmented reduction over the warp
    const uint32_t fprev = __shfl_up_sync(0xffffffffu, f, 1);
    const bool head = lane == 0 || fprev != f;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t fo = __shfl_down_sync(0xffffffffu, f, d);
#pragma unroll
        for (int i = 0; i < 6; i++) {
            const float o = __shfl_down_sync(0xffffffffu, acc[i], d);
            if (lane + d < 32 && fo == f) acc[i] += o;
        }
    }
    // a lane's sum may include lanes past its segment only if f matched all the way, which the
    // contiguity of fills guarantees; heads hold their segment's total
    if (valid && head) {
        for (int i = 0; i < 6; i++)
            if (acc[i] != 0.0f) atomicAdd(dl_dxf + 6 * (size_t)f + i, acc[i]);
    }
}

// Runs the forward chain with signed tile coverage (the backward's
// recomputation and the coverage render share it).
static int run_signed_chain(ochre_gpu_ctx* ctx, const ochre_batch* in, cudaStream_t s, ochre_result* res) {
    const uint32_t saved = ctx->flags;
    ctx->flags = (saved | OCHRE_CTX_WANT_COV | OCHRE_CTX_CHAIN_ONLY);
    ctx->cov_signed = true;
    const int st = run_device(ctx, in, res, s);
    ctx->flags = saved;
    ctx->cov_signed = false;
    return st;
}

static BatchView view_of(ochre_gpu_ctx* ctx, const ochre_batch* in) {
    return BatchView{in->verbs, in->pts, in->fill_cmd_off, in->fill_xf, in->fill_flags, in->raster_fill_off,
                     in->n_fills, in->n_rasters, in->n_cmds, ctx->cmd_foff.as<uint32_t>(),
                     ctx->cmd_mv.as<uint32_t>(), ctx->cmd_ep.as<uint32_t>(), in->n_floats};
}

int stage_diff_tail(ochre_gpu_ctx* ctx, const ochre_batch* in, const DiffStep& d, cudaStream_t s) {
    DevScalars* ds = dev_scalars(ctx);
    const GraphPlan* plan = ctx->plan;
    const uint32_t R = in->n_rasters, w = d.w, h = d.h;
    const size_t npx = (size_t)R * w * h;
    // capacities; the counts stay on the device (span capacity = tile capacity)
    const uint32_t T = plan->tiles, L = plan->lines;
    const uint32_t* t_dev = &ds->n_tiles;
    const uint32_t* n_dev = &ds->n_spans;
    const uint32_t* l_dev = &ds->n_lines;
    const uint32_t* tile_xy = ctx->out_tile_xy.as<uint32_t>();
    const float* tile_sum = ctx->out_tile_cov.as<float>();
    const uint32_t* tile_off = ctx->out_raster_tile_off.as<uint32_t>();
    // coverage render (ochre_gpu_render_coverage)
    if (npx) OCHRE_CUDA_TRY(cudaMemsetAsync(d.cov, 0, npx * sizeof(float), s));
    if (npx && T) {
        OCHRE_LAUNCH(ctx, "composite_tiles", s,
                     k_composite_tiles<<<(unsigned)(((uint64_t)T * 64 + 255) / 256), 256, 0, s>>>(
                         tile_xy, tile_sum, T, t_dev, tile_off, R, w, h, d.cov));
        OCHRE_LAUNCH(ctx, "composite_spans", s,
                     k_composite_spans<<<(unsigned)(((uint64_t)T * 32 + 255) / 256), 256, 0, s>>>(
                         ctx->out_span_xy.as<uint32_t>(), ctx->out_span_w.as<uint16_t>(), T, n_dev,
                         ctx->out_raster_span_off.as<uint32_t>(), R, w, h, d.cov));
    }
    // loss and dL/dcov (ochre_gpu_l2_loss)
    OCHRE_CUDA_TRY(cudaMemsetAsync(d.loss, 0, sizeof(double), s));
    if (npx) {
        const int blocks = (int)std::min<uint64_t>((npx + 255) / 256, 152u * 16u);
        OCHRE_LAUNCH(ctx, "l2_loss", s, k_l2<<<blocks, 256, 0, s>>>(d.cov, d.target, npx, d.loss, d.dl_dcov));
    }
    OCHRE_CUDA_TRY(cudaGetLastError());
    // backward (ochre_gpu_fill_backward) on this run's lines and tiles
    if (in->n_floats) OCHRE_CUDA_TRY(cudaMemsetAsync(d.dl_dpts, 0, in->n_floats * sizeof(float), s));
    if (in->n_fills) OCHRE_CUDA_TRY(cudaMemsetAsync(d.dl_dxf, 0, (size_t)in->n_fills * 6 * sizeof(float), s));
    if (R == 0 || in->n_cmds == 0 || L == 0 || npx == 0) return OCHRE_OK;
    OCHRE_CUDA_TRY(ctx->grad_g.ensure(npx * 4));
    OCHRE_CUDA_TRY(ctx->grad_gs.ensure(npx * 4));
    OCHRE_CUDA_TRY(ctx->grad_left.ensure((size_t)R * h * 4));
    OCHRE_CUDA_TRY(ctx->grad_line.ensure((size_t)L * sizeof(LineGrad)));
    OCHRE_CUDA_TRY(ctx->grad_pts.ensure(in->n_floats * 4));
    float* gsig = ctx->grad_g.as<float>();
    OCHRE_CUDA_TRY(cudaMemsetAsync(gsig, 0, npx * 4, s));
    if (T)
        OCHRE_LAUNCH(ctx, "grad_sigma", s,
                     k_gsigma<<<(unsigned)(((uint64_t)T * 64 + 255) / 256), 256, 0, s>>>(
                         tile_xy, tile_sum, T, t_dev, tile_off, R, w, h, d.dl_dcov, gsig));
    const uint64_t rows = (uint64_t)R * h;
    OCHRE_LAUNCH(ctx, "grad_row_suffix", s,
                 k_row_suffix<<<(unsigned)((rows * 32 + 255) / 256), 256, 0, s>>>(
                     gsig, rows, w, ctx->grad_gs.as<float>(), ctx->grad_left.as<float>()));
    OCHRE_LAUNCH(ctx, "grad_lines", s,
                 k_line_grad<<<(L + 127) / 128, 128, 0, s>>>(ctx->lines.as<float4>(), ctx->line_raster.as<uint32_t>(),
                                                             L, l_dev, w, h, gsig, ctx->grad_gs.as<float>(),
                                                             ctx->grad_left.as<float>(), ctx->grad_line.as<LineGrad>()));
    OCHRE_CUDA_TRY(cudaMemsetAsync(ctx->grad_pts.p, 0, in->n_floats * 4, s));
    const BatchView b = view_of(ctx, in);
    const unsigned cb = (unsigned)((in->n_cmds + 127) / 128);
    OCHRE_LAUNCH(ctx, "grad_commands", s,
                 k_cmd_grad<<<cb, 128, 0, s>>>(b, ctx->cmd_line_off.as<uint32_t>(), L, l_dev, &ds->err,
                                               ctx->grad_line.as<LineGrad>(), ctx->grad_pts.as<float>(), w, h, gsig,
                                               ctx->grad_gs.as<float>(), ctx->grad_left.as<float>()));
    OCHRE_LAUNCH(ctx, "grad_fills", s, k_fill_grad<<<cb, 128, 0, s>>>(b, ctx->grad_pts.as<float>(), d.dl_dpts, d.dl_dxf));
    OCHRE_CUDA_TRY(cudaGetLastError());
    return OCHRE_OK;
}

}  // namespace ochre

using namespace ochre;

extern "C" {

int ochre_gpu_render_coverage(ochre_gpu_ctx* ctx, const ochre_batch* in, uint32_t w, uint32_t h, float* cov,
                              void* stream) {
    if (!ctx || !in || (!cov && in->n_rasters && w && h) || w > MAX_CANVAS || h > MAX_CANVAS) return OCHRE_E_INVALID;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return OCHRE_E_CUDA;
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->own_stream;
    ctx->saved.valid = false;
    ochre_result res;
    int st = run_signed_chain(ctx, in, s, &res);
    if (st != OCHRE_OK) return st;
    if (!in->fill_width)
        ctx->saved = ochre_gpu_ctx::SavedForward{true, ctx->epoch, *in, res, (uint32_t)ctx->stats.n_lines};
    const size_t npx = (size_t)in->n_rasters * w * h;
    if (npx) OCHRE_CUDA_TRY(cudaMemsetAsync(cov, 0, npx * sizeof(float), s));
    if (res.n_tiles) {
        const uint64_t threads = (uint64_t)res.n_tiles * 64;
        OCHRE_LAUNCH(ctx, "composite_tiles", s,
                     k_composite_tiles<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(
                         reinterpret_cast<const uint32_t*>(res.tile_xy), res.tile_cov, res.n_tiles, nullptr,
                         res.raster_tile_off, in->n_rasters, w, h, cov));
    }
    if (res.n_spans) {
        const uint64_t threads = (uint64_t)res.n_spans * 32;
        OCHRE_LAUNCH(ctx, "composite_spans", s,
                     k_composite_spans<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(
                         reinterpret_cast<const uint32_t*>(res.span_xy), res.span_width, res.n_spans, nullptr,
                         res.raster_span_off, in->n_rasters, w, h, cov));
    }
    OCHRE_CUDA_TRY(cudaGetLastError());
    ctx->stats.n_launches = ctx->launches;
    collect_timings(ctx, s);
    return OCHRE_OK;
}

int ochre_gpu_l2_loss(ochre_gpu_ctx* ctx, const float* cov, const float* target, uint64_t n, double* loss,
                      float* dl_dcov, void* stream) {
    if (!ctx || !cov || !target || !loss) return OCHRE_E_INVALID;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return OCHRE_E_CUDA;
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->own_stream;
    ctx->prof_used = 0;
    ctx->launches = 0;
    OCHRE_CUDA_TRY(cudaMemsetAsync(loss, 0, sizeof(double), s));
    if (n == 0) return OCHRE_OK;
    int blocks = (int)std::min<uint64_t>((n + 255) / 256, 152u * 16u);
    OCHRE_LAUNCH(ctx, "l2_loss", s, k_l2<<<blocks, 256, 0, s>>>(cov, target, n, loss, dl_dcov));
    OCHRE_CUDA_TRY(cudaGetLastError());
    collect_timings(ctx, s);
    return OCHRE_OK;
}

int ochre_gpu_fill_backward(ochre_gpu_ctx* ctx, const ochre_batch* in, uint32_t w, uint32_t h,
                            const float* dl_dcov, float* dl_dpts, float* dl_dxf, void* stream) {
    if (!ctx || !in || (in->n_rasters && w && h && !dl_dcov) || (in->n_floats && !dl_dpts) ||
        (in->n_fills && !dl_dxf) || w > MAX_CANVAS || h > MAX_CANVAS)
        return OCHRE_E_INVALID;
    if (in->fill_width) return OCHRE_E_INVALID;   // stroked fills are not differentiated
    if (cudaSetDevice(ctx->device) != cudaSuccess) return OCHRE_E_CUDA;
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->own_stream;
    // the forward structure (lines, cells, tiles) and signed coverage: the
    // one the last render_coverage of this batch left, else recomputed
    ochre_result res;
    uint32_t L;
    if (ctx->saved.valid && ctx->saved.epoch == ctx->epoch && same_batch(ctx->saved.in, *in)) {
        res = ctx->saved.res;
        L = ctx->saved.n_lines;
        ctx->prof_used = 0;
        ctx->launches = 0;
    } else {
        const int st = run_signed_chain(ctx, in, s, &res);
        if (st != OCHRE_OK) return st;
        L = (uint32_t)ctx->stats.n_lines;
    }
    const uint32_t R = in->n_rasters;
    const size_t npx = (size_t)R * w * h;
    if (in->n_floats) OCHRE_CUDA_TRY(cudaMemsetAsync(dl_dpts, 0, in->n_floats * sizeof(float), s));
    if (in->n_fills) OCHRE_CUDA_TRY(cudaMemsetAsync(dl_dxf, 0, (size_t)in->n_fills * 6 * sizeof(float), s));
    if (R == 0 || in->n_cmds == 0 || L == 0 || w == 0 || h == 0) {
        ctx->stats.n_launches = ctx->launches;
        collect_timings(ctx, s);
        return OCHRE_OK;
    }
    OCHRE_CUDA_TRY(ctx->grad_g.ensure(npx * 4));
    OCHRE_CUDA_TRY(ctx->grad_gs.ensure(npx * 4));
    OCHRE_CUDA_TRY(ctx->grad_left.ensure((size_t)R * h * 4));
    OCHRE_CUDA_TRY(ctx->grad_line.ensure((size_t)L * sizeof(LineGrad)));
    OCHRE_CUDA_TRY(ctx->grad_pts.ensure(in->n_floats * 4));
    float* gsig = ctx->grad_g.as<float>();
    OCHRE_CUDA_TRY(cudaMemsetAsync(gsig, 0, npx * 4, s));
    if (res.n_tiles) {
        const uint64_t threads = (uint64_t)res.n_tiles * 64;
        OCHRE_LAUNCH(ctx, "grad_sigma", s,
                     k_gsigma<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(
                         reinterpret_cast<const uint32_t*>(res.tile_xy), res.tile_cov, res.n_tiles, nullptr,
                         res.raster_tile_off, R, w, h, dl_dcov, gsig));
    }
    const uint64_t rows = (uint64_t)R * h;
    OCHRE_LAUNCH(ctx, "grad_row_suffix", s,
                 k_row_suffix<<<(unsigned)((rows * 32 + 255) / 256), 256, 0, s>>>(
                     gsig, rows, w, ctx->grad_gs.as<float>(), ctx->grad_left.as<float>()));
    OCHRE_LAUNCH(ctx, "grad_lines", s,
                 k_line_grad<<<(L + 127) / 128, 128, 0, s>>>(ctx->lines.as<float4>(), ctx->line_raster.as<uint32_t>(),
                                                             L, nullptr, w, h, gsig, ctx->grad_gs.as<float>(),
                                                             ctx->grad_left.as<float>(), ctx->grad_line.as<LineGrad>()));
    OCHRE_CUDA_TRY(cudaMemsetAsync(ctx->grad_pts.p, 0, in->n_floats * 4, s));
    const BatchView b = view_of(ctx, in);
    const unsigned cb = (unsigned)((in->n_cmds + 127) / 128);
    OCHRE_LAUNCH(ctx, "grad_commands", s,
                 k_cmd_grad<<<cb, 128, 0, s>>>(b, ctx->cmd_line_off.as<uint32_t>(), L, nullptr, nullptr,
                                               ctx->grad_line.as<LineGrad>(),
                                               ctx->grad_pts.as<float>(), w, h, gsig, ctx->grad_gs.as<float>(),
                                               ctx->grad_left.as<float>()));
    OCHRE_LAUNCH(ctx, "grad_fills", s,
                 k_fill_grad<<<cb, 128, 0, s>>>(b, ctx->grad_pts.as<float>(), dl_dpts, dl_dxf));
    OCHRE_CUDA_TRY(cudaGetLastError());
    ctx->stats.n_launches = ctx->launches;
    collect_timings(ctx, s);
    return OCHRE_OK;
}

}  // extern "C"
