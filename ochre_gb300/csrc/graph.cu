// CUDA-graph execution of the whole fill -> finish launch chain.
//
// The eager chain (run_device) reads three or four counts back to the host
// between stages to size its buffers.  A graph cannot do that, so a graph is
// built from a plan:
//   1. one eager run of the batch gives its counts (lines, sort entries,
//      tiles, key bits, tile rows) and its execution form (fused or chain);
//   2. capacities = counts x headroom (+ a margin); every buffer is sized to
//      them by one uncaptured run of the planned chain, which also checks it;
//   3. the planned chain is captured on the context's stream: the counts stay
//      on the device, each kernel reads its own and its grid covers the
//      capacity; check kernels zero a count that exceeds its capacity and flag
//      ERR_CAPACITY (plan_lines, plan_entries, plan_tiles); the last node
//      copies the device scalars to mapped host memory.
// A launch replays the graph and reads the scalars.  If a count outgrew its
// capacity (or, in the fused form, a raster no longer fits the fused kernel),
// the graph is re-planned from an eager run and replayed once.
//
// The graph owns a private context: the buffers its nodes point at belong to
// it alone, so eager calls on the caller's context never move them.  The
// batch's device pointers and counts are fixed at creation; the values behind
// them (points, transforms, verbs of the same float layout, stroke widths)
// may change between launches.
//
// Stroked fills: the stroke stage (stroke.cu) is planned as well (polyline
// and output command and float capacities, its counts on the device, a check
// after each of its two scans), and its output is padded with Close commands
// to the planned command count on the batch's last fill, so the chain after
// it sees fixed command and float counts.  A trailing Close adds no line and
// leaves the raster's closing line last, so the padding changes no output.
// Such a plan always uses the general chain (every pad command sits on the
// last raster, which the fused kernel's per-raster command limit would
// refuse).
//
// A differentiable step (ochre_graph_create_diff) is the chain with signed
// tile coverage followed by stage_diff_tail (grad.cu): the coverage render,
// the L2 loss and the backward, on caller buffers fixed at creation, every
// count read on the device.
#include "common.cuh"
#include "internal.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

struct ochre_graph {
    ochre_gpu_ctx* ctx = nullptr;   // private context (buffers, stream, scalars)
    ochre_batch batch{};
    float headroom = 1.25f;
    ochre::GraphPlan plan{};
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint32_t kernels = 0;           // kernel launches captured
    uint32_t replans = 0;
    ochre_stats stats{};
    bool is_diff = false;           // a differentiable step (ochre_graph_create_diff)
    ochre::DiffStep diff{};
};

namespace ochre {

namespace {

uint32_t cap_of(uint64_t n, float headroom, uint64_t limit = MAX_COUNT) {
    const uint64_t c = (uint64_t)((double)n * headroom) + 1024u;
    return (uint32_t)std::min<uint64_t>(c, limit);
}

// The planned chain: the stages of run_device with ctx->plan set (no host
// read-backs), then the scalars copied to the host.
int planned_body(ochre_gpu_ctx* ctx, const ochre_batch* batch, cudaStream_t s) {
    DevScalars* ds = dev_scalars(ctx);
    ctx->launches = 0;
    const uint32_t R = batch->n_rasters;
    // stroked fills become plain fills first, padded to the planned command
    // count; the chain below keeps the stroke stage's error bits
    ochre_batch stroked = *batch;
    const bool stroke = ctx->plan->stroke;
    if (stroke) {
        OCHRE_CUDA_TRY(cudaMemsetAsync(ds, 0, sizeof(DevScalars), s));
        const int sst = stage_stroke(ctx, batch, s, &stroked);
        if (sst != OCHRE_OK) return sst;
    }
    const ochre_batch* in = &stroked;
    OCHRE_CUDA_TRY(ctx->out_raster_tile_off.ensure((size_t)(R + 1) * 4));
    OCHRE_CUDA_TRY(ctx->out_raster_span_off.ensure((size_t)(R + 1) * 4));
    int st;
    if (ctx->plan->fused) {
        bool handled = false;
        uint32_t T = 0, N = 0;
        st = stage_fused(ctx, in, s, &handled, &T, &N);
        if (st != OCHRE_OK) return st;
    } else {
        const size_t keep = stroke ? offsetof(DevScalars, ticket) : 0;
        OCHRE_CUDA_TRY(cudaMemsetAsync(reinterpret_cast<char*>(ds) + keep, 0, sizeof(DevScalars) - keep, s));
        uint32_t L = 0, bits = 0, passes = 0, T = 0, N = 0;
        uint64_t E = 0;
        st = stage_flatten(ctx, in, s, &L);
        if (st != OCHRE_OK) return st;
        st = stage_bin(ctx, in, L, s, &E, &bits);
        if (st != OCHRE_OK) return st;
        st = stage_sort(ctx, E, bits, s, &passes);
        if (st != OCHRE_OK) return st;
        st = stage_tiles(ctx, in, E, s, &T, &N);
        if (st != OCHRE_OK) return st;
        ctx->stats.sort_passes = passes;
        if (ctx->plan->diff) {
            st = stage_diff_tail(ctx, in, *ctx->plan->diff, s);
            if (st != OCHRE_OK) return st;
        }
    }
    // the scalars to the host: a kernel store into mapped memory, else a copy
    ctx->launches++;
    return copy_scalars_async(ctx, s);
}

// The context's device buffer addresses, sorted (the sort swaps its key and
// value buffers between passes, which keeps this set).
std::vector<void*> buffer_set(ochre_gpu_ctx* ctx) {
    std::vector<void*> v;
    for (const DevBuf* b : device_buffers(ctx)) v.push_back(b->p);
    std::sort(v.begin(), v.end());
    return v;
}

void drop_graph(ochre_graph* g) {
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    g->exec = nullptr;
    g->graph = nullptr;
}

// Eager run -> plan -> sizing run of the planned chain -> capture.
int build(ochre_graph* g) {
    ochre_gpu_ctx* ctx = g->ctx;
    cudaStream_t s = ctx->own_stream;
    drop_graph(g);
    ctx->plan = nullptr;
    ochre_result res;
    int st = run_device(ctx, &g->batch, &res, s);
    if (st != OCHRE_OK) return st;
    const ochre_stats& es = ctx->stats;
    GraphPlan p{};
    p.fused = es.fused != 0;
    p.tiles = cap_of(es.n_tiles, g->headroom);
    if (!p.fused) {
        p.lines = cap_of(es.n_lines, g->headroom);
        p.entries = cap_of(es.n_entries, g->headroom);
        p.incs = cap_of(host_scalars(ctx)->inc_total, g->headroom, MAX_INCS);
        // key bits: the key space (areas of tile boxes) with headroom^2, up
        // to the next digit boundary (no extra sort pass for it), and never
        // into 64-bit keys when 32 hold the planning run
        const double want = (double)host_scalars(ctx)->keyspace * g->headroom * g->headroom;
        uint32_t kb = std::max<uint32_t>(es.key_bits, 1u);
        while (kb < 64 && std::ldexp(1.0, (int)kb) < want) kb++;
        kb = std::min<uint32_t>((kb + 7u) / 8u * 8u, 64u);
        if (es.key_bits <= 32 && kb > 32) kb = 32;
        p.key_bits = kb;
        p.rows = std::max<uint32_t>(host_scalars(ctx)->n_rows, 1u);
    }
    p.diff = g->is_diff ? &g->diff : nullptr;
    // stroked fills: the stroke stage's counts of the planning run
    p.stroke = g->batch.fill_width != nullptr;
    if (p.stroke) {
        p.stroke_poly = cap_of(ctx->stroke_counts[0], g->headroom);
        p.stroke_poly_floats = cap_of(ctx->stroke_counts[1], g->headroom, 0xffffffffull);
        p.stroke_cmds = cap_of(ctx->stroke_counts[2], g->headroom);
        p.stroke_floats = cap_of(ctx->stroke_counts[3], g->headroom, 0xffffffffull);
    }
    g->plan = p;
    ctx->plan = &g->plan;
    // sizing run: every buffer reaches its planned size before the capture
    st = planned_body(ctx, &g->batch, s);
    if (st == OCHRE_OK) st = cudaStreamSynchronize(s) == cudaSuccess ? OCHRE_OK : OCHRE_E_CUDA;
    if (st == OCHRE_OK) st = check_device_error(ctx);
    if (st != OCHRE_OK) {
        ctx->plan = nullptr;
        return st;
    }
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
        ctx->plan = nullptr;
        return OCHRE_E_CUDA;
    }
    const std::vector<void*> before = buffer_set(ctx);
    st = planned_body(ctx, &g->batch, s);
    cudaGraph_t graph = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(s, &graph);
    ctx->plan = nullptr;
    // a buffer that grew during the capture would leave earlier nodes on its
    // freed memory: the sizing run must have made every allocation
    if (st == OCHRE_OK && buffer_set(ctx) != before) st = OCHRE_E_CUDA;
    if (st != OCHRE_OK || ce != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        return st != OCHRE_OK ? st : OCHRE_E_CUDA;
    }
    g->graph = graph;
    g->kernels = ctx->launches;
    if (cudaGraphInstantiate(&g->exec, g->graph, 0) != cudaSuccess) {
        cudaGetLastError();
        drop_graph(g);
        return OCHRE_E_CUDA;
    }
    return OCHRE_OK;
}

// One replay; *overflow when the plan no longer holds the batch.
int replay(ochre_graph* g, cudaStream_t s, bool* overflow) {
    *overflow = false;
    OCHRE_CUDA_TRY(cudaGraphLaunch(g->exec, s));
    OCHRE_CUDA_TRY(cudaStreamSynchronize(s));
    const DevScalars* hs = host_scalars(g->ctx);
    if ((hs->err & ERR_CAPACITY) || (g->plan.fused && hs->fused_fallback)) {
        *overflow = true;
        return OCHRE_OK;
    }
    return check_device_error(g->ctx);
}

void fill_result(ochre_graph* g, ochre_result* out) {
    ochre_gpu_ctx* ctx = g->ctx;
    const DevScalars* hs = host_scalars(ctx);
    std::memset(out, 0, sizeof *out);
    ochre_stats st{};
    if (g->plan.fused) {
        st.n_tiles = hs->fused_tiles;
        st.n_spans = hs->fused_spans;
        st.fused = 1;
    } else {
        st.n_lines = hs->n_lines;
        st.n_entries = hs->n_entries;
        st.n_tiles = hs->n_tiles;
        st.n_spans = hs->n_spans;
        st.n_bins = hs->n_bins;
        st.key_bits = g->plan.key_bits;
        st.sort_passes = (g->plan.key_bits + 7) / 8;
    }
    st.n_launches = g->kernels;
    g->stats = st;
    out->n_tiles = (uint32_t)st.n_tiles;
    out->n_spans = (uint32_t)st.n_spans;
    out->tile_xy = ctx->out_tile_xy.as<int16_t>();
    out->tile_alpha = ctx->out_tile_alpha.as<uint8_t>();
    out->tile_cov = (ctx->flags & OCHRE_CTX_WANT_COV) ? ctx->out_tile_cov.as<float>() : nullptr;
    out->span_xy = ctx->out_span_xy.as<int16_t>();
    out->span_width = ctx->out_span_w.as<uint16_t>();
    out->span_tile = ctx->out_span_tile.as<uint32_t>();
    out->raster_tile_off = ctx->out_raster_tile_off.as<uint32_t>();
    out->raster_span_off = ctx->out_raster_span_off.as<uint32_t>();
}

}  // namespace

}  // namespace ochre

using namespace ochre;

extern "C" {

int ochre_graph_create(ochre_gpu_ctx* ctx, const ochre_batch* in, float headroom, ochre_graph** out) {
    if (!ctx || !in || !out) return OCHRE_E_INVALID;
    *out = nullptr;
    if (in->n_rasters == 0 || in->n_rasters > MAX_RASTERS || in->n_cmds > MAX_COUNT) return in->n_rasters ? OCHRE_E_CAPACITY : OCHRE_E_INVALID;
    if (in->raster_fill_off == nullptr && in->n_rasters != in->n_fills) return OCHRE_E_INVALID;
    if (!(headroom >= 1.0f) || headroom > 16.0f) return OCHRE_E_INVALID;
    ochre_graph* g = new (std::nothrow) ochre_graph();
    if (!g) return OCHRE_E_NOMEM;
    // stroked fills are planned on the general chain (their padded output
    // puts every pad command on one raster)
    const uint32_t chain = in->fill_width != nullptr ? OCHRE_CTX_CHAIN_ONLY : 0u;
    int st = ochre_gpu_create(&g->ctx, ctx->device, (ctx->flags & (OCHRE_CTX_WANT_COV | OCHRE_CTX_CHAIN_ONLY)) | chain);
    if (st != OCHRE_OK) {
        delete g;
        return st;
    }
    g->ctx->tune_fused_threads = ctx->tune_fused_threads;
    g->ctx->tune_fused_chunk = ctx->tune_fused_chunk;
    g->ctx->tune_chain_tiles_per_warp = ctx->tune_chain_tiles_per_warp;
    g->ctx->tune_chain_coverage_form = ctx->tune_chain_coverage_form;
    g->ctx->tune_chain_long_cells = ctx->tune_chain_long_cells;
    g->ctx->tune_sort_digit_bits = ctx->tune_sort_digit_bits;
    g->ctx->tune_chain_walk_refill = ctx->tune_chain_walk_refill;
    g->ctx->cov_signed = ctx->cov_signed;
    g->batch = *in;
    g->headroom = headroom;
    st = build(g);
    if (st != OCHRE_OK) {
        ochre_graph_destroy(g);
        return st;
    }
    *out = g;
    return OCHRE_OK;
}

int ochre_graph_create_diff(ochre_gpu_ctx* ctx, const ochre_batch* in, uint32_t w, uint32_t h, const float* target,
                            float* cov, float* dl_dcov, double* loss, float* dl_dpts, float* dl_dxf, float headroom,
                            ochre_graph** out) {
    if (!ctx || !in || !out || !loss) return OCHRE_E_INVALID;
    *out = nullptr;
    if (in->n_rasters == 0 || in->n_rasters > MAX_RASTERS || in->n_cmds > MAX_COUNT) return in->n_rasters ? OCHRE_E_CAPACITY : OCHRE_E_INVALID;
    if (in->raster_fill_off == nullptr && in->n_rasters != in->n_fills) return OCHRE_E_INVALID;
    if (in->fill_width != nullptr) return OCHRE_E_INVALID;   // stroked fills are not differentiated
    if (w > MAX_CANVAS || h > MAX_CANVAS || !(headroom >= 1.0f) || headroom > 16.0f) return OCHRE_E_INVALID;
    if (w && h && (!target || !cov || !dl_dcov)) return OCHRE_E_INVALID;
    if ((in->n_floats && !dl_dpts) || (in->n_fills && !dl_dxf)) return OCHRE_E_INVALID;
    ochre_graph* g = new (std::nothrow) ochre_graph();
    if (!g) return OCHRE_E_NOMEM;
    // the forward with signed tile coverage on the general chain, as the
    // eager differentiable entries run it
    int st = ochre_gpu_create(&g->ctx, ctx->device, OCHRE_CTX_WANT_COV | OCHRE_CTX_CHAIN_ONLY);
    if (st != OCHRE_OK) {
        delete g;
        return st;
    }
    g->ctx->tune_chain_tiles_per_warp = ctx->tune_chain_tiles_per_warp;
    g->ctx->tune_chain_coverage_form = ctx->tune_chain_coverage_form;
    g->ctx->tune_chain_long_cells = ctx->tune_chain_long_cells;
    g->ctx->tune_sort_digit_bits = ctx->tune_sort_digit_bits;
    g->ctx->tune_chain_walk_refill = ctx->tune_chain_walk_refill;
    g->ctx->cov_signed = true;
    g->batch = *in;
    g->headroom = headroom;
    g->is_diff = true;
    g->diff = DiffStep{w, h, target, cov, dl_dcov, loss, dl_dpts, dl_dxf};
    st = build(g);
    if (st != OCHRE_OK) {
        ochre_graph_destroy(g);
        return st;
    }
    *out = g;
    return OCHRE_OK;
}

int ochre_graph_launch(ochre_graph* g, ochre_result* out, void* stream) {
    if (!g || !out || !g->exec) return OCHRE_E_INVALID;
    if (cudaSetDevice(g->ctx->device) != cudaSuccess) return OCHRE_E_CUDA;
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : g->ctx->own_stream;
    bool overflow = false;
    int st = replay(g, s, &overflow);
    if (st != OCHRE_OK) return st;
    if (overflow) {
        // the batch outgrew the plan: re-plan from an eager run, replay once
        g->replans++;
        st = build(g);
        if (st != OCHRE_OK) return st;
        st = replay(g, s, &overflow);
        if (st != OCHRE_OK) return st;
        if (overflow) return OCHRE_E_CAPACITY;
    }
    fill_result(g, out);
    return OCHRE_OK;
}

int ochre_graph_last_stats(const ochre_graph* g, ochre_stats* out) {
    if (!g || !out) return OCHRE_E_INVALID;
    *out = g->stats;
    return OCHRE_OK;
}

int ochre_graph_info(const ochre_graph* g, uint32_t* kernels, uint32_t* replans, uint32_t* fused) {
    if (!g) return OCHRE_E_INVALID;
    if (kernels) *kernels = g->kernels;
    if (replans) *replans = g->replans;
    if (fused) *fused = g->plan.fused ? 1u : 0u;
    return OCHRE_OK;
}

void ochre_graph_destroy(ochre_graph* g) {
    if (!g) return;
    if (g->ctx) cudaSetDevice(g->ctx->device);
    drop_graph(g);
    ochre_gpu_destroy(g->ctx);
    delete g;
}

}  // extern "C"
