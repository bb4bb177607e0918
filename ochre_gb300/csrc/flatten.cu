// Stage 1: commands -> line segments (flattening).
//
// Reference: Rasterizer::fill / command (rasterizer.rs:145-165),
// PathCmd::transform (path.rs:16-37), PathCmd::flatten (path.rs:41-109),
// and the implicit closing lines of move_to / finish (rasterizer.rs:62-64,
// 181-183).
//
// A raster's line list is the sequence of its line_to calls.  Each command
// contributes, in order:
//   Move   : the closing line last -> first when last != first
//   Line   : last -> point
//   Quad   : n lines from the serial t recurrence (path.rs:52-57)
//   Cubic  : n lines (path.rs:65-73)
//   Conic  : 2 lines per subdivision leaf (path.rs:76-101)
//   Close  : nothing (rasterizer.rs:154 ignores it)
// plus, on the raster's last command, the final closing line of finish.
// `last` for a command is the transformed end point of the most recent
// earlier non-Close command of the raster (or (0,0)), `first` the point of
// the most recent earlier Move (or (0,0)); both come from one scan.
#include "common.cuh"
#include "flatten.cuh"
#include "internal.h"
#include "scan.cuh"

namespace ochre {


// Runs the flattening of one command, calling line(a, b) for each line_to
// in order.  Returns false when a cap was hit.
template <class Line>
__device__ bool flatten_cmd(const CmdCtx& k, Line line) {
    bool capped = false;
    V2 prev = k.last;
    auto to = [&](V2 p) { line(prev, p); prev = p; };
    switch (k.verb) {
    case V_MOVE:
        if (!veq(k.last, k.first)) line(k.last, k.first);
        break;
    case V_LINE:
        to(k.pt[0]);
        break;
    case V_QUAD: {
        const float dt = quad_dt(k.last, k.pt[0], k.pt[1]);
        float t = 0.0f;
        uint32_t n = 0;
        while (t < 1.0f) {
            t = rmin(__fadd_rn(t, dt), 1.0f);
            to(quad_point(t, k.last, k.pt[0], k.pt[1]));
            if (++n >= FLATTEN_CAP) { capped = true; break; }
        }
        break;
    }
    case V_CUBIC: {
        const float dt = cubic_dt(k.last, k.pt[0], k.pt[1], k.pt[2]);
        float t = 0.0f;
        uint32_t n = 0;
        while (t < 1.0f) {
            t = rmin(__fadd_rn(t, dt), 1.0f);
            to(cubic_point(t, k.last, k.pt[0], k.pt[1], k.pt[2]));
            if (++n >= FLATTEN_CAP) { capped = true; break; }
        }
        break;
    }
    case V_CONIC:
        conic_flatten(k.last, k.pt[0], k.pt[1], k.w, &capped, to);
        break;
    default:
        break;
    }
    if (k.last_of_raster) {
        // finish(): line_to(first) when last != first (rasterizer.rs:181-183)
        const V2 last_end = k.verb == V_CLOSE ? k.last : k.verb == V_CUBIC ? k.pt[2]
                          : k.verb == V_MOVE || k.verb == V_LINE ? k.pt[0] : k.pt[1];
        const V2 first_end = k.verb == V_MOVE ? k.pt[0] : k.first;
        if (!veq(last_end, first_end)) line(last_end, first_end);
    }
    return !capped;
}

// Line count of one command (the count pass never materialises points for
// curves: it only replays the t recurrence).
__device__ uint32_t count_cmd(const CmdCtx& k, bool* capped) {
    uint32_t n = 0;
    switch (k.verb) {
    case V_MOVE: n = veq(k.last, k.first) ? 0u : 1u; break;
    case V_LINE: n = 1; break;
    case V_QUAD: n = flatten_steps(quad_dt(k.last, k.pt[0], k.pt[1]), capped); break;
    case V_CUBIC: n = flatten_steps(cubic_dt(k.last, k.pt[0], k.pt[1], k.pt[2]), capped); break;
    case V_CONIC: conic_flatten(k.last, k.pt[0], k.pt[1], k.w, capped, [&](V2) { n++; }); break;
    default: break;
    }
    if (k.last_of_raster) {
        const V2 last_end = k.verb == V_CLOSE ? k.last : k.verb == V_CUBIC ? k.pt[2]
                          : k.verb == V_MOVE || k.verb == V_LINE ? k.pt[0] : k.pt[1];
        const V2 first_end = k.verb == V_MOVE ? k.pt[0] : k.first;
        if (!veq(last_end, first_end)) n++;
    }
    return n;
}

// Line counts folded straight into the line-offset scan.
struct CountIn {
    BatchView b;
    uint32_t* err;
    __device__ __forceinline__ uint32_t operator()(uint64_t i) const {
        const CmdCtx k = load_cmd(b, (uint32_t)i);
        if (!k.ok) { atomicOr(err, ERR_INVALID); return 0u; }
        bool capped = false;
        const uint32_t n = count_cmd(k, &capped);
        if (capped) atomicOr(err, ERR_LIMIT);
        return n;
    }
};
struct OffOut {
    uint32_t* off;
    __device__ __forceinline__ void operator()(uint64_t i, uint32_t ex, uint32_t) const { off[i] = ex; }
};
struct Load32 {
    const uint32_t* v;
    __device__ __forceinline__ uint32_t operator()(uint64_t i) const { return v[i]; }
};

// One thread per command: the line counts of a batch with few commands
// (a scan would give each of a handful of threads eight serial t loops).
template <class In>
__global__ void __launch_bounds__(128) k_count_each(uint64_t n, In in, uint32_t* __restrict__ out) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = in(i);
}
// Below this many scan tiles the counts get their own kernel.
constexpr uint64_t SPLIT_COUNT_TILES = 256;

// Lines of more than long_cells cells (walk_cells) are also queued for the
// long-line walkers of the DDA stage (long_cells 0: none are).
__global__ void k_cmd_emit(BatchView b, const uint32_t* __restrict__ line_off, uint32_t n_lines_cap,
                           float4* __restrict__ lines, uint32_t* __restrict__ line_raster, uint32_t long_cells,
                           uint32_t* __restrict__ long_lines, uint32_t* n_long, uint32_t* err) {
    const uint64_t c = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (c >= b.n_cmds) return;
    const CmdCtx k = load_cmd(b, (uint32_t)c);
    if (!k.ok) return;
    uint32_t o = line_off[c];
    flatten_cmd(k, [&](V2 a, V2 p) {
        if (o < n_lines_cap) {
            const float4 l = make_float4(a.x, a.y, p.x, p.y);
            lines[o] = l;
            line_raster[o] = k.raster;
            if (long_cells && walk_cells(l) > long_cells) long_lines[atomicAdd(n_long, 1u)] = o;
        } else {
            atomicOr(err, ERR_CAPACITY);
        }
        o++;
    });
}

int stage_flatten(ochre_gpu_ctx* ctx, const ochre_batch* in, cudaStream_t s, uint32_t* n_lines) {
    const uint64_t n = in->n_cmds;
    DevScalars* ds = dev_scalars(ctx);
    *n_lines = 0;
    if (n == 0) return OCHRE_OK;
    OCHRE_CUDA_TRY(ctx->cmd_foff.ensure(n * 4));
    OCHRE_CUDA_TRY(ctx->cmd_mv.ensure(n * 4));
    OCHRE_CUDA_TRY(ctx->cmd_ep.ensure(n * 4));
    OCHRE_CUDA_TRY(ctx->cmd_line_off.ensure(n * 4));
    OCHRE_CUDA_TRY(ctx->scan_status.ensure(scan_tiles(n) * sizeof(ScanStatus<CmdScan>)));

    CmdScan total_id{0, 0, 0};
    OCHRE_LAUNCH(ctx, "cmd_scan", s, OCHRE_CUDA_TRY(launch_scan<CmdScan>(n, CmdIn{in->verbs, &ds->err},
                                        CmdOut{ctx->cmd_foff.as<uint32_t>(), ctx->cmd_mv.as<uint32_t>(),
                                               ctx->cmd_ep.as<uint32_t>()},
                                        OpCmd{}, total_id, ctx->scan_status.p, &ds->ticket,
                                        reinterpret_cast<CmdScan*>(&ds->n_floats), &ds->err, s)));

    // A command whose points lie beyond the point array is flagged invalid
    // by the kernels that read it (load_cmd), reported at the next read-back.
    const GraphPlan* plan = ctx->plan;
    int st = OCHRE_OK;
    const DevScalars* hs = host_scalars(ctx);

    wait_inputs(ctx, s);   // the counts read points
    BatchView b{in->verbs, in->pts, in->fill_cmd_off, in->fill_xf, in->fill_flags, in->raster_fill_off,
                in->n_fills, in->n_rasters, n, ctx->cmd_foff.as<uint32_t>(), ctx->cmd_mv.as<uint32_t>(),
                ctx->cmd_ep.as<uint32_t>(), in->n_floats};
    if (scan_tiles(n) < SPLIT_COUNT_TILES) {
        // counts first (one thread per command), then the offsets in place
        OCHRE_LAUNCH(ctx, "flatten_count", s, k_count_each<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(
            n, CountIn{b, &ds->err}, ctx->cmd_line_off.as<uint32_t>()));
        OCHRE_CUDA_TRY(cudaGetLastError());
        OCHRE_LAUNCH(ctx, "flatten_count_scan", s, OCHRE_CUDA_TRY(launch_scan<uint32_t>(
            n, Load32{ctx->cmd_line_off.as<uint32_t>()}, OffOut{ctx->cmd_line_off.as<uint32_t>()}, OpSumU32{}, 0u,
            ctx->scan_status.p, &ds->ticket, &ds->n_lines, &ds->err, s)));
    } else {
        OCHRE_LAUNCH(ctx, "flatten_count_scan", s, OCHRE_CUDA_TRY(launch_scan<uint32_t>(
            n, CountIn{b, &ds->err}, OffOut{ctx->cmd_line_off.as<uint32_t>()}, OpSumU32{}, 0u, ctx->scan_status.p,
            &ds->ticket, &ds->n_lines, &ds->err, s)));
    }
    uint32_t L;
    if (plan) {
        // the line count stays on the device; above the plan it is zeroed
        OCHRE_LAUNCH(ctx, "plan_lines", s, OCHRE_CUDA_TRY(launch_plan_cap(ctx, &ds->n_lines, plan->lines, s)));
        L = plan->lines;
    } else {
        st = read_scalars(ctx, s);
        if (st != OCHRE_OK) return st;
        st = check_device_error(ctx);
        if (st != OCHRE_OK) return st;
        L = hs->n_lines;
    }
    *n_lines = L;
    if (L == 0) return OCHRE_OK;
    if (L > MAX_COUNT) return OCHRE_E_CAPACITY;
    OCHRE_CUDA_TRY(ctx->lines.ensure((size_t)L * sizeof(float4)));
    OCHRE_CUDA_TRY(ctx->line_raster.ensure((size_t)L * 4));
    const uint32_t long_cells = (uint32_t)ctx->tune_chain_long_cells;
    if (long_cells) OCHRE_CUDA_TRY(ctx->long_lines.ensure((size_t)L * 4));
    OCHRE_CUDA_TRY(cudaMemsetAsync(&ds->n_long, 0, 4, s));
    const unsigned blocks = (unsigned)((n + 255) / 256);
    OCHRE_LAUNCH(ctx, "flatten_emit", s, k_cmd_emit<<<blocks, 256, 0, s>>>(
        b, ctx->cmd_line_off.as<uint32_t>(), L, ctx->lines.as<float4>(), ctx->line_raster.as<uint32_t>(), long_cells,
        long_cells ? ctx->long_lines.as<uint32_t>() : nullptr, &ds->n_long, &ds->err));
    OCHRE_CUDA_TRY(cudaGetLastError());
    return OCHRE_OK;
}

}  // namespace ochre
