"""Benchmark of the GB300 rasterization path (ochre Rasterizer::fill -> finish).

Workload (default): the glyph-like text run — 100,000 independent closed
paths of 8-40 quadratics over 1-3 contours under random affine transforms on
a 4096x4096 canvas (seeded synthetic data, one rasterizer per path).  A step
rasterizes the whole batch: every path's flatten -> DDA binning -> sort ->
tile coverage -> spans, producing the tiles and spans of every path.

  value  : paths/s with the batch resident in HBM (CUDA events on the
           launching stream; L2 flushed between timed steps).
  e2e    : paths/s through the host C-ABI entry point (ochre_gpu_rasterize)
           from pinned host buffers, every input brought to the GPU (points
           read in place over the host link, the rest copied) and all tiles
           and spans written to host memory inside the timed region.
  --impl reference : the reference's CPU algorithm (the oracle restatement,
           all host threads) on the same workload.

The same JSON line also carries the extension workloads (uneven-size mix
against one call per path, strokes, compositing, the differentiable render +
loss + backward with its gradient checks and compulsory-byte roofline, and
CUDA-graph replay against the eager call), the SM clocks sampled during the
timed region (raw samples in $OCHRE_BENCH_CLOCKS_DIR, default /tmp) and the
kernel launch count.

Multi-GPU: paths are independent, so each rank rasterizes its own batch
(weak scaling, no collective on the data path); value = all paths / max time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "tiles/s & paths/s batched vs plain GPU at ≤1 LSB alpha; fwd+bwd scenes/s"
PEAKS_FALLBACK = {"hbm_gbs": 6800.0}
NOMINAL_HBM_GBS = 7900.0   # GB300 HBM3e, nominal


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d, "measured"
    return PEAKS_FALLBACK, "fallback"


def make_workload(name: str, n: int, seed: int):
    from ochre_gb300 import workloads as W
    if name == "diff_union":
        return W.diff_union(n_paths=n)
    if name == "diff_scenes":
        return W.diff_scenes(n_scenes=n)
    if name == "glyph_run":
        return W.glyph_run(n_paths=n, seed=seed)
    if name == "cubic_boxes":
        return W.cubic_boxes(n_paths=n, seed=seed)
    if name == "uneven_mix":
        return W.uneven_mix(n_paths=n, seed=seed)
    if name == "stroke_run":
        return W.stroke_run(n_paths=n, seed=seed)
    raise SystemExit(f"unknown workload {name}")


def output_bytes(n_tiles: int, n_spans: int, n_rasters: int) -> int:
    """Compulsory output: 68 B per tile (64 alpha + 2 x i16 position), 6 B per
    span (i16 x, i16 y, u16 width)."""
    return 68 * n_tiles + 6 * n_spans


def kernel_bytes(name: str, st: dict, batch) -> int:
    """Bytes each kernel of the chain must move for its job (every input array
    read once, every output array written once).  Used as the roofline
    numerator of the dominant kernel."""
    C, R = batch.n_cmds, batch.n_rasters
    L, E, T, B, N = st["n_lines"], st["n_entries"], st["n_tiles"], st["n_bins"], st["n_spans"]
    kb = 8 if st["key_bits"] > 32 else 4
    if name == "cmd_scan":
        return C * 1 + C * 12
    if name == "flatten_count":
        return batch.verbs.nbytes + batch.pts.nbytes + 24 * batch.n_fills + C * 12 + C * 4
    if name == "flatten_count_scan":
        return batch.verbs.nbytes + batch.pts.nbytes + 24 * batch.n_fills + C * 12 + C * 4
    if name == "flatten_emit":
        return batch.verbs.nbytes + batch.pts.nbytes + 24 * batch.n_fills + C * 16 + L * 20
    I = st.get("n_incs", 0)
    if name == "dda_count":
        # line + raster read, entry and increment counts written, raster boxes
        return L * 20 + L * 8 + R * 16
    if name == "dda_offset_scan":
        return L * 16
    if name == "dda_emit":
        # line, raster, both offsets; raster box and key base; every entry's
        # key and value, every bin's record (16 B), every increment (8 B)
        return L * 28 + R * 24 + E * (kb + 4) + B * 16 + I * 8
    if name == "sort_onesweep":
        return 2 * E * (kb + 4)
    if name == "sort_hist":
        return E * kb
    if name == "tile_head_scan":
        return E * (kb + 4) + T * 4
    if name == "tile_info":
        # head, bin count and winding of the tile (and the next tile's bin
        # count); value and record of its head and its predecessor's; info out
        return T * 16 + T * 2 * (4 + 16) + T * 32 + R * 8
    if name == "tile_coverage":
        # entries: value 4; bins: record 16; increments 8; tiles: info 32 +
        # 68 out + 12 span slot
        return E * 4 + B * 16 + I * 8 + T * (32 + 68 + 12)
    if name == "span_scan":
        return T * 4 + T * 8 + N * 10 + R * 4
    if name == "raster_fused":
        # the whole path in one kernel: compulsory input + output bytes, and
        # the float offset of every command (from the command scan)
        return batch.input_bytes() + 4 * (batch.n_fills + 1) + 4 * C + 68 * T + 10 * N + 8 * (R + 1)
    if name == "fused_float_scan":
        return C * 1 + C * 4
    return 0


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int, path: str):
        self.path = path
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self) -> dict:
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def cpu_baseline(batch, reps: int = 3) -> dict:
    import numpy as np
    import oracle
    threads = os.cpu_count() or 1
    with np.errstate(all="ignore"):
        oracle.run(batch, threads=threads)  # warm
        t0 = time.perf_counter()
        for _ in range(reps):
            r = oracle.run(batch, threads=threads)
        dt = (time.perf_counter() - t0) / reps
    n_tiles = int(len(r["tile_xy"]))
    # one core, on the first 10,000 paths (a few seconds)
    from ochre_gb300.batch import subset
    n1 = min(batch.n_rasters, 10000)
    one = subset(batch, range(n1))
    with np.errstate(all="ignore"):
        t0 = time.perf_counter()
        r1 = oracle.run(one, threads=1)
        dt1 = time.perf_counter() - t0
    return {"value": batch.n_rasters / dt, "unit": "paths/s", "cores": threads, "kind": "port",
            "tiles_per_s": n_tiles / dt, "cpu_model": _cpu_model(),
            "sample": f"the full workload ({batch.n_rasters} paths) x {reps} repetitions, "
                      f"oracle/ochre_oracle.c on {threads} threads",
            "one_core": {"value": n1 / dt1, "unit": "paths/s", "tiles_per_s": len(r1["tile_xy"]) / dt1,
                         "sample": f"the first {n1} paths of the workload, one thread"}}


def _cpu_model() -> str:
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                key = line.split(":")[0].strip().lower()
                if key in ("model name", "cpu model", "hardware"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.processor() or platform.machine()


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
            dist.init_process_group("nccl")
        else:   # host-only ranks (the reference arm, tests)
            dist.init_process_group("gloo")
    return ws, rank, local


def reduce_max(x: float, ws: int) -> float:
    """Max over ranks (the timing rule: the slowest rank's time)."""
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], device=dev, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws: int):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def run_reference(args, ws, rank):
    if rank != 0:
        return
    import numpy as np
    import oracle
    batch = make_workload(args.workload, args.n_paths, args.seed)
    threads = os.cpu_count() or 1
    with np.errstate(all="ignore"):
        for _ in range(args.warmup):
            oracle.run(batch, threads=threads)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            r = oracle.run(batch, threads=threads)
        dt = time.perf_counter() - t0
    n_tiles = int(len(r["tile_xy"]))
    value = batch.n_rasters * args.steps / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "paths/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": bench_config(args, batch.n_rasters, ws),
        "tiles_per_s": n_tiles * args.steps / dt,
        "cpu_baseline": {"value": value, "unit": "paths/s", "cores": threads, "kind": "port",
                         "sample": f"the full workload ({batch.n_rasters} paths) per step, "
                                   f"oracle/ochre_oracle.c (strict-f32 restatement of the reference) on {threads} threads"},
        "e2e": {"value": value, "unit": "paths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


L2_RULE = "flushed (256 MiB write) between timed GPU steps, outside the events"
MASK_EPS = 1e-3   # gradient check: |S| this close to a kink of min(|S|, 1) is left out


def bench_config(args, n_paths: int, ws: int) -> dict:
    """The workload of a bench line; both arms print the same dict."""
    return {"workload": args.workload, "n_paths_per_gpu": n_paths, "seed": args.seed,
            "parallelism": f"replicas{ws}" if ws > 1 else "single", "l2": L2_RULE}


def _event_ms(fn, stream, flush, reps):
    """Median device time of fn() over reps calls, L2 flushed before each."""
    import torch
    out = []
    for i in range(reps):
        flush.fill_(i & 0xff)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        torch.cuda.synchronize()
        out.append(a.elapsed_time(b))
    return statistics.median(out)


def _kernel_shares(ctx, fn):
    import torch
    ctx.set_profile(True)
    fn()
    torch.cuda.synchronize()
    per = {}
    for name, ms in ctx.timings():
        d = per.setdefault(name, [0.0, 0])
        d[0] += ms
        d[1] += 1
    ctx.set_profile(False)
    total = sum(v[0] for v in per.values()) or 1.0
    return sorted(({"kernel": k, "ms": v[0], "launches": v[1], "share": v[0] / total} for k, v in per.items()),
                  key=lambda x: -x["ms"])


def bench_uneven(ctx, stream, flush, steps, peak):
    """Batched uneven-size mix (20,000 paths, lognormal segment counts) in one
    call, against the plain chain run once per path (sampled)."""
    import numpy as np
    import torch
    from ochre_gb300 import DeviceBatch, batch as B, workloads as W
    bt = W.uneven_mix()
    db = DeviceBatch(bt, ctx.device)
    sp = stream.cuda_stream
    for _ in range(2):
        ctx.rasterize_device(db, sp)
    st = ctx.stats()
    ms = _event_ms(lambda: ctx.rasterize_device(db, sp), stream, flush, max(3, min(steps, 5)))
    kernels = _kernel_shares(ctx, lambda: ctx.rasterize_device(db, sp))
    dom = kernels[0]
    dom_bytes = kernel_bytes(dom["kernel"], st, bt) / max(1, dom["launches"])
    dom_ms = dom["ms"] / max(1, dom["launches"])
    ach = dom_bytes / (dom_ms / 1e3) / 1e9 if dom_ms > 0 else 0.0
    # the plain per-path chain: one chain (flatten -> DDA -> sort -> tiles) per path
    rng = np.random.default_rng(0)
    idx = np.sort(rng.choice(bt.n_rasters, 500, replace=False))
    subs = [DeviceBatch(B.subset(bt, [int(i)]), ctx.device) for i in idx]
    ctx.set_chain_only(True)
    for d in subs[:10]:
        ctx.rasterize_device(d, sp)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for d in subs:
        ctx.rasterize_device(d, sp)
    torch.cuda.synchronize()
    per_path_s = (time.perf_counter() - t0) / len(subs)
    chain_ms = _event_ms(lambda: ctx.rasterize_device(db, sp), stream, flush, 3)
    ctx.set_chain_only(False)
    # parity (the metric's bar): the same 500 sampled paths, rasterized in one
    # batched call, against the oracle
    import oracle
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from compare import compare
    samp = B.subset(bt, [int(i) for i in idx])
    got = ctx.rasterize(samp)
    with np.errstate(all="ignore"):
        cst = compare(got, oracle.run(samp, threads=os.cpu_count() or 1), samp.n_rasters)
    parity = {"sample_paths": samp.n_rasters, "tiles": cst["tiles"], "spans": cst["spans"],
              "tiles_spans_exact": True, "alpha_max_lsb": cst["max_lsb"],
              "alpha_diff_fraction": cst["diff_fraction"],
              "note": "500 paths sampled from the mix, one batched call; full size in tests/test_parity_gpu.py"}
    comp = bt.input_bytes() + output_bytes(st["n_tiles"], st["n_spans"], bt.n_rasters)
    return {
        "workload": "uneven_mix: 20000 paths, lognormal(median 32) segments clipped to 4-20000, 8192x8192",
        "paths_per_s": bt.n_rasters / (ms / 1e3), "tiles_per_s": st["n_tiles"] / (ms / 1e3), "ms_per_step": ms,
        "tiles": st["n_tiles"], "spans": st["n_spans"], "lines": st["n_lines"], "sort_entries": st["n_entries"],
        "path": "fused" if st.get("fused") else "chain", "launches_per_step": st["n_launches"],
        "plain_per_path_chain": {"paths_per_s": 1.0 / per_path_s, "ms_per_path": 1e3 * per_path_s,
                                 "sample_paths": len(subs), "timing": "host wall clock over the sample"},
        "speedup_vs_per_path_chain": (bt.n_rasters / (ms / 1e3)) * per_path_s,
        "one_call_chain_ms": chain_ms,
        "parity": parity,
        "roofline": {"kernel": dom["kernel"], "achieved_gbs": ach, "frac": ach / peak,
                     "frac_of_nominal": ach / NOMINAL_HBM_GBS,
                     "algorithmic_bytes_per_launch": dom_bytes, "ms_per_launch": dom_ms},
        "path_roofline": {"compulsory_bytes": comp, "achieved_gbs": comp / (ms / 1e3) / 1e9,
                          "frac": comp / (ms / 1e3) / 1e9 / peak},
        "kernels": kernels[:8],
    }


def bench_configs(ctx, stream, flush, peak, glyphs, scenes):
    """Every seeded configuration rasterized (fill -> finish: tiles and spans,
    the reference's output) three ways: on the GPU in one batched call
    (device-resident inputs, L2 flushed, CUDA events), through the plain
    general chain once per raster (a sample, host wall clock per call), and
    by the CPU port (oracle/ochre_oracle.c) on all host cores and on one
    (bounded samples, stated per row)."""
    import numpy as np
    import torch
    import oracle
    from ochre_gb300 import DeviceBatch, batch as B, workloads as W
    sp = stream.cuda_stream
    cores = os.cpu_count() or 1
    rows = []
    cfgs = [
        ("cubic_boxes", "1,000 closed paths x 16 cubics in 512^2 boxes on 2048^2", W.cubic_boxes(), 200, 200),
        ("glyph_run", "100,000 glyph-like paths, 8-40 quadratics", glyphs, 1000, 10000),
        ("uneven_mix", "20,000 paths, lognormal segment counts (median 32, 4-20,000)", W.uneven_mix(), 200, 100),
        ("diff_union", "256 paths x 32 cubics in one raster, 1024^2", W.diff_union(), 1, 1),
        ("diff_scenes", f"{scenes.n_rasters:,} scenes of 512^2, 8-512 paths each", scenes, 64, 16),
    ]
    rng = np.random.default_rng(0)
    for name, what, b, n_plain, n_one in cfgs:
        db = DeviceBatch(b, ctx.device)
        for _ in range(2):
            ctx.rasterize_device(db, sp)
        st = ctx.stats()
        ms = _event_ms(lambda: ctx.rasterize_device(db, sp), stream, flush, 5)
        # the plain chain once per raster, on a sample of the rasters
        idx = np.sort(rng.choice(b.n_rasters, min(n_plain, b.n_rasters), replace=False))
        subs = [DeviceBatch(B.subset(b, [int(i)]), ctx.device) for i in idx]
        ctx.set_chain_only(True)
        for d in subs[:5]:
            ctx.rasterize_device(d, sp)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for d in subs:
            ctx.rasterize_device(d, sp)
        torch.cuda.synchronize()
        plain_s = (time.perf_counter() - t0) / len(subs)
        ctx.set_chain_only(False)
        del subs, db
        # the CPU port: the whole configuration on every core, a prefix on one
        with np.errstate(all="ignore"):
            t0 = time.perf_counter()
            oracle.run(b, threads=cores)
            cpu_all_s = time.perf_counter() - t0
            one = B.subset(b, list(range(min(n_one, b.n_rasters))))
            t0 = time.perf_counter()
            oracle.run(one, threads=1)
            cpu_one_s = time.perf_counter() - t0
        comp = b.input_bytes() + output_bytes(st["n_tiles"], st["n_spans"], b.n_rasters)
        rows.append({
            "config": name, "workload": what, "rasters": b.n_rasters, "tiles": st["n_tiles"], "spans": st["n_spans"],
            "path": "fused" if st.get("fused") else "chain",
            "gpu_batched": {"rasters_per_s": b.n_rasters / (ms / 1e3), "tiles_per_s": st["n_tiles"] / (ms / 1e3),
                            "ms_per_call": ms},
            "gpu_plain_per_raster": {"rasters_per_s": 1.0 / plain_s, "sample_rasters": len(idx)},
            "batched_over_plain": (b.n_rasters / (ms / 1e3)) * plain_s,
            "cpu_all_cores": {"rasters_per_s": b.n_rasters / cpu_all_s, "cores": cores,
                              "sample": f"all {b.n_rasters} rasters, once"},
            "cpu_one_core": {"rasters_per_s": one.n_rasters / cpu_one_s, "sample": f"the first {one.n_rasters} rasters"},
            "gpu_over_cpu_all_cores": cpu_all_s / (ms / 1e3),
            "path_roofline": {"compulsory_bytes": comp, "achieved_gbs": comp / (ms / 1e3) / 1e9,
                              "frac": comp / (ms / 1e3) / 1e9 / peak},
        })
    return {"note": "rasters = paths (scenes for diff_scenes); GPU batched by CUDA events with device-resident "
                    "inputs and L2 flushed; plain per-raster and CPU by host wall clock; cpu_model "
                    + _cpu_model(), "rows": rows}


def bench_svg_documents(ctx, stream, flush):
    """The reference's example documents (examples/res/*.svg, read by this
    project's SVG reader into the committed fixture tests/golden/svg_docs.npz):
    every painted path one raster, rasterized in one call and composited onto
    the document's canvas (CUDA events, L2 flushed), against the CPU port on
    all host cores."""
    import numpy as np
    import torch
    import oracle
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from golden.make_svg_docs import load
    from ochre_gb300 import DeviceBatch
    sp = stream.cuda_stream
    cores = os.cpu_count() or 1
    out = []
    for name in ("tiger", "calabi_yau", "lorem_ipsum"):
        b, colors, (w, h), _ = load(name)
        W, H = int(w or 1024), int(h or 1024)
        db = DeviceBatch(b, ctx.device)
        for _ in range(2):
            ctx.rasterize_device(db, sp)
        st = ctx.stats()
        ms = _event_ms(lambda: ctx.rasterize_device(db, sp), stream, flush, 5)
        col = torch.as_tensor(np.ascontiguousarray(colors), device=f"cuda:{ctx.device}")
        canvas = torch.full((H, W, 4), 255, dtype=torch.uint8, device=col.device)
        r = ctx.rasterize_device(db, sp)
        comp_ms = _event_ms(lambda: ctx.composite(r, b.n_rasters, col, canvas, stream=sp), stream, flush, 5)
        with np.errstate(all="ignore"):
            oracle.run(b, threads=cores)
            t0 = time.perf_counter()
            oracle.run(b, threads=cores)
            cpu_s = time.perf_counter() - t0
        out.append({"document": name, "rasters": b.n_rasters, "commands": b.n_cmds, "tiles": st["n_tiles"],
                    "spans": st["n_spans"], "path": "fused" if st.get("fused") else "chain",
                    "canvas": [W, H], "rasterize_ms": ms, "composite_ms": comp_ms,
                    "cpu_rasterize_ms": 1e3 * cpu_s, "cpu_cores": cores,
                    "gpu_over_cpu": 1e3 * cpu_s / ms})
    return {"note": "GPU by CUDA events (device-resident inputs, L2 flushed); CPU port by host wall clock, "
                    "rasterization only", "documents": out}


def bench_stroke(ctx, stream, flush, steps):
    """Stroked paths (Rasterizer::stroke): 20,000 rasters of 2-24 mixed
    segments, widths 0.5-8 px; the device stroke stage plus the fill path,
    with parity on a 1,000-path sample."""
    import numpy as np

    import oracle
    from ochre_gb300 import DeviceBatch, batch as B, workloads as W
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from compare import compare
    bt = W.stroke_run()
    db = DeviceBatch(bt, ctx.device)
    sp = stream.cuda_stream
    for _ in range(2):
        ctx.rasterize_device(db, sp)
    st = ctx.stats()
    ms = _event_ms(lambda: ctx.rasterize_device(db, sp), stream, flush, max(3, min(steps, 10)))
    samp = B.subset(bt, list(range(0, bt.n_rasters, 20)))
    with np.errstate(all="ignore"):
        cst = compare(ctx.rasterize(samp), oracle.run(samp, threads=os.cpu_count() or 1), samp.n_rasters)
    return {"workload": "stroke_run: 20000 stroked paths, 2-24 segments, width 0.5-8 px", "paths_per_s":
            bt.n_rasters / (ms / 1e3), "ms_per_step": ms, "tiles": st["n_tiles"], "path": "fused" if st.get("fused")
            else "chain", "parity_sample": {"paths": samp.n_rasters, "tiles_spans_exact": True,
                                           "alpha_max_lsb": cst["max_lsb"], "alpha_diff_fraction": cst["diff_fraction"]},
            "kernels": _kernel_shares(ctx, lambda: ctx.rasterize_device(db, sp))[:6]}


def bench_composite(ctx, stream, flush, steps):
    """Headless compositing (the reference example's GL draw, restated) of the
    glyph run's 100,000 rasters onto a 4096x4096 RGBA8 canvas in raster order,
    with a bit-exact check against the oracle's compositing of the same
    rasterization on a 4,000-raster sample."""
    import numpy as np
    import torch

    import oracle
    from ochre_gb300 import DeviceBatch, batch as B, workloads as W
    sp = stream.cuda_stream
    bt = W.glyph_run()
    rng = np.random.default_rng(9)
    colors_np = rng.integers(0, 256, size=(bt.n_rasters, 4), dtype=np.uint8)
    colors = torch.as_tensor(colors_np, device=f"cuda:{ctx.device}")
    canvas = torch.full((4096, 4096, 4), 255, dtype=torch.uint8, device=f"cuda:{ctx.device}")
    r = ctx.rasterize_device(DeviceBatch(bt, ctx.device), sp)
    st = ctx.stats()
    for _ in range(2):
        ctx.composite(r, bt.n_rasters, colors, canvas, sp)
    ms = _event_ms(lambda: ctx.composite(r, bt.n_rasters, colors, canvas, sp), stream, flush, max(3, min(steps, 10)))
    kernels = _kernel_shares(ctx, lambda: ctx.composite(r, bt.n_rasters, colors, canvas, sp))
    # parity on a sample: GPU rasterization composited on the GPU and by the oracle
    samp = B.subset(bt, range(4000))
    rs = ctx.rasterize_device(DeviceBatch(samp, ctx.device), sp)
    res = ctx.device_result_to_numpy(rs, samp.n_rasters)
    cv = torch.full((4096, 4096, 4), 255, dtype=torch.uint8, device=f"cuda:{ctx.device}")
    ctx.composite(rs, samp.n_rasters, colors[:samp.n_rasters].contiguous(), cv, sp)
    torch.cuda.synchronize()
    want = oracle.composite(res, samp.n_rasters, colors_np[:samp.n_rasters], 4096, 4096)
    exact = bool(np.array_equal(cv.cpu().numpy(), want))
    return {"workload": "glyph_run: 100000 rasters (2.1 M tiles, 254 k spans) composited onto 4096x4096 RGBA8",
            "ms_per_step": ms, "rasters_per_s": bt.n_rasters / (ms / 1e3), "tiles": st["n_tiles"],
            "spans": st["n_spans"], "parity_sample": {"rasters": samp.n_rasters, "bit_exact": exact},
            "kernels": kernels[:6]}


def bench_graph(ctx, stream, steps):
    """CUDA-graph replay (ochre_graph_launch) against the eager chain
    (ochre_gpu_rasterize_device) on batches rasterized again and again with
    the same structure: host wall clock per call, each call ending with its
    results on the device and the host synchronised."""
    import numpy as np
    import torch
    from ochre_gb300 import DeviceBatch, batch as B, workloads as W
    sp = stream.cuda_stream
    um = W.uneven_mix(n_paths=64, seed=3)
    sizes = np.diff(um.fill_cmd_off)
    mid = int(np.argsort(sizes)[len(sizes) // 2])
    cases = [
        ("one glyph", B.subset(W.glyph_run(n_paths=8, seed=2), [0])),
        ("one uneven-mix path (median size)", B.subset(um, [mid])),
        ("glyph run, 1,000 paths", W.glyph_run(n_paths=1000, seed=2)),
        ("union of 256 cubic fills on 1024x1024", W.diff_union()),
        ("uneven mix, 1,000 paths", W.uneven_mix(n_paths=1000, seed=4)),
        ("stroke run, 1,000 stroked paths", W.stroke_run(n_paths=1000, seed=4)),
    ]
    reps = max(30, 5 * steps)

    def per_call(fn):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        return (time.perf_counter() - t0) / reps * 1e3

    out = []
    for name, b in cases:
        db = DeviceBatch(b, ctx.device)
        eager_r = ctx.rasterize_device(db, sp)
        n_tiles = eager_r.n_tiles
        g = ctx.graph(db)
        try:
            r = g.launch(sp)
            assert r.n_tiles == n_tiles and g.info()["replans"] == 0, (name, r.n_tiles, n_tiles)
            eager_ms = per_call(lambda: ctx.rasterize_device(db, sp))
            eager_launches = ctx.stats()["n_launches"]
            graph_ms = per_call(lambda: g.launch(sp))
            info = g.info()
            out.append({"batch": name, "rasters": b.n_rasters, "tiles": int(n_tiles),
                        "form": "fused" if info["fused"] else "chain", "eager_ms_per_call": eager_ms,
                        "graph_ms_per_call": graph_ms, "speedup": eager_ms / graph_ms,
                        "eager_launches": eager_launches, "graph_kernels": info["kernels"]})
        finally:
            g.close()
    # the whole differentiable step (forward with signed coverage, coverage
    # render, L2 loss, backward) on the 256-path union, 1024^2
    b, w = W.diff_union(), 1024
    db = DeviceBatch(b, ctx.device)
    tgt = ctx.render_coverage(DeviceBatch(W.diff_union(perturb=2.0), ctx.device), w, w, stream=sp).clone()
    cov, dl = torch.empty_like(tgt), torch.empty_like(tgt)

    def eager_step():
        ctx.render_coverage(db, w, w, cov, stream=sp)
        ctx.l2_loss(cov, tgt, dl, stream=sp)
        ctx.fill_backward(db, w, w, dl, stream=sp)
        torch.cuda.synchronize()

    g = ctx.graph_diff(db, w, w, tgt)
    try:
        eager_ms = per_call(eager_step)
        graph_ms = per_call(lambda: g.launch(sp))
        out.append({"batch": "differentiable step: union of 256 cubic fills on 1024x1024 (render, loss, backward)",
                    "rasters": 1, "form": "chain", "eager_ms_per_call": eager_ms, "graph_ms_per_call": graph_ms,
                    "speedup": eager_ms / graph_ms, "graph_kernels": g.info()["kernels"]})
    finally:
        g.close()
    return {"timing": f"host wall clock, mean of {reps} calls after 3 warm-up calls", "cases": out}


def bench_differentiable(ctx, stream, flush, steps, n_scenes, scenes=None):
    """Forward (coverage render + L2 loss) and forward + backward scenes/s on
    the single-raster union (256 paths x 32 cubics, 1024^2) and on batched
    scenes (n_scenes x 512^2), with a gradient check against the FP64
    reference on the union and on the first scenes of the batch."""
    import copy

    import numpy as np
    import torch

    import oracle
    from ochre_gb300 import DeviceBatch, batch as B, workloads as W
    out = {}
    sp = stream.cuda_stream
    cases = [("diff_union", W.diff_union(), W.diff_union(perturb=2.0), 1024, 1024)]
    t0 = time.time()
    sc = scenes if scenes is not None else W.diff_scenes(n_scenes=n_scenes)
    pert = copy.copy(sc)
    pert.pts = (sc.pts + np.random.default_rng(4).normal(0, 2.0, sc.pts.shape)).astype(np.float32)
    gen_s = time.time() - t0
    cases.append(("diff_scenes", sc, pert, 512, 512))
    for name, b, p, w, h in cases:
        db, dp = DeviceBatch(b, ctx.device), DeviceBatch(p, ctx.device)
        tgt = ctx.render_coverage(dp, w, h, stream=sp).clone()
        del dp
        cov = torch.empty((b.n_rasters, h, w), dtype=torch.float32, device=tgt.device)
        dl = torch.empty_like(cov)
        dpts = torch.empty(max(1, len(b.pts)), dtype=torch.float32, device=tgt.device)
        dxf = torch.empty((max(1, b.n_fills), 6), dtype=torch.float32, device=tgt.device)

        def fwd():
            ctx.render_coverage(db, w, h, cov, stream=sp)
            ctx.l2_loss(cov, tgt, dl, stream=sp)

        def fwd_bwd():
            fwd()
            ctx.fill_backward(db, w, h, dl, dpts, dxf, stream=sp)

        for _ in range(2):
            fwd_bwd()
        torch.cuda.synchronize()
        reps = max(3, min(steps, 5))
        f_ms = _event_ms(fwd, stream, flush, reps)
        fb_ms = _event_ms(fwd_bwd, stream, flush, reps)
        st = ctx.stats()
        # gradient check against the FP64 reference (prefix of the batch)
        k = b.n_rasters if name == "diff_union" else min(4, b.n_rasters)
        sub = b if k == b.n_rasters else B.subset(b, list(range(k)))
        g_dp = dpts.cpu().numpy()[:len(sub.pts)].astype(np.float64)
        g_dx = dxf.cpu().numpy()[:sub.n_fills].astype(np.float64)
        t_np = tgt[:k].cpu().numpy().astype(np.float64)
        _, a_dp, a_dx = oracle.adjoint64(sub, w, h, t_np)
        _, r_dp, r_dx = oracle.diff64(sub, w, h, t_np)
        rel = lambda a, r: float(np.linalg.norm(a - r) / max(np.linalg.norm(r), 1e-300))
        # the same against the all-double forward, with the pixels near the
        # kinks of min(|S|, 1) (|S| within MASK_EPS of 0 or 1, in the f32 or
        # the double forward) taken out of both gradients: there dL/dS
        # switches, and the f32 and double forwards fall on different sides
        S32, T32, _ = oracle._tile_images(sub, w, h)
        S64 = oracle.forward64(sub, w, h)
        near = lambda S: (np.abs(np.abs(S) - 1.0) < MASK_EPS) | (np.abs(S) < MASK_EPS)
        keep = ~((T32 & near(S32.astype(np.float64))) | near(S64))
        c64 = np.minimum(np.abs(S64), 1.0)
        g64 = np.where(keep & (np.abs(S64) < 1.0), np.sign(S64) * 2.0 * (c64 - t_np), 0.0)
        m_dp, m_dx = oracle.backward64(sub, w, h, g64)
        dl_m = dl.clone()
        dl_m[:k] *= torch.as_tensor(keep, device=dl.device, dtype=dl.dtype)
        if k < b.n_rasters:
            dl_m[k:] = 0
        gm_dp, gm_dx = ctx.fill_backward(db, w, h, dl_m, stream=sp)
        torch.cuda.synchronize()
        gm_dp = gm_dp.cpu().numpy()[:len(sub.pts)].astype(np.float64)
        gm_dx = gm_dx.cpu().numpy()[:sub.n_fills].astype(np.float64)
        del dl_m
        out[name] = {
            "scenes": b.n_rasters, "canvas": [w, h], "fills": b.n_fills, "lines": st["n_lines"],
            "fwd_ms": f_ms, "fwd_bwd_ms": fb_ms,
            "fwd_scenes_per_s": b.n_rasters / (f_ms / 1e3), "fwd_bwd_scenes_per_s": b.n_rasters / (fb_ms / 1e3),
            "fwd_bwd_over_fwd": f_ms / fb_ms,
            "roofline": _diff_roofline(b, w, h, f_ms, fb_ms),
            "grad_rel_err": {
                "scenes_checked": k,
                "vs_fp64_reference": {"points": rel(g_dp, a_dp), "transforms": rel(g_dx, a_dx),
                                      "note": "f32 forward (the reference's arithmetic), adjoint in double"},
                "vs_fp64_forward": {"points": rel(g_dp, r_dp), "transforms": rel(g_dx, r_dx),
                                    "note": "forward in double too: pixels whose |S| falls on the other "
                                            "side of 1 in f32 change dL/dS there"},
                "vs_fp64_forward_masked": {"points": rel(gm_dp, m_dp), "transforms": rel(gm_dx, m_dx),
                                           "eps": MASK_EPS, "masked_fraction": float(1.0 - keep.mean()),
                                           "note": "pixels with |S| within eps of 0 or 1 (f32 or double "
                                                   "forward) left out of both gradients"}},
            "kernels_backward": _kernel_shares(ctx, lambda: ctx.fill_backward(db, w, h, dl, dpts, dxf,
                                                                              stream=sp))[:6],
        }
        del db, cov, dl, tgt, dpts, dxf
        torch.cuda.empty_cache()
    out["diff_scenes"]["generation_s"] = gen_s
    out["fd_check"] = _fd_check(ctx, sp)
    return out


def _diff_roofline(b, w, h, f_ms, fb_ms):
    """Compulsory bytes of the differentiable step against the measured HBM
    bandwidth.  Forward: the input read and 4 B of coverage written per
    pixel; forward + backward adds 4 B of dL/dcov read per pixel, the input
    read again and the gradients written (4 B per input float, 24 B per
    transform)."""
    peaks, kind = load_peaks()
    peak = float(peaks.get("hbm_gbs", PEAKS_FALLBACK["hbm_gbs"]))
    px = b.n_rasters * w * h
    fwd = b.input_bytes() + 4 * px
    fb = fwd + 4 * px + b.input_bytes() + 4 * len(b.pts) + 24 * b.n_fills
    out = {"unit": "GB/s", "peak": peak, "peak_kind": f"{kind} hbm_gbs", "bound": "hbm"}
    for k, by, ms in (("fwd", fwd, f_ms), ("fwd_bwd", fb, fb_ms)):
        gbs = by / (ms * 1e6)
        out[k] = {"bytes": by, "achieved": gbs, "frac": gbs / peak}
    return out


def _fd_check(ctx, sp, n_paths=256, n_params=64, h_px=1e-3):
    """GPU gradient against central finite differences (h = 1e-3 px) of the
    FP64 loss, on 64 random parameters of the differentiable configuration
    itself (a union of 256 blobs x 32 cubics on 1024^2)."""
    import copy

    import numpy as np
    import torch

    import oracle
    from ochre_gb300 import DeviceBatch, workloads as W
    b, w, h = W.diff_union(n_paths=n_paths), 1024, 1024
    tgt = oracle.coverage_image(W.diff_union(n_paths=n_paths, perturb=2.0), w, h)
    db = DeviceBatch(b, ctx.device)
    cov = ctx.render_coverage(db, w, h, stream=sp)
    t = torch.as_tensor(tgt, device=cov.device)
    dl = torch.empty_like(cov)
    ctx.l2_loss(cov, t, dl, stream=sp)
    dp, dx = ctx.fill_backward(db, w, h, dl, stream=sp)
    torch.cuda.synchronize()
    dp, dx = dp.cpu().numpy().astype(np.float64), dx.cpu().numpy().astype(np.float64)
    counts = oracle.seg_counts(b)
    t64 = tgt.astype(np.float64)
    rng = np.random.default_rng(2)
    pi = rng.choice(len(b.pts), n_params - 8, replace=False)
    xi = rng.choice(6 * b.n_fills, 8, replace=False)
    fd, an = [], []
    for i in pi:
        v = []
        for sgn in (1.0, -1.0):
            bb = copy.copy(b)
            bb.pts = b.pts.copy()
            bb.pts[i] = np.float32(float(b.pts[i]) + sgn * h_px)
            v.append((oracle.diff64(bb, w, h, t64, counts, grad=False)[0], float(bb.pts[i])))
        fd.append((v[0][0] - v[1][0]) / (v[0][1] - v[1][1]))
        an.append(dp[i])
    for i in xi:
        f, k = divmod(int(i), 6)
        step = h_px if k >= 4 else h_px / 1024.0   # linear part: points move ~1e-3 px
        v = []
        for sgn in (1.0, -1.0):
            bb = copy.copy(b)
            bb.fill_xf = b.fill_xf.copy()
            bb.fill_xf[f, k] = np.float32(float(b.fill_xf[f, k]) + sgn * step)
            v.append((oracle.diff64(bb, w, h, t64, counts, grad=False)[0], float(bb.fill_xf[f, k])))
        fd.append((v[0][0] - v[1][0]) / (v[0][1] - v[1][1]))
        an.append(dx[f, k])
    fd, an = np.array(fd), np.array(an)
    return {"workload": f"diff_union {n_paths} paths x 32 cubics, 1024^2", "params": n_params, "h_px": h_px,
            "rel_err": float(np.linalg.norm(an - fd) / np.linalg.norm(fd))}


def run_profile(args):
    """Untimed runs of one workload for an external profiler (ncu): warmup +
    steps calls of the rasterization (or of render + loss + backward, or of
    the compositing of one rasterization onto a 4096x4096 RGBA8 canvas)."""
    import torch
    from ochre_gb300 import DeviceBatch, GpuContext
    batch = make_workload(args.workload, args.n_paths, args.seed)
    ctx = GpuContext(0, chain_only=args.chain_only)
    if args.fused_shape:
        from ochre_gb300 import autotune
        shape = [p for p in autotune.fused_candidates() if autotune.shape_name(p) == args.fused_shape]
        if not shape:
            raise SystemExit(f"unknown fused shape {args.fused_shape}")
        autotune.apply(ctx, shape[0])
    db = DeviceBatch(batch, 0)
    sp = torch.cuda.current_stream().cuda_stream
    if args.mode == "profile":
        for _ in range(args.warmup + args.steps):
            ctx.rasterize_device(db, sp)
    elif args.mode == "profile-composite":
        import numpy as np
        rng = np.random.default_rng(9)
        colors = torch.as_tensor(rng.integers(0, 256, size=(batch.n_rasters, 4), dtype=np.uint8), device="cuda:0")
        canvas = torch.full((4096, 4096, 4), 255, dtype=torch.uint8, device="cuda:0")
        r = ctx.rasterize_device(db, sp)
        for _ in range(args.warmup + args.steps):
            ctx.composite(r, batch.n_rasters, colors, canvas, sp)
    else:
        w = h = 1024 if args.workload == "diff_union" else 512
        tgt = torch.zeros((batch.n_rasters, h, w), dtype=torch.float32, device="cuda:0")
        cov = torch.empty_like(tgt)
        dl = torch.empty_like(tgt)
        for _ in range(args.warmup + args.steps):
            ctx.render_coverage(db, w, h, cov, stream=sp)
            ctx.l2_loss(cov, tgt, dl, stream=sp)
            ctx.fill_backward(db, w, h, dl, stream=sp)
    torch.cuda.synchronize()
    print(json.dumps({"mode": args.mode, "workload": args.workload, "stats": ctx.stats()}), flush=True)
    ctx.close()


def run_ours(args, ws, rank, local):
    import numpy as np
    import torch

    from ochre_gb300 import DeviceBatch, GpuContext

    torch.cuda.set_device(local)
    batch = make_workload(args.workload, args.n_paths, args.seed + 1000 * rank)
    ctx = GpuContext(local)
    db = DeviceBatch(batch, local)
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")  # > 126 MB L2
    # launch shapes: the project's autotuner on a sample of this workload
    from ochre_gb300 import autotune
    # (large enough that each persistent CTA takes tens of rasters, as in the
    # full step, so that tail effects rank the shapes as the step does)
    sample = make_workload(args.workload, min(args.n_paths, 50_000), args.seed + 7)
    tuned = autotune.tune(ctx, fused_sample=sample)

    for _ in range(max(3, args.warmup)):
        ctx.rasterize_device(db, sp)
    torch.cuda.synchronize()
    st = ctx.stats()

    # ---- timed: device-resident inputs ----
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    # raw clock samples of the timed region (the JSON line carries their summary)
    clocks_path = os.path.join(os.environ.get("OCHRE_BENCH_CLOCKS_DIR", "/tmp"), f"bench_clocks_r{rank}.csv")
    barrier(ws)
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    with ClockSampler(local, clocks_path) as clk:
        for i in range(args.steps):
            flush.fill_(i & 0xff)
            ev[i][0].record(stream)
            ctx.rasterize_device(db, sp)
            ev[i][1].record(stream)
        torch.cuda.synchronize()
    barrier(ws)
    wall = time.perf_counter() - wall0
    step_ms = [a.elapsed_time(b) for a, b in ev]
    dev_s = sum(step_ms) / 1000.0
    dev_s_max = reduce_max(dev_s, ws)
    launches = st["n_launches"] * args.steps

    # ---- per-kernel profile (separate, untimed pass) ----
    ctx.set_profile(True)
    flush.fill_(1)
    torch.cuda.synchronize()
    ctx.rasterize_device(db, sp)
    torch.cuda.synchronize()
    prof = ctx.timings()
    ctx.set_profile(False)
    per = {}
    for name, ms in prof:
        d = per.setdefault(name, [0.0, 0])
        d[0] += ms
        d[1] += 1
    total_k = sum(v[0] for v in per.values())
    kernels = sorted(({"kernel": k, "ms": v[0], "launches": v[1], "share": v[0] / total_k if total_k else 0.0}
                      for k, v in per.items()), key=lambda x: -x["ms"])
    dom = kernels[0]
    peaks, peak_kind = load_peaks()
    peak = float(peaks.get("hbm_gbs", PEAKS_FALLBACK["hbm_gbs"]))
    dom_bytes = kernel_bytes(dom["kernel"], st, batch) / max(1, dom["launches"])
    dom_ms = dom["ms"] / max(1, dom["launches"])
    achieved = dom_bytes / (dom_ms / 1000.0) / 1e9 if dom_ms > 0 else 0.0
    # DRAM traffic per launch and warp instructions per raster of the dominant
    # kernel, from committed ncu captures, each keyed by the launch shape it
    # was taken at: used only when that is the shape this run tuned to
    from ochre_gb300 import autotune
    shape = autotune.shape_name(tuned["choice"]) if dom["kernel"] == "raster_fused" else "chain"
    traffic = None
    inst_per_unit = None
    tfile = os.path.join(ROOT, "profiles", f"traffic_{args.workload}.json")
    if os.path.exists(tfile):
        with open(tfile) as f:
            tj = json.load(f)
        def keyed(table):
            per_kernel = tj.get(table, {}).get(dom["kernel"], {})
            return per_kernel.get(shape) if isinstance(per_kernel, dict) else None
        traffic = keyed("dram_bytes_per_launch")
        inst_per_unit = keyed("warp_instructions_per_raster")

    # ---- e2e: host C-ABI entry, pinned host inputs, H2D + D2H in the timed region ----
    def pinned(a):
        t = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
        return t.numpy()

    from ochre_gb300.batch import Batch
    hb = Batch(pinned(batch.verbs), pinned(batch.pts), pinned(batch.fill_cmd_off), pinned(batch.fill_xf),
               None if batch.fill_flags is None else pinned(batch.fill_flags),
               None if batch.raster_fill_off is None else pinned(batch.raster_fill_off), batch.n_rasters)
    h2d = (hb.verbs.nbytes + hb.pts.nbytes + hb.fill_cmd_off.nbytes + hb.fill_xf.nbytes
           + (0 if hb.fill_flags is None else hb.fill_flags.nbytes)
           + (0 if hb.raster_fill_off is None else hb.raster_fill_off.nbytes))
    for _ in range(2):
        res = ctx.rasterize_raw(hb)
    n_t, n_s = res.n_tiles, res.n_spans
    d2h = n_t * 68 + n_s * 10 + 2 * 4 * (batch.n_rasters + 1)
    e2e_steps = max(1, min(args.steps, 10))
    barrier(ws)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        ctx.rasterize_raw(hb)
    e2e_s = reduce_max((time.perf_counter() - t0) / e2e_steps, ws)

    # ---- the general kernel chain on the same batch (the plain GPU method) ----
    ctx.set_chain_only(True)
    for _ in range(2):
        ctx.rasterize_device(db, sp)
    chain_st = ctx.stats()
    torch.cuda.synchronize()
    chain_ms = []
    for i in range(max(3, min(args.steps, 10))):
        flush.fill_(i & 0xff)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        ctx.rasterize_device(db, sp)
        b.record(stream)
        torch.cuda.synchronize()
        chain_ms.append(a.elapsed_time(b))
    ctx.set_chain_only(False)
    chain_step_ms = sum(chain_ms) / len(chain_ms)

    # ---- parity on a sample of this workload (the bar of the metric) ----
    parity = None
    if rank == 0:
        import numpy as np
        import oracle
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        from compare import compare
        from ochre_gb300 import batch as B
        samp = B.subset(batch, list(range(0, batch.n_rasters, max(1, batch.n_rasters // 2000))))
        ctx.set_want_cov(True)
        got = ctx.rasterize(samp)
        ctx.set_want_cov(False)
        with np.errstate(all="ignore"):
            ref = oracle.run(samp, threads=os.cpu_count() or 1)
            cst = compare(got, ref, samp.n_rasters)
            e64 = oracle.tile_cov_error_vs_fp64(samp, got["tile_xy"], got["tile_cov"], got["raster_tile_off"])
        parity = {"sample_paths": samp.n_rasters, "tiles_spans_exact": True, "alpha_max_lsb": cst["max_lsb"],
                  "alpha_diff_fraction": cst["diff_fraction"], "cov_err_vs_fp64_max": e64["max_abs"],
                  "cov_err_vs_fp64_mean": e64["mean_abs"]}

    if rank != 0:
        ctx.close()
        return
    peaks, _ = load_peaks()
    extensions = {}
    if not args.no_extensions:
        extensions["uneven_mix"] = bench_uneven(ctx, stream, flush, args.steps,
                                                float(peaks.get("hbm_gbs", PEAKS_FALLBACK["hbm_gbs"])))
        t_gen = time.time()
        from ochre_gb300 import workloads as W
        scenes = W.diff_scenes(n_scenes=args.diff_scenes)
        t_gen = time.time() - t_gen
        extensions["differentiable"] = bench_differentiable(ctx, stream, flush, args.steps, args.diff_scenes, scenes)
        extensions["differentiable"]["diff_scenes"]["generation_s"] = t_gen
        extensions["configs"] = bench_configs(ctx, stream, flush, float(peaks.get("hbm_gbs", PEAKS_FALLBACK["hbm_gbs"])),
                                              batch, scenes)
        extensions["stroke"] = bench_stroke(ctx, stream, flush, args.steps)
        extensions["svg_documents"] = bench_svg_documents(ctx, stream, flush)
        extensions["graph"] = bench_graph(ctx, stream, args.steps)
        extensions["composite"] = bench_composite(ctx, stream, flush, args.steps)
    n_paths_all = batch.n_rasters * ws
    value = n_paths_all * args.steps / dev_s_max
    # The dominant kernel is issue-bound: its warp instructions per second
    # against 4 per SM per cycle at the SM clock sampled in the timed region.
    issue = None
    clocks = clk.summary()
    mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz")
    try:
        if inst_per_unit and mhz and dom_ms:
            sms = torch.cuda.get_device_properties(local).multi_processor_count
            peak_inst = sms * 4 * mhz * 1e6
            ach_inst = inst_per_unit * batch.n_rasters / (dom_ms / 1e3)
            issue = {"bound": "issue", "kernel": dom["kernel"], "shape": shape, "unit": "warp instructions/s",
                     "achieved": ach_inst, "peak": peak_inst, "frac": ach_inst / peak_inst,
                     "warp_instructions_per_raster": inst_per_unit,
                     "note": f"peak = {sms} SMs x 4 schedulers x {mhz:.0f} MHz; instructions per raster from "
                             "the committed ncu capture, time from this run"}
        else:
            issue = {"kernel": dom["kernel"], "shape": shape, "achieved": None,
                     "note": "no committed ncu capture of this kernel at this launch shape"}
    except (RuntimeError, TypeError, ValueError, ZeroDivisionError) as e:
        issue = {"error": str(e)}
    cpu = cpu_baseline(batch) if ws == 1 else None
    comp_in = batch.input_bytes()
    comp_out = output_bytes(st["n_tiles"], st["n_spans"], batch.n_rasters)
    path_gbs = (comp_in + comp_out) / (dev_s / args.steps) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": "paths/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * dev_s_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": bench_config(args, batch.n_rasters, ws),
        "workload_counts": {"tiles_per_step": st["n_tiles"], "spans_per_step": st["n_spans"],
                            "lines_per_step": st["n_lines"], "sort_entries_per_step": st["n_entries"],
                            "key_bits": st["key_bits"], "sort_passes": st["sort_passes"]},
        "tuning": {"launch_shape": tuned["choice"], "autotune_ms": tuned["ms"]},
        "tiles_per_s": st["n_tiles"] * ws * args.steps / dev_s_max,
        "wall_s_timed_region": wall,
        "roofline": {"bound": "hbm", "kernel": dom["kernel"], "achieved": achieved, "peak": peak,
                     "peak_kind": f"{peak_kind} hbm_gbs", "unit": "GB/s", "frac": achieved / peak,
                     "frac_of_nominal": achieved / NOMINAL_HBM_GBS,
                     "traffic": traffic, "algorithmic_bytes_per_launch": dom_bytes, "ms_per_launch": dom_ms},
        "issue_roofline": issue,
        "path_roofline": {"compulsory_bytes_per_step": comp_in + comp_out, "achieved_gbs": path_gbs,
                          "frac": path_gbs / peak, "note": "input verbs+points+transforms and 68 B/tile + 6 B/span"},
        "kernels": kernels,
        "parity": parity,
        "path": "fused" if st.get("fused") else "chain",
        "plain_chain": {"value": batch.n_rasters * ws / (chain_step_ms / 1000.0), "unit": "paths/s",
                        "ms_per_step": chain_step_ms, "launches_per_step": chain_st["n_launches"],
                        "note": "general flatten/DDA/sort/tile chain on the same batch"},
        "cpu_baseline": cpu,
        "batched_uneven_mix": extensions.get("uneven_mix"),
        "differentiable": extensions.get("differentiable"),
        "stroke": extensions.get("stroke"),
        "graph": extensions.get("graph"),
        "composite": extensions.get("composite"),
        "configs": extensions.get("configs"),
        "svg_documents": extensions.get("svg_documents"),
        "e2e": {"value": n_paths_all / e2e_s, "unit": "paths/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": 1000 * e2e_s,
                "note": "pinned host inputs: points read by the kernels in place over the host link, the "
                        "other arrays copied; outputs written by the kernels into mapped host memory"},
        "gpu_launches": launches,
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="glyph_run")
    ap.add_argument("--n-paths", type=int, default=100_000)
    ap.add_argument("--seed", type=int, default=2)
    ap.add_argument("--diff-scenes", type=int, default=4096,
                    help="scenes in the batched differentiable workload (512x512 each)")
    ap.add_argument("--no-extensions", action="store_true",
                    help="skip the uneven-mix and differentiable measurements")
    ap.add_argument("--mode", default="bench", choices=["bench", "profile", "profile-diff", "profile-composite"],
                    help="profile: run warmup + steps rasterizations of the workload untimed, for ncu; "
                         "profile-diff: the same for render + loss + backward of --workload diff_union|diff_scenes; "
                         "profile-composite: one rasterization, then warmup + steps compositings onto 4096x4096")
    ap.add_argument("--chain-only", action="store_true", help="profile mode: force the general chain")
    ap.add_argument("--fused-shape", default="", help="profile mode: fused kernel shape (threads x tiles per chunk), e.g. 96x16")
    args = ap.parse_args()
    if args.mode != "bench":
        from ochre_gb300 import build
        build.build()
        run_profile(args)
        return
    ws, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, ws, rank)
    else:
        from ochre_gb300 import build
        build.build()
        run_ours(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
