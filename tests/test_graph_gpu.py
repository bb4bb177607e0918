"""CUDA-graph execution (ochre_graph_*): replays match the oracle and the
eager chain, values may change between launches, and a batch that outgrows
its plan is re-planned.  Runs through the C ABI on the GPU."""
import dataclasses

import numpy as np
import pytest

import oracle
from compare import compare
from golden.make_golden import NAMES, load
from ochre_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _scaled(b, k):
    """The batch with every fill's matrix (not its offset) scaled by k."""
    xf = b.fill_xf.copy()
    xf[:, :4] *= np.float32(k)
    return dataclasses.replace(b, fill_xf=xf)


def _same_as_eager(got, eager):
    """Tile/span structure identical; alpha within 1 LSB and coverage within
    1e-5 (shared-memory atomics add a tile's increments in no fixed order)."""
    for k in ("tile_xy", "span_xy", "span_w", "span_tile", "raster_tile_off", "raster_span_off"):
        assert np.array_equal(got[k], eager[k]), k
    d = np.abs(got["tile_alpha"].astype(np.int16) - eager["tile_alpha"].astype(np.int16))
    assert d.size == 0 or d.max() <= 1
    if "tile_cov" in eager:
        assert np.abs(got["tile_cov"] - eager["tile_cov"]).max(initial=0.0) <= 1e-5


def _check(ctx, g, b):
    got = g.rasterize()
    compare(got, oracle.run(b, threads=8), b.n_rasters)
    return got


@pytest.mark.parametrize("name", NAMES)
def test_golden_graph_matches_eager(any_ctx, name):
    from ochre_gb300 import DeviceBatch
    b, exp = load(name)
    db = DeviceBatch(b)
    eager = any_ctx.device_result_to_numpy(any_ctx.rasterize_device(db), b.n_rasters)
    g = any_ctx.graph(db)
    try:
        for _ in range(3):   # replays are repeatable
            got = g.rasterize()
            compare(got, exp, b.n_rasters)
            _same_as_eager(got, eager)
        assert g.info()["replans"] == 0
    finally:
        g.close()


@pytest.mark.parametrize("gen,kw", [
    (W.glyph_run, dict(n_paths=2000)),
    (W.uneven_mix, dict(n_paths=120)),
    (W.cubic_boxes, dict(n_paths=40)),
    (W.diff_union, dict()),
])
def test_workload_graph_parity(any_ctx, gen, kw):
    from ochre_gb300 import DeviceBatch
    b = gen(**kw)
    db = DeviceBatch(b)
    g = any_ctx.graph(db)
    try:
        _check(any_ctx, g, b)
        st = g.stats()
        assert st.n_tiles > 0 and st.n_launches == g.info()["kernels"]
    finally:
        g.close()


def test_new_values_between_launches(gpu_ctx_chain):
    """Transforms rewritten in place on the device: the same graph
    rasterizes the new geometry (counts within the plan's headroom)."""
    from ochre_gb300 import DeviceBatch
    b = W.uneven_mix(n_paths=100, seed=5)
    db = DeviceBatch(b)
    g = gpu_ctx_chain.graph(db, headroom=2.0)
    try:
        _check(gpu_ctx_chain, g, b)
        for k in (1.1, 0.7, 1.3):
            b2 = _scaled(b, k)
            db.fill_xf.copy_(db.fill_xf.new_tensor(b2.fill_xf.reshape(-1)))
            _check(gpu_ctx_chain, g, b2)
        assert g.info()["replans"] == 0
    finally:
        g.close()


def test_outgrown_plan_replans(gpu_ctx_chain):
    """Counts above the plan's capacities: flagged on the device, re-planned
    from an eager run, replayed; results exact."""
    from ochre_gb300 import DeviceBatch
    b = W.uneven_mix(n_paths=100, seed=7)
    db = DeviceBatch(b)
    g = gpu_ctx_chain.graph(db, headroom=1.0)
    try:
        _check(gpu_ctx_chain, g, b)
        b2 = _scaled(b, 2.5)
        db.fill_xf.copy_(db.fill_xf.new_tensor(b2.fill_xf.reshape(-1)))
        _check(gpu_ctx_chain, g, b2)
        assert g.info()["replans"] == 1
        # the new plan holds the grown batch: no further re-plan
        _check(gpu_ctx_chain, g, b2)
        assert g.info()["replans"] == 1
    finally:
        g.close()


def test_fused_plan_falls_back_to_chain(gpu_ctx):
    """A batch planned on the fused kernel whose raster grows past the fused
    limits is re-planned onto the general chain."""
    from ochre_gb300 import DeviceBatch
    b = W.glyph_run(n_paths=500, seed=3)
    db = DeviceBatch(b)
    g = gpu_ctx.graph(db)
    try:
        assert g.info()["fused"]
        _check(gpu_ctx, g, b)
        xf = b.fill_xf.copy()
        xf[17, :4] *= np.float32(12.0)   # one glyph ~12x larger: past the fused grid
        b2 = dataclasses.replace(b, fill_xf=xf)
        db.fill_xf.copy_(db.fill_xf.new_tensor(b2.fill_xf.reshape(-1)))
        _check(gpu_ctx, g, b2)
        info = g.info()
        assert info["replans"] == 1 and not info["fused"]
    finally:
        g.close()


def _set(dev_tensor, host_array):
    dev_tensor.copy_(dev_tensor.new_tensor(np.ascontiguousarray(host_array).reshape(-1)))


@pytest.mark.parametrize("ctx_name", ["gpu_ctx", "gpu_ctx_chain"])
def test_stroke_graph_matches_oracle_and_eager(request, ctx_name):
    """Stroked fills (Rasterizer::stroke) replayed from a graph: the stroke
    stage runs in the graph with its counts on the device and its output
    padded with Close commands; results equal the oracle's and the eager
    call's, on every replay."""
    from ochre_gb300 import DeviceBatch
    ctx = request.getfixturevalue(ctx_name)
    b = W.stroke_run(n_paths=400, seed=11)
    db = DeviceBatch(b)
    eager = ctx.device_result_to_numpy(ctx.rasterize_device(db), b.n_rasters)
    ref = oracle.run(b, threads=8)
    g = ctx.graph(db)
    try:
        assert not g.info()["fused"]
        for _ in range(3):
            got = g.rasterize()
            compare(got, ref, b.n_rasters)
            _same_as_eager(got, eager)
        assert g.info()["replans"] == 0
    finally:
        g.close()


def test_stroke_graph_new_widths_and_points(gpu_ctx_chain):
    """Stroke widths and points rewritten in place between launches, within
    the plan's headroom: the same graph strokes and fills the new geometry
    (the stroke stage's output counts change with the joins)."""
    from ochre_gb300 import DeviceBatch
    b = W.stroke_run(n_paths=300, seed=12)
    db = DeviceBatch(b)
    g = gpu_ctx_chain.graph(db, headroom=2.0)
    try:
        _check(gpu_ctx_chain, g, b)
        for k in (0.6, 1.4):
            b2 = dataclasses.replace(b, fill_width=(b.fill_width * np.float32(k)).astype(np.float32))
            _set(db.fill_width, b2.fill_width)
            _check(gpu_ctx_chain, g, b2)
        b3 = dataclasses.replace(b, pts=(b.pts * np.float32(1.2)).astype(np.float32))
        _set(db.fill_width, b.fill_width)
        _set(db.pts, b3.pts)
        _check(gpu_ctx_chain, g, b3)
        assert g.info()["replans"] == 0
    finally:
        g.close()


def test_stroke_graph_outgrown_plan_replans(gpu_ctx_chain):
    """Path-space points scaled up: the curves flatten into more polyline
    segments than the stroke stage's plan holds (checked on the device after
    its scans); the launch re-plans from an eager run and replays, exact."""
    from ochre_gb300 import DeviceBatch
    b = W.stroke_run(n_paths=300, seed=13)
    db = DeviceBatch(b)
    g = gpu_ctx_chain.graph(db, headroom=1.0)
    try:
        _check(gpu_ctx_chain, g, b)
        b2 = dataclasses.replace(b, pts=(b.pts * np.float32(9.0)).astype(np.float32),
                                 fill_xf=_scaled(b, 1.0 / 9.0).fill_xf)
        _set(db.pts, b2.pts)
        _set(db.fill_xf, b2.fill_xf)
        _check(gpu_ctx_chain, g, b2)
        assert g.info()["replans"] == 1
        _check(gpu_ctx_chain, g, b2)
        assert g.info()["replans"] == 1
    finally:
        g.close()


def test_graph_with_coverage_output():
    """A graph of a context that also writes pre-quantisation coverage
    (fused and chain plans): coverage identical to the eager call."""
    from ochre_gb300 import DeviceBatch, GpuContext
    for chain_only, b in ((False, W.glyph_run(n_paths=300, seed=4)), (True, W.diff_union())):
        ctx = GpuContext(0, want_cov=True, chain_only=chain_only)
        try:
            db = DeviceBatch(b)
            eager = ctx.device_result_to_numpy(ctx.rasterize_device(db), b.n_rasters)
            g = ctx.graph(db)
            try:
                got = g.rasterize()
                assert g.info()["fused"] == (not chain_only)
                _same_as_eager(got, eager)
            finally:
                g.close()
        finally:
            ctx.close()


def _eager_step(ctx, db, w, h, tgt):
    import torch
    cov = ctx.render_coverage(db, w, h)
    dl = torch.empty_like(cov)
    loss, _ = ctx.l2_loss(cov, tgt, dl)
    dpts, dxf = ctx.fill_backward(db, w, h, dl)
    torch.cuda.synchronize()
    return cov, loss, dpts, dxf


def _rel_l2(a, b):
    """||a - b|| / ||b|| (float64)."""
    a, b = a.double(), b.double()
    return ((a - b).norm() / b.norm().clamp_min(1e-30)).item()


def _same_step(g, eager):
    """Coverage within 1e-5, the loss within 1e-5 relative and the gradients
    within 1e-3 relative (L2, the bound of the differentiable tests): the
    graph runs the eager step's kernels, and only the order of the atomic
    sums differs, which moves a tile sum that lands within rounding of 1 to
    either side of the kink of min(|S|, 1) in either run."""
    cov, loss, dpts, dxf = eager
    assert (g.cov - cov).abs().max().item() <= 1e-5
    assert abs(g.loss.item() - loss.item()) <= 1e-5 * abs(loss.item())
    assert _rel_l2(g.dl_dpts[:dpts.numel()], dpts) <= 1e-3
    assert _rel_l2(g.dl_dxf[:dxf.shape[0]], dxf) <= 1e-3


@pytest.mark.parametrize("case", ["union", "scenes"])
def test_differentiable_step_graph_matches_eager(gpu_ctx, case):
    """The whole differentiable step captured into one graph (forward with
    signed coverage, coverage render, L2 loss, backward) gives the eager
    calls' coverage, loss and gradients; points rewritten in place between
    launches give the new step's; a batch grown past the plan re-plans."""
    import torch
    from ochre_gb300 import DeviceBatch
    if case == "union":
        b, p, w, h = W.diff_union(n_paths=48), W.diff_union(n_paths=48, perturb=2.0), 1024, 1024
    else:
        b, w, h = W.diff_scenes(n_scenes=6, max_paths=48, max_seg=48), 512, 512
        p = dataclasses.replace(b, pts=(b.pts + np.random.default_rng(4).normal(0, 2.0, b.pts.shape)).astype(np.float32))
    db = DeviceBatch(b)
    tgt = gpu_ctx.render_coverage(DeviceBatch(p), w, h).clone()
    g = gpu_ctx.graph_diff(db, w, h, tgt, headroom=1.5)
    try:
        for _ in range(2):
            g.launch()
            torch.cuda.synchronize()
            _same_step(g, _eager_step(gpu_ctx, db, w, h, tgt))
        # new points, within the plan's headroom
        moved = (b.pts + np.random.default_rng(9).normal(0, 0.7, b.pts.shape)).astype(np.float32)
        db.pts.copy_(torch.from_numpy(moved).to(db.pts.device))
        g.launch()
        torch.cuda.synchronize()
        _same_step(g, _eager_step(gpu_ctx, db, w, h, tgt))
        assert g.info()["replans"] == 0
        # every transform's matrix scaled up: more lines and tiles than planned
        db.fill_xf.copy_(db.fill_xf.new_tensor(_scaled(b, 2.0).fill_xf.reshape(-1)))
        g.launch()
        torch.cuda.synchronize()
        assert g.info()["replans"] == 1
        _same_step(g, _eager_step(gpu_ctx, db, w, h, tgt))
    finally:
        g.close()


def test_differentiable_graph_rejects_strokes(gpu_ctx):
    import torch
    from ochre_gb300 import DeviceBatch, OchreError
    b = W.stroke_run(n_paths=4)
    tgt = torch.zeros((b.n_rasters, 64, 64), dtype=torch.float32, device="cuda:0")
    with pytest.raises(OchreError):
        gpu_ctx.graph_diff(DeviceBatch(b), 64, 64, tgt)
