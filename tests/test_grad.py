"""Differentiable fill: coverage render, L2 loss and the hand-written backward.

The FP64 model in the oracle (``oracle.diff64``, conics included) is first checked against
central finite differences (h = 1e-3 px on control points and translations;
the same 1e-3 px displacement on the linear part of a transform).  The GPU's
gradient is then checked against the FP64 reference gradient of the f32
model (``oracle.adjoint64``: the f32 forward, adjoint in double), against the
all-double model, and against central differences.  Tolerance: relative L2
error <= 1e-3 over the checked parameters.
"""
from __future__ import annotations

import copy

import numpy as np
import pytest

import oracle
from ochre_gb300 import workloads as W

REL_TOL = 1e-3
FD_H = 1e-3


def _rel(a, b):
    a, b = np.asarray(a, np.float64).ravel(), np.asarray(b, np.float64).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _params(batch, n_pts, n_xf, seed):
    """n_pts point coordinates and n_xf transform entries, picked at random
    among those with a non-trivial gradient (non-raw fills)."""
    rng = np.random.default_rng(seed)
    pts = rng.choice(len(batch.pts), n_pts, replace=False)
    xf = rng.choice(6 * batch.n_fills, n_xf, replace=False)
    return pts, xf


def _central_fd(batch, w, h, target, counts, pts_idx, xf_idx):
    """Central differences of the FP64 loss; steps are taken on the f32
    inputs and divided by the step actually represented."""
    out = []
    for i in pts_idx:
        vals = []
        for s in (1.0, -1.0):
            b = copy.copy(batch)
            b.pts = batch.pts.copy()
            b.pts[i] = np.float32(float(batch.pts[i]) + s * FD_H)
            vals.append((oracle.diff64(b, w, h, target, counts, grad=False)[0], float(b.pts[i])))
        out.append((vals[0][0] - vals[1][0]) / (vals[0][1] - vals[1][1]))
    for i in xf_idx:
        f, k = divmod(int(i), 6)
        if k < 4:
            # the linear part scales coordinates: step so points move ~1e-3 px
            c0, c1 = batch.fill_cmd_off[f], batch.fill_cmd_off[f + 1]
            span = np.abs(batch.pts[_float_range(batch, c0, c1)]).max()
            step = FD_H / max(float(span), 1.0)
        else:
            step = FD_H
        vals = []
        for s in (1.0, -1.0):
            b = copy.copy(batch)
            b.fill_xf = batch.fill_xf.copy()
            b.fill_xf[f, k] = np.float32(float(batch.fill_xf[f, k]) + s * step)
            vals.append((oracle.diff64(b, w, h, target, counts, grad=False)[0], float(b.fill_xf[f, k])))
        out.append((vals[0][0] - vals[1][0]) / (vals[0][1] - vals[1][1]))
    return np.array(out)


def _float_range(batch, c0, c1):
    from ochre_gb300.batch import FLOATS_PER_VERB
    nf = FLOATS_PER_VERB[batch.verbs].astype(np.int64)
    off = np.concatenate([[0], np.cumsum(nf)])
    return slice(int(off[c0]), int(off[c1]))


def _small_scenes():
    return W.diff_scenes(n_scenes=3, seed=11, size=128.0, min_paths=2, max_paths=4, min_seg=4, max_seg=12)


# ---------------------------------------------------------------- CPU: oracle


@pytest.mark.parametrize("case", ["union", "scenes"])
def test_fp64_gradient_matches_central_differences(case):
    if case == "union":
        b, w, h = W.diff_union(n_paths=6), 1024, 1024
        tgt = oracle.coverage_image(W.diff_union(n_paths=6, perturb=2.0), w, h)
    else:
        b, w, h = _small_scenes(), 128, 128
        pert = copy.copy(b)
        pert.pts = (b.pts + np.random.default_rng(3).normal(0, 1.0, b.pts.shape)).astype(np.float32)
        tgt = oracle.coverage_image(pert, w, h)
    tgt = tgt.astype(np.float64)
    counts = oracle.seg_counts(b)
    loss, dp, dx = oracle.diff64(b, w, h, tgt, counts)
    assert loss > 0.0
    pi, xi = _params(b, 56, 8, seed=1)
    fd = _central_fd(b, w, h, tgt, counts, pi, xi)
    an = np.concatenate([dp[pi], dx.reshape(-1)[xi]])
    assert np.linalg.norm(an) > 0.0
    assert _rel(an, fd) <= REL_TOL, (_rel(an, fd), np.c_[an, fd])


@pytest.mark.parametrize("on_grid", [False, True])
def test_fp64_gradient_matches_central_differences_everywhere(on_grid):
    """Every parameter of a small batch, including points on pixel corners
    (the coverage is continuously differentiable there too)."""
    b, w, h = _raw_and_multi_contour_batch(on_grid), 128, 128
    pert = copy.copy(b)
    pert.pts = (b.pts + np.random.default_rng(5).normal(0, 1.5, b.pts.shape)).astype(np.float32)
    tgt = oracle.coverage_image(pert, w, h).astype(np.float64)
    counts = oracle.seg_counts(b)
    _, dp, dx = oracle.diff64(b, w, h, tgt, counts)
    fd = _central_fd(b, w, h, tgt, counts, np.arange(len(b.pts)), np.arange(6 * b.n_fills))
    an = np.concatenate([dp, dx.ravel()])
    assert _rel(an, fd) <= REL_TOL, _rel(an, fd)


def test_fp64_gradient_is_zero_at_the_target():
    b = W.diff_union(n_paths=4)
    tgt = oracle.coverage_image(b, 1024, 1024).astype(np.float64)
    loss, dp, dx = oracle.diff64(b, 1024, 1024, tgt)
    # the f32 image differs from the FP64 area only by rounding (~1e-4 per
    # edge pixel), so loss and gradient nearly vanish; against a target
    # perturbed by 2 px they are ~1e3 and ~1e1 (points) / ~1e4 (transforms)
    assert loss < 1e-4
    assert np.abs(dp).max() < 1e-2 and np.abs(dx).max() < 10.0


def _conic_batch(seed=0):
    """Three rasters: a circle of four conics (w = cos 45 deg) under a
    shear, and a blob bounded by two conics of random weights."""
    from ochre_gb300.batch import BatchBuilder
    rng = np.random.default_rng(seed)
    bb = BatchBuilder()
    for r in range(3):
        bb.begin_raster()
        cx, cy = rng.uniform(40, 90, 2)
        R = rng.uniform(15, 30)
        w = 0.70710677
        bb.fill([0, 4, 4, 4, 4, 5],
                [cx + R, cy, cx + R, cy + R, cx, cy + R, w, cx - R, cy + R, cx - R, cy, w,
                 cx - R, cy - R, cx, cy - R, w, cx + R, cy - R, cx + R, cy, w],
                [1.0, 0.1 * r, -0.05, 1.1, 3.0 * r, 2.0])
        bb.fill([0, 4, 1, 4, 5],
                [cx - 10, cy - 5, cx, cy - 35, cx + 12, cy - 4, rng.uniform(0.3, 2.5), cx + 8, cy + 10,
                 cx - 4, cy + 30, cx - 10, cy - 5, rng.uniform(0.3, 2.5)],
                [0.9, 0.0, 0.0, 0.9, 5.0, 4.0])
    return bb.build()


def _conic_target(b, w, h):
    pert = copy.copy(b)
    pert.pts = (b.pts + np.random.default_rng(5).normal(0, 1.5, b.pts.shape)).astype(np.float32)
    return oracle.coverage_image(pert, w, h).astype(np.float64)


def test_fp64_conic_gradient_matches_central_differences():
    """Conics (path.rs:75-104): the emitted points are the conic at the f32
    subdivision's parameters (held fixed), differentiated in the control
    points, the weight and the transform."""
    b, w, h = _conic_batch(), 128, 128
    tgt = _conic_target(b, w, h)
    counts = oracle.seg_counts(b)
    loss, dp, dx = oracle.diff64(b, w, h, tgt, counts)
    assert loss > 0.0
    fd = _central_fd(b, w, h, tgt, counts, np.arange(len(b.pts)), np.arange(6 * b.n_fills))
    an = np.concatenate([dp, dx.ravel()])
    assert _rel(an, fd) <= REL_TOL, _rel(an, fd)
    from ochre_gb300.batch import FLOATS_PER_VERB
    off = np.concatenate([[0], np.cumsum(FLOATS_PER_VERB[b.verbs])])
    weights = [int(off[c]) + 4 for c in range(b.n_cmds) if b.verbs[c] == 4]
    assert np.abs(dp[weights]).max() > 1.0   # the weights are differentiated too


# ---------------------------------------------------------------- GPU


def _gpu_grad(batch, w, h, target):
    import torch
    from ochre_gb300 import DeviceBatch, GpuContext
    ctx = GpuContext(0)
    db = DeviceBatch(batch, 0)
    cov = ctx.render_coverage(db, w, h)
    t = torch.as_tensor(np.ascontiguousarray(target, np.float32), device="cuda:0")
    dl = torch.empty_like(cov)
    loss, _ = ctx.l2_loss(cov, t, dl)
    dp, dx = ctx.fill_backward(db, w, h, dl)
    torch.cuda.synchronize()
    out = (float(loss.item()), dp.cpu().numpy()[:len(batch.pts)].astype(np.float64),
           dx.cpu().numpy()[:batch.n_fills].astype(np.float64), cov.cpu().numpy())
    ctx.close()
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["union", "scenes", "edge_cases"])
def test_render_coverage_matches_oracle(name):
    import torch
    from ochre_gb300 import DeviceBatch, GpuContext
    from tests.edge_cases import edge_batch
    if name == "union":
        b, w, h = W.diff_union(n_paths=32), 1024, 1024
    elif name == "scenes":
        b, w, h = W.diff_scenes(n_scenes=8, seed=12, size=256.0, min_paths=4, max_paths=32), 256, 256
    else:
        b, w, h = edge_batch()[0], 96, 80
    ctx = GpuContext(0)
    cov = ctx.render_coverage(DeviceBatch(b, 0), w, h)
    torch.cuda.synchronize()
    got = cov.cpu().numpy()
    ctx.close()
    ref = oracle.coverage_image(b, w, h)
    assert got.shape == ref.shape
    # same f32 accumulation up to summation order (pixels whose sum cancels
    # to ~0 may differ in being exactly zero; the tile/span structure itself
    # is checked exactly by the parity tests)
    assert np.abs(got - ref).max() < 1e-3


@pytest.mark.gpu
def test_l2_loss_and_upstream_gradient():
    import torch
    from ochre_gb300 import GpuContext
    g = torch.Generator(device="cuda:0").manual_seed(0)
    cov = torch.rand((3, 70, 33), device="cuda:0", generator=g)
    tgt = torch.rand((3, 70, 33), device="cuda:0", generator=g)
    ctx = GpuContext(0)
    dl = torch.empty_like(cov)
    loss, _ = ctx.l2_loss(cov, tgt, dl)
    torch.cuda.synchronize()
    c, t = cov.cpu().double().numpy(), tgt.cpu().double().numpy()
    # per thread a compensated float sum, thread sums in double: relative
    # error of order the float epsilon
    assert abs(loss.item() - ((c - t) ** 2).sum()) < 3e-7 * max(1.0, ((c - t) ** 2).sum())
    assert np.allclose(dl.cpu().numpy(), 2.0 * (cov - tgt).cpu().numpy(), atol=0, rtol=0)
    ctx.close()


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["union", "scenes"])
def test_gpu_gradient_matches_fp64(case):
    """dL/d(control points) and dL/d(transform) against the FP64 reference
    gradient of the same model (relative L2 error <= 1e-3)."""
    if case == "union":
        b, w, h = W.diff_union(n_paths=32), 1024, 1024
        pert = W.diff_union(n_paths=32, perturb=2.0)
    else:
        b, w, h = W.diff_scenes(n_scenes=6, seed=13, size=256.0, min_paths=4, max_paths=24), 256, 256
        pert = copy.copy(b)
        pert.pts = (b.pts + np.random.default_rng(4).normal(0, 2.0, b.pts.shape)).astype(np.float32)
    tgt = oracle.coverage_image(pert, w, h)
    loss, dp, dx, cov = _gpu_grad(b, w, h, tgt)
    aloss, adp, adx = oracle.adjoint64(b, w, h, tgt)
    assert abs(loss - aloss) <= 1e-5 * aloss, (loss, aloss)
    assert _rel(dp, adp) <= REL_TOL, _rel(dp, adp)
    assert _rel(dx, adx) <= REL_TOL, _rel(dx, adx)
    # sparse scenes: even the all-double forward agrees to the same bound
    rloss, rdp, rdx = oracle.diff64(b, w, h, tgt.astype(np.float64))
    assert abs(loss - rloss) <= 1e-3 * rloss, (loss, rloss)
    assert _rel(dp, rdp) <= REL_TOL, _rel(dp, rdp)
    assert _rel(dx, rdx) <= REL_TOL, _rel(dx, rdx)


@pytest.mark.gpu
def test_gpu_conic_gradient_matches_fp64():
    """Conic control points, weights and transforms against the FP64
    reference gradient of the f32 model."""
    b, w, h = _conic_batch(), 128, 128
    tgt = _conic_target(b, w, h).astype(np.float32)
    loss, dp, dx, cov = _gpu_grad(b, w, h, tgt)
    aloss, adp, adx = oracle.adjoint64(b, w, h, tgt)
    assert abs(loss - aloss) <= 1e-5 * aloss, (loss, aloss)
    assert _rel(dp, adp) <= REL_TOL, _rel(dp, adp)
    assert _rel(dx, adx) <= REL_TOL, _rel(dx, adx)


@pytest.mark.gpu
def test_gpu_gradient_dense_scenes():
    """Dense scenes (256-512 overlapping blobs per 512^2 scene).  Against the
    FP64 reference gradient of the f32 model (f32 forward as the reference
    computes it, adjoint in double) the bound is 1e-3.  The all-double
    forward differs more: its |S| lands on the other side of 1 at some
    boundary pixels of overlapping blobs (the reference's f32 walk drifts by
    ~1e-4 along long rows), which switches dL/dS there."""
    b = W.diff_scenes(n_scenes=2, seed=21, size=512.0, min_paths=256, max_paths=512)
    w = h = 512
    pert = copy.copy(b)
    pert.pts = (b.pts + np.random.default_rng(6).normal(0, 2.0, b.pts.shape)).astype(np.float32)
    tgt = oracle.coverage_image(pert, w, h)
    loss, dp, dx, _ = _gpu_grad(b, w, h, tgt)
    _, adp, adx = oracle.adjoint64(b, w, h, tgt)
    assert _rel(dp, adp) <= REL_TOL, _rel(dp, adp)
    assert _rel(dx, adx) <= REL_TOL, _rel(dx, adx)
    _, rdp, rdx = oracle.diff64(b, w, h, tgt.astype(np.float64))
    assert _rel(dp, rdp) <= 3e-2, _rel(dp, rdp)


@pytest.mark.gpu
def test_gpu_gradient_matches_central_differences():
    """The differentiable-fill workload's check: GPU gradient against FP64
    central differences (h = 1e-3 px) on 64 random parameters."""
    b, w, h = W.diff_union(n_paths=24), 1024, 1024
    tgt = oracle.coverage_image(W.diff_union(n_paths=24, perturb=2.0), w, h)
    _, dp, dx, _ = _gpu_grad(b, w, h, tgt)
    counts = oracle.seg_counts(b)
    pi, xi = _params(b, 56, 8, seed=2)
    fd = _central_fd(b, w, h, tgt.astype(np.float64), counts, pi, xi)
    an = np.concatenate([dp[pi], dx.reshape(-1)[xi]])
    assert _rel(an, fd) <= REL_TOL, (_rel(an, fd), np.c_[an, fd])


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_gpu_gradient_fuzz(seed):
    """Seeded random rasters (every verb in any order, conics, degenerate
    curves, repeated points, pixel corners, shears, device-space fills;
    some outlines cross the canvas edges): the GPU gradient against the FP64
    reference gradient of the f32 model, the target the same rasters with
    every transformed fill moved by N(0, 1.5) px."""
    from fuzz_cases import fuzz_batch
    b, w, h = fuzz_batch(12, seed, big_share=0.0), 768, 768
    pert = copy.copy(b)
    xf = b.fill_xf.copy()
    xf[:, 4:] += np.random.default_rng(seed).normal(0, 1.5, (b.n_fills, 2)).astype(np.float32)
    pert.fill_xf = xf
    tgt = oracle.coverage_image(pert, w, h)
    loss, dp, dx, _ = _gpu_grad(b, w, h, tgt)
    rloss, rdp, rdx = oracle.adjoint64(b, w, h, tgt)
    assert abs(loss - rloss) <= 1e-5 * rloss
    assert _rel(dp, rdp) <= REL_TOL, _rel(dp, rdp)
    assert _rel(dx, rdx) <= REL_TOL, _rel(dx, rdx)


@pytest.mark.gpu
def test_backward_reuses_the_forward_structure():
    """The backward right after render_coverage of the same batch reuses its
    lines and tiles (fewer launches); after another rasterization on the
    context, or on a fresh context, it recomputes them.  Same gradients."""
    import torch
    from ochre_gb300 import DeviceBatch, GpuContext
    b, w, h = W.diff_union(n_paths=32), 1024, 1024
    tgt = oracle.coverage_image(W.diff_union(n_paths=32, perturb=2.0), w, h)
    ctx, fresh = GpuContext(0), GpuContext(0)
    try:
        db = DeviceBatch(b, 0)
        cov = ctx.render_coverage(db, w, h)
        dl = torch.empty_like(cov)
        ctx.l2_loss(cov, torch.as_tensor(np.ascontiguousarray(tgt, np.float32), device="cuda:0"), dl)
        runs = []
        runs.append([t.cpu().numpy() for t in ctx.fill_backward(db, w, h, dl)] + [ctx.stats()["n_launches"]])
        ctx.rasterize_device(DeviceBatch(W.glyph_run(n_paths=50), 0))
        runs.append([t.cpu().numpy() for t in ctx.fill_backward(db, w, h, dl)] + [ctx.stats()["n_launches"]])
        runs.append([t.cpu().numpy() for t in fresh.fill_backward(db, w, h, dl)] + [fresh.stats()["n_launches"]])
        torch.cuda.synchronize()
    finally:
        ctx.close()
        fresh.close()
    (dp0, dx0, n0), (dp1, dx1, n1), (dp2, dx2, n2) = runs
    assert n0 < n1 and n1 == n2
    for dp, dx in ((dp1, dx1), (dp2, dx2)):
        # float atomics add the per-line terms in no fixed order
        assert _rel(dp0, dp) <= 1e-5 and _rel(dx0, dx) <= 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("on_grid", [False, True])
def test_gpu_gradient_raw_fills_and_multiple_contours(on_grid):
    """Raw (untransformed) fills get point gradients and a zero transform
    gradient; contours closed by Move, by Close and by finish all count.
    With ``on_grid`` every point sits on a pixel corner, where the end points
    and the lines through corners must take the walk's cells consistently."""
    b = _raw_and_multi_contour_batch(on_grid)
    w, h = 128, 128
    pert = copy.copy(b)
    pert.pts = (b.pts + np.random.default_rng(5).normal(0, 1.5, b.pts.shape)).astype(np.float32)
    tgt = oracle.coverage_image(pert, w, h)
    loss, dp, dx, _ = _gpu_grad(b, w, h, tgt)
    for ref in (oracle.adjoint64, lambda *a: oracle.diff64(*a[:3], a[3].astype(np.float64))):
        _, rdp, rdx = ref(b, w, h, tgt)
        assert _rel(dp, rdp) <= REL_TOL, np.c_[dp, rdp]
        assert _rel(dx, rdx) <= REL_TOL, np.c_[dx.ravel(), rdx.ravel()]
    assert np.all(dx[1] == 0.0)


def _raw_and_multi_contour_batch(on_grid=False):
    """Two rasters: a transformed fill with two contours (the first closed by
    the second Move) plus a raw fill, and a fill closed exactly at its start
    under a general affine transform."""
    from ochre_gb300.batch import BatchBuilder
    bb = BatchBuilder()
    bb.begin_raster()
    # two contours, the first closed implicitly by the second Move
    bb.fill([0, 3, 3, 0, 2, 2, 5],
            [10, 10, 30, 5, 50, 20, 52, 40, 48, 60, 20, 55, 12, 30,
             70, 70, 90, 72, 95, 90, 80, 100, 68, 88], [1, 0, 0, 1, 0, 0])
    bb.fill([0, 1, 1, 1], [20, 80, 40, 82, 35, 100, 18, 96], [1, 0, 0, 1, 0, 0], raw=True)
    bb.begin_raster()
    bb.fill([0, 2, 2, 2], [5, 5, 40, 0, 60, 30, 70, 60, 30, 70, 8, 40, 5, 5], [0.9, 0.2, -0.1, 1.1, 4.5, 3.25])
    b = bb.build()
    if not on_grid:
        off = np.tile(np.array([0.3719, 0.6133], np.float32), len(b.pts) // 2)
        b.pts = (b.pts + off).astype(np.float32)
    return b
