"""Seeded synthetic workloads with the shapes of the five rasterization
configurations (no public dataset exists for this path; these stand in).

All randomness comes from numpy's PCG64 (``np.random.default_rng(seed)``),
which is platform independent; ``seed`` defaults to the configuration number.
Trigonometric values may differ by an ulp between machines, so golden
fixtures store their inputs instead of regenerating them.

* ``cubic_boxes``   — 1,000 closed paths of 16 cubics, control points uniform
  in a 512x512 box placed uniformly on a 2048x2048 canvas, identity transform.
* ``glyph_run``     — 100,000 glyph-like paths: 8-40 quadratics over 1-3
  contours (perturbed circles / rounded rects, holes reversed), em 10-48 px,
  random rotation, scale 0.5-2 and translation on 4096x4096.
* ``uneven_mix``    — 20,000 paths, segment count lognormal (median 32,
  sigma 1.5, clipped to 4..20,000), 50/50 quadratic/cubic, random-walk control
  points (step N(0, s^2), s ~ U[8, 200] px per path) reflected into
  [0, 8192)^2, closed.
* ``diff_union``    — 256 closed blobs of 32 cubics in one rasterizer on
  1024x1024 (differentiable fill).
* ``diff_scenes``   — independent 512x512 scenes of 8-512 blobs of 4-128 mixed
  quadratic/cubic segments, one random affine per scene.
"""
from __future__ import annotations

import math
from typing import Optional

import numpy as np

from .batch import (CLOSE, CUBIC, FLOATS_PER_VERB, IDENTITY, MOVE, QUADRATIC, Batch,
                    BatchBuilder)


def readme_path() -> Batch:
    """The single path of ochre's README / examples/basic.rs."""
    bb = BatchBuilder()
    bb.fill([MOVE, QUADRATIC, CUBIC, CLOSE],
            [400.0, 300.0,
             500.0, 200.0, 400.0, 100.0,
             350.0, 150.0, 100.0, 250.0, 400.0, 300.0], IDENTITY)
    return bb.build()


def _contour_stream(n_seg: np.ndarray, kind: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Verb stream of closed contours: ``n_seg[c]`` segments per contour,
    ``kind`` per segment (QUADRATIC or CUBIC); each contour is Move(start),
    segments, Close.  Returns the verbs and the command index of every
    segment."""
    n_c = len(n_seg)
    seg_start = np.concatenate([[0], np.cumsum(n_seg)[:-1]]).astype(np.int64)
    ncmd_c = n_seg + 2
    cmd_start = np.concatenate([[0], np.cumsum(ncmd_c)[:-1]]).astype(np.int64)
    n_cmd = int(ncmd_c.sum())
    verbs = np.empty(n_cmd, np.uint8)
    verbs[cmd_start] = MOVE
    verbs[cmd_start + ncmd_c - 1] = CLOSE
    seg_contour = np.repeat(np.arange(n_c), n_seg)
    seg_local = np.arange(len(kind)) - seg_start[seg_contour]
    seg_cmd = cmd_start[seg_contour] + 1 + seg_local
    verbs[seg_cmd] = kind
    return verbs, seg_cmd


def _streams(n_seg, kind, start_xy, seg_floats):
    """Build verbs and the float stream for contours (start point + segments)."""
    verbs, seg_cmd = _contour_stream(n_seg, kind)
    nf = FLOATS_PER_VERB[verbs]
    foff = np.concatenate([[0], np.cumsum(nf)]).astype(np.int64)
    pts = np.zeros(int(foff[-1]), np.float32)
    n_c = len(n_seg)
    cmd_start = np.concatenate([[0], np.cumsum(n_seg + 2)[:-1]]).astype(np.int64)
    pts[foff[cmd_start]] = start_xy[:, 0]
    pts[foff[cmd_start] + 1] = start_xy[:, 1]
    q = kind == QUADRATIC
    base = foff[seg_cmd]
    for j in range(4):
        pts[base[q] + j] = seg_floats[q, j]
    for j in range(6):
        pts[base[~q] + j] = seg_floats[~q, j]
    return verbs, pts, n_c


def _batch_from_streams(verbs, pts, contour_ncmd, contour_fill, xf, n_fills, raster_fill_off, n_rasters):
    fill_ncmd = np.bincount(contour_fill, weights=contour_ncmd, minlength=n_fills).astype(np.int64)
    off = np.zeros(n_fills + 1, np.uint32)
    off[1:] = np.cumsum(fill_ncmd)
    b = Batch(verbs, pts, off, np.asarray(xf, np.float32).reshape(n_fills, 6), None, raster_fill_off, n_rasters)
    b.validate()
    return b


def cubic_boxes(n_paths: int = 1000, seed: int = 1, canvas: float = 2048.0, box: float = 512.0,
                n_cubics: int = 16) -> Batch:
    rng = np.random.default_rng(seed)
    origin = rng.uniform(0.0, canvas - box, size=(n_paths, 2))
    start = origin + rng.uniform(0.0, box, size=(n_paths, 2))
    ctrl = origin[:, None, None, :] + rng.uniform(0.0, box, size=(n_paths, n_cubics, 3, 2))
    ctrl[:, -1, 2, :] = start  # the last cubic ends where the path started
    n_seg = np.full(n_paths, n_cubics, np.int64)
    kind = np.full(n_paths * n_cubics, CUBIC, np.uint8)
    seg = ctrl.reshape(-1, 6).astype(np.float32)
    verbs, pts, _ = _streams(n_seg, kind, start.astype(np.float32), seg)
    xf = np.tile(IDENTITY, (n_paths, 1))
    return _batch_from_streams(verbs, pts, n_seg + 2, np.arange(n_paths), xf, n_paths, None, n_paths)


def _blob_segments(rng, n_seg, centers, radii, direction, shape_p, kinds, jitter=0.08):
    """Closed blob contours (perturbed superellipses) as quadratic/cubic
    segments.  Returns (start_xy[n_c, 2], seg_floats[n_s, 6])."""
    n_c = len(n_seg)
    seg_contour = np.repeat(np.arange(n_c), n_seg)
    seg_start = np.concatenate([[0], np.cumsum(n_seg)[:-1]])
    k = np.arange(len(seg_contour)) - seg_start[seg_contour]
    n = n_seg[seg_contour].astype(np.float64)
    phase = rng.uniform(0, 2 * np.pi, size=n_c)

    def radius(theta, c):
        p = shape_p[c]
        ct, st = np.abs(np.cos(theta)), np.abs(np.sin(theta))
        return radii[c] / np.power(np.power(ct, p) + np.power(st, p), 1.0 / p)

    def point(theta, c, eps):
        r = radius(theta, c) * (1.0 + eps)
        return np.stack([centers[c, 0] + r * np.cos(theta), centers[c, 1] + r * np.sin(theta)], axis=-1)

    d = direction[seg_contour]
    # on-curve vertex k (vertex n == vertex 0)
    eps_v = rng.uniform(-jitter, jitter, size=len(seg_contour))
    theta0 = phase[seg_contour] + d * 2 * np.pi * k / n
    v0 = point(theta0, seg_contour, eps_v)
    # end vertex of each segment = start vertex of the next one in the contour
    nxt = np.arange(len(seg_contour)) + 1
    last_in_contour = k == n_seg[seg_contour] - 1
    nxt[last_in_contour] = seg_start[seg_contour[last_in_contour]]
    v1 = v0[nxt]
    step = d * 2 * np.pi / n
    seg = np.zeros((len(seg_contour), 6))
    q = kinds == QUADRATIC
    # quadratic: the control point makes the curve pass through the mid-angle point
    m = point(theta0 + 0.5 * step, seg_contour, rng.uniform(-jitter, jitter, size=len(seg_contour)))
    cq = 2.0 * m - 0.5 * (v0 + v1)
    seg[q, 0:2] = cq[q]
    seg[q, 2:4] = v1[q]
    # cubic: control points at 1/3 and 2/3 of the arc, pushed so the curve passes near them
    a1 = point(theta0 + step / 3.0, seg_contour, rng.uniform(-jitter, jitter, size=len(seg_contour)))
    a2 = point(theta0 + 2.0 * step / 3.0, seg_contour, rng.uniform(-jitter, jitter, size=len(seg_contour)))
    c1 = (-5.0 * v0 + 18.0 * a1 - 9.0 * a2 + 2.0 * v1) / 6.0
    c2 = (2.0 * v0 - 9.0 * a1 + 18.0 * a2 - 5.0 * v1) / 6.0
    seg[~q, 0:2] = c1[~q]
    seg[~q, 2:4] = c2[~q]
    seg[~q, 4:6] = v1[~q]
    start = v0[seg_start]
    return start, seg


def glyph_run(n_paths: int = 100_000, seed: int = 2, canvas: float = 4096.0) -> Batch:
    rng = np.random.default_rng(seed)
    n_seg_path = rng.integers(8, 41, size=n_paths)
    n_cont = rng.integers(1, 4, size=n_paths)
    # split each path's segments over its contours, each contour >= 2 segments
    cont_path = np.repeat(np.arange(n_paths), n_cont)
    first_c = np.concatenate([[0], np.cumsum(n_cont)[:-1]])
    ci = np.arange(len(cont_path)) - first_c[cont_path]
    w = rng.uniform(0.5, 1.0, size=len(cont_path))
    w[ci == 0] += 1.5  # outer contour gets the most segments
    wsum = np.bincount(cont_path, weights=w)
    spare = n_seg_path - 2 * n_cont
    share = np.floor(spare[cont_path] * w / wsum[cont_path]).astype(np.int64)
    rem = spare - np.bincount(cont_path, weights=share, minlength=n_paths).astype(np.int64)
    share[first_c] += rem
    n_seg = 2 + share
    em = rng.uniform(10.0, 48.0, size=n_paths)
    outer_r = 0.45 * em[cont_path]
    radii = np.where(ci == 0, outer_r, outer_r * rng.uniform(0.25, 0.45, size=len(cont_path)))
    centers = np.zeros((len(cont_path), 2))
    off_r = np.where(ci == 0, 0.0, outer_r * 0.35)
    ang = rng.uniform(0, 2 * np.pi, size=len(cont_path))
    centers[:, 0] = off_r * np.cos(ang)
    centers[:, 1] = off_r * np.sin(ang)
    direction = np.where(ci == 0, 1.0, -1.0)  # holes reversed
    shape_p = np.where(rng.uniform(size=len(cont_path)) < 0.5, 2.0, 4.0)
    kinds = np.full(int(n_seg.sum()), QUADRATIC, np.uint8)
    start, seg = _blob_segments(rng, n_seg, centers, radii, direction, shape_p, kinds)
    verbs, pts, _ = _streams(n_seg, kinds, start.astype(np.float32), seg.astype(np.float32))
    rot = rng.uniform(0, 2 * np.pi, size=n_paths)
    scale = rng.uniform(0.5, 2.0, size=n_paths)
    tr = rng.uniform(0.0, canvas, size=(n_paths, 2))
    xf = np.stack([scale * np.cos(rot), -scale * np.sin(rot), scale * np.sin(rot), scale * np.cos(rot),
                   tr[:, 0], tr[:, 1]], axis=1)
    return _batch_from_streams(verbs, pts, n_seg + 2, cont_path, xf, n_paths, None, n_paths)


def uneven_mix(n_paths: int = 20_000, seed: int = 3, canvas: float = 8192.0, median: float = 32.0,
               sigma: float = 1.5, max_seg: int = 20_000) -> Batch:
    rng = np.random.default_rng(seed)
    n_seg = np.clip(np.round(np.exp(rng.normal(math.log(median), sigma, size=n_paths))), 4, max_seg).astype(np.int64)
    total = int(n_seg.sum())
    kinds = np.where(rng.uniform(size=total) < 0.5, QUADRATIC, CUBIC).astype(np.uint8)
    s = rng.uniform(8.0, 200.0, size=n_paths)
    seg_path = np.repeat(np.arange(n_paths), n_seg)
    # random walk over all control points of a path (quadratics use 2 points, cubics 3)
    npt = np.where(kinds == QUADRATIC, 2, 3)
    start = rng.uniform(0.0, canvas, size=(n_paths, 2))
    steps = rng.normal(0.0, 1.0, size=(int(npt.sum()), 2)) * s[np.repeat(seg_path, npt)][:, None]
    pt_path = np.repeat(seg_path, npt)
    pstart = np.concatenate([[0], np.cumsum(np.bincount(pt_path, minlength=n_paths))[:-1]])
    walk = np.cumsum(steps, axis=0)
    # make each path's walk start from its own start point
    walk_prev = np.concatenate([np.zeros((1, 2)), walk[:-1]])
    base = walk_prev[pstart]
    walk = walk - base[pt_path] + start[pt_path]

    def reflect(v):
        period = 2.0 * canvas
        v = np.mod(v, period)
        v = np.where(v >= canvas, period - v, v)
        return np.minimum(v, np.nextafter(canvas, 0))

    walk = reflect(walk)
    seg = np.zeros((total, 6))
    first_pt = np.concatenate([[0], np.cumsum(npt)[:-1]])
    for j in range(3):
        has = j < npt
        seg[has, 2 * j:2 * j + 2] = walk[first_pt[has] + j]
    verbs, pts, _ = _streams(n_seg, kinds, start.astype(np.float32), seg.astype(np.float32))
    xf = np.tile(IDENTITY, (n_paths, 1))
    return _batch_from_streams(verbs, pts, n_seg + 2, np.arange(n_paths), xf, n_paths, None, n_paths)


def diff_union(n_paths: int = 256, seed: int = 4, canvas: float = 1024.0, n_cubics: int = 32,
               perturb: float = 0.0, base_seed: Optional[int] = None) -> Batch:
    """256 closed cubic blobs in ONE rasterizer (one fill per blob)."""
    rng = np.random.default_rng(seed if base_seed is None else base_seed)
    n_seg = np.full(n_paths, n_cubics, np.int64)
    centers = rng.uniform(64.0, canvas - 64.0, size=(n_paths, 2))
    radii = rng.uniform(16.0, 56.0, size=n_paths)
    direction = np.ones(n_paths)
    shape_p = np.full(n_paths, 2.0)
    kinds = np.full(n_paths * n_cubics, CUBIC, np.uint8)
    start, seg = _blob_segments(rng, n_seg, centers, radii, direction, shape_p, kinds, jitter=0.15)
    if perturb > 0.0:
        prng = np.random.default_rng(seed + 1000)
        seg = seg + prng.normal(0.0, perturb, size=seg.shape)
        # keep contours closed: the last segment of each contour ends at its (perturbed) start
        start = start + prng.normal(0.0, perturb, size=start.shape)
        last = np.cumsum(n_seg) - 1
        seg[last, 4:6] = start
    verbs, pts, _ = _streams(n_seg, kinds, start.astype(np.float32), seg.astype(np.float32))
    xf = np.tile(IDENTITY, (n_paths, 1))
    roff = np.array([0, n_paths], np.uint32)
    return _batch_from_streams(verbs, pts, n_seg + 2, np.arange(n_paths), xf, n_paths, roff, 1)


def diff_scenes(n_scenes: int = 4096, seed: int = 5, size: float = 512.0, min_paths: int = 8,
                max_paths: int = 512, min_seg: int = 4, max_seg: int = 128) -> Batch:
    """Independent scenes (one rasterizer each) of mixed quadratic/cubic blobs."""
    rng = np.random.default_rng(seed)
    n_paths_scene = rng.integers(min_paths, max_paths + 1, size=n_scenes)
    n_fills = int(n_paths_scene.sum())
    fill_scene = np.repeat(np.arange(n_scenes), n_paths_scene)
    n_seg = rng.integers(min_seg, max_seg + 1, size=n_fills)
    kinds = np.where(rng.uniform(size=int(n_seg.sum())) < 0.5, QUADRATIC, CUBIC).astype(np.uint8)
    radii = rng.uniform(6.0, 48.0, size=n_fills)
    centers = rng.uniform(0.0, size, size=(n_fills, 2)) - 0.5 * size
    direction = np.where(rng.uniform(size=n_fills) < 0.8, 1.0, -1.0)
    shape_p = np.where(rng.uniform(size=n_fills) < 0.5, 2.0, 4.0)
    start, seg = _blob_segments(rng, n_seg, centers, radii, direction, shape_p, kinds)
    verbs, pts, _ = _streams(n_seg, kinds, start.astype(np.float32), seg.astype(np.float32))
    rot = rng.uniform(-0.3, 0.3, size=n_scenes)
    sc = rng.uniform(0.8, 1.0, size=n_scenes)
    sh = rng.uniform(-0.1, 0.1, size=n_scenes)
    m0 = sc * np.cos(rot)
    m1 = -sc * np.sin(rot) + sh
    m2 = sc * np.sin(rot)
    m3 = sc * np.cos(rot)
    xf_scene = np.stack([m0, m1, m2, m3, np.full(n_scenes, 0.5 * size), np.full(n_scenes, 0.5 * size)], axis=1)
    xf = xf_scene[fill_scene]
    roff = np.zeros(n_scenes + 1, np.uint32)
    roff[1:] = np.cumsum(n_paths_scene)
    return _batch_from_streams(verbs, pts, n_seg + 2, np.arange(n_fills), xf, n_fills, roff, n_scenes)


def stroke_run(n_paths: int = 20_000, seed: int = 6, canvas: float = 2048.0) -> Batch:
    """Stroked paths (Rasterizer::stroke), one rasterizer each: open and
    closed contours of 2-24 mixed line / quadratic / cubic segments (a random
    walk with steps of 4-60 px), widths 0.5-8 px, random rotation and scale
    0.5-2 per path, placed on a canvas.  About a quarter are closed."""
    from .batch import FILL_STROKE, LINE
    rng = np.random.default_rng(seed)
    n_seg = rng.integers(2, 25, size=n_paths)
    closed = rng.uniform(size=n_paths) < 0.25
    tot = int(n_seg.sum())
    kinds = rng.choice(np.array([LINE, QUADRATIC, CUBIC], np.uint8), size=tot, p=[0.4, 0.3, 0.3])
    step = rng.uniform(4.0, 60.0, size=n_paths)
    seg_path = np.repeat(np.arange(n_paths), n_seg)
    # every segment gets 3 random-walk points; lines use the last, quadratics the last 2
    walk = rng.normal(0.0, 1.0, size=(tot, 3, 2)) * step[seg_path, None, None]
    ends = np.cumsum(walk.reshape(-1, 2), axis=0).reshape(tot, 3, 2)
    first = np.concatenate([[0], np.cumsum(n_seg)[:-1]])
    base = ends[first, 0] - walk[first, 0]          # path start: the walk's origin
    ends = ends - np.repeat(base, n_seg, axis=0)[:, None, :]
    ncmd = n_seg + 1 + closed.astype(np.int64)
    verbs = np.empty(int(ncmd.sum()), np.uint8)
    cstart = np.concatenate([[0], np.cumsum(ncmd)[:-1]])
    verbs[cstart] = MOVE
    seg_local = np.arange(tot) - first[seg_path]
    seg_cmd = cstart[seg_path] + 1 + seg_local
    verbs[seg_cmd] = kinds
    verbs[(cstart + ncmd - 1)[closed]] = CLOSE
    fpv = FLOATS_PER_VERB[verbs]
    foff = np.concatenate([[0], np.cumsum(fpv)]).astype(np.int64)
    pts = np.zeros(int(foff[-1]), np.float32)
    o = foff[seg_cmd]
    lin = kinds == LINE
    pts[o[lin]], pts[o[lin] + 1] = ends[lin, 2, 0], ends[lin, 2, 1]
    q = kinds == QUADRATIC
    pts[o[q]], pts[o[q] + 1], pts[o[q] + 2], pts[o[q] + 3] = ends[q, 1, 0], ends[q, 1, 1], ends[q, 2, 0], ends[q, 2, 1]
    c = kinds == CUBIC
    for k in range(3):
        pts[o[c] + 2 * k], pts[o[c] + 2 * k + 1] = ends[c, k, 0], ends[c, k, 1]
    ang = rng.uniform(0.0, 2.0 * np.pi, size=n_paths)
    sc = rng.uniform(0.5, 2.0, size=n_paths)
    tx = rng.uniform(128.0, canvas - 128.0, size=(n_paths, 2))
    xf = np.stack([sc * np.cos(ang), -sc * np.sin(ang), sc * np.sin(ang), sc * np.cos(ang), tx[:, 0], tx[:, 1]], axis=1)
    off = np.concatenate([[0], np.cumsum(ncmd)]).astype(np.uint32)
    flags = np.full(n_paths, FILL_STROKE, np.uint8)
    width = rng.uniform(0.5, 8.0, size=n_paths).astype(np.float32)
    b = Batch(verbs, pts, off, xf.astype(np.float32), flags, None, n_paths, width)
    b.validate()
    return b


CONFIGS = {
    1: ("cubic_boxes", cubic_boxes),
    2: ("glyph_run", glyph_run),
    3: ("uneven_mix", uneven_mix),
    4: ("diff_union", diff_union),
    5: ("diff_scenes", diff_scenes),
}
