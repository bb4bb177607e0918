"""Seeded random rasters for fuzz tests (test inputs).

Each raster is one to three fills of random command sequences: every verb,
in any order (Close without a Move, repeated points, points on pixel
corners, degenerate curves, conics with weights from 0.2 to 3), random
affine transforms (rotation, anisotropic scale, shear, translation) or
device-space (raw) commands.  Ordinary rasters fit the fused kernel; the
large share (eight times the size, fills that may lack a leading Move and so
start at the origin) does not, and sends its batch to the general chain.
"""
from __future__ import annotations

import numpy as np

from ochre_gb300.batch import CLOSE, CONIC, CUBIC, LINE, MOVE, QUADRATIC, BatchBuilder

_FLOATS = {MOVE: 2, LINE: 2, QUADRATIC: 4, CUBIC: 6, CONIC: 5, CLOSE: 0}


def _fill(rng, span, lead_move):
    # ordinary rasters: three fills stay within 64 commands and 256 lines
    n = int(rng.integers(1, 20 if lead_move else 24))
    verbs = rng.choice([MOVE, LINE, QUADRATIC, CUBIC, CONIC, CLOSE], size=n,
                       p=[0.12, 0.3, 0.2, 0.2, 0.06, 0.12]).astype(np.uint8)
    # without a leading Move a fill starts at the origin (rasterizer.rs:54-55)
    if lead_move or rng.random() < 0.8:
        verbs[0] = MOVE
    base = rng.uniform(-span * 0.15, span * 0.15, size=2)
    pts = []
    prev = base.copy()
    for v in verbs:
        k = _FLOATS[int(v)]
        if k == 0:
            continue
        m = k // 2 if v != CONIC else 2
        for _ in range(m):
            if rng.random() < 0.08:
                p = prev.copy()                     # repeated point
            elif rng.random() < 0.05:
                p = np.floor(prev) + rng.integers(-3, 4, size=2)   # pixel corners
            else:
                p = prev + rng.normal(0.0, span * 0.05, size=2)
            pts.extend(p.tolist())
            prev = p
        if v == CONIC:
            pts.append(float(rng.choice([0.2, 0.7071068, 1.0, 3.0])))
    return verbs, np.asarray(pts, np.float32)


def _shift(verbs, pts, d):
    """Points moved by d (conic weights untouched)."""
    out = pts.copy()
    k = 0
    for v in verbs:
        n = _FLOATS[int(v)]
        pairs = 2 if v == CONIC else n // 2
        for j in range(pairs):
            out[k + 2 * j] += np.float32(d[0])
            out[k + 2 * j + 1] += np.float32(d[1])
        k += n
    return out


def _transform(rng, center):
    a = rng.uniform(-np.pi, np.pi)
    sx, sy = rng.uniform(0.3, 2.0, size=2)
    sh = rng.uniform(-0.5, 0.5)
    c, s = np.cos(a), np.sin(a)
    m = np.array([[c, -s], [s, c]]) @ np.array([[sx, sh], [0.0, sy]])
    t = center + rng.normal(0.0, 10.0, size=2)
    return [m[0, 0], m[0, 1], m[1, 0], m[1, 1], t[0], t[1]]


def fuzz_batch(n_rasters: int, seed: int, span: float = 60.0, big_share: float = 0.1, stroke_share: float = 0.0):
    """``big_share`` of the rasters are eight times larger (most of those do
    not fit the fused kernel, so the batch runs on the general chain);
    ``stroke_share`` of the transformed fills are strokes (width 0.25-12)."""
    rng = np.random.default_rng(seed)
    bb = BatchBuilder()
    for _ in range(n_rasters):
        bb.begin_raster()
        big = rng.random() < big_share
        center = rng.uniform(0, 700, size=2)     # the fills of a raster stay together
        for _ in range(int(rng.integers(1, 4))):
            verbs, pts = _fill(rng, span * (8.0 if big else 1.0), lead_move=not big)
            if rng.random() < 0.15:
                bb.fill(verbs, _shift(verbs, pts, center), [1.0, 0.0, 0.0, 1.0, 0.0, 0.0], raw=True)
            elif rng.random() < stroke_share:
                bb.fill(verbs, pts, _transform(rng, center), stroke_width=float(rng.uniform(0.25, 12.0)))
            else:
                bb.fill(verbs, pts, _transform(rng, center))
    return bb.build()
