"""Edge-case rasters drawn from the reference's behaviour (test inputs).

Each entry is one raster (one Rasterizer::new -> fill*/move_to/line_to ->
finish sequence); ``edge_batch()`` packs them all into one Batch.
"""
from __future__ import annotations

import math

import numpy as np

from ochre_gb300.batch import CLOSE, CONIC, CUBIC, IDENTITY, LINE, MOVE, QUADRATIC, BatchBuilder


def _rot(a, s=1.0, tx=0.0, ty=0.0):
    return [s * math.cos(a), -s * math.sin(a), s * math.sin(a), s * math.cos(a), tx, ty]


# name -> list of (verbs, floats, transform or None for raw)
CASES = {
    # rasterizer.rs:194-208: no increments still emits one zero tile at (0,0)
    "empty": [],
    "only_move": [([MOVE], [10.0, 10.0], IDENTITY)],
    "zero_length_lines": [([MOVE, LINE, LINE, CLOSE], [5.0, 5.0, 5.0, 5.0, 5.0, 5.0], IDENTITY)],
    # a path with no Move starts at (0, 0) (rasterizer.rs:54-55)
    "no_move": [([LINE, LINE, LINE], [20.0, 0.0, 20.0, 20.0, 0.0, 20.0], IDENTITY)],
    # Close is a no-op: the next Line continues from the previous point (rasterizer.rs:154)
    "close_then_line": [([MOVE, LINE, LINE, CLOSE, LINE, LINE],
                         [2.0, 2.0, 30.0, 2.0, 30.0, 30.0, 2.0, 30.0, 16.0, 40.0], IDENTITY)],
    "pixel_square": [([MOVE, LINE, LINE, LINE, CLOSE], [1.0, 1.0, 3.0, 1.0, 3.0, 3.0, 1.0, 3.0], None)],
    "rect_spans": [([MOVE, LINE, LINE, LINE, CLOSE], [4.0, 4.0, 60.0, 4.0, 60.0, 28.0, 4.0, 28.0], IDENTITY)],
    # exact pixel corners and diagonals (ties step x first, rasterizer.rs:108)
    "diagonals": [([MOVE, LINE, LINE, LINE, CLOSE], [0.0, 0.0, 16.0, 16.0, 32.0, 0.0, 16.0, -16.0], IDENTITY)],
    "horizontal_vertical": [([MOVE, LINE, LINE, LINE, LINE, LINE, CLOSE],
                             [0.5, 0.5, 40.5, 0.5, 40.5, 9.0, 20.0, 9.0, 20.0, 30.25, 0.5, 30.25], IDENTITY)],
    "negative_coords": [([MOVE, QUADRATIC, CUBIC, CLOSE],
                         [-30.0, -20.0, -5.0, -60.0, 25.0, -18.0, 10.0, 5.0, -40.0, 12.0, -30.0, -20.0], IDENTITY)],
    # zero curvature: |last - 2c + p| = 0 -> dt = inf -> one line (path.rs:50)
    "degenerate_quad": [([MOVE, QUADRATIC, LINE, CLOSE], [0.0, 0.0, 10.0, 10.0, 20.0, 20.0, 0.0, 20.0], IDENTITY)],
    "degenerate_cubic": [([MOVE, CUBIC, CUBIC, CLOSE],
                          [3.0, 3.0, 3.0, 3.0, 3.0, 3.0, 3.0, 3.0, 10.0, 4.0, 20.0, 30.0, 3.0, 20.0], IDENTITY)],
    "conic": [([MOVE, CONIC, CONIC, CLOSE],
               [50.0, 10.0, 90.0, 10.0, 90.0, 50.0, 0.7071068, 90.0, 90.0, 50.0, 90.0, 2.0], IDENTITY)],
    # two fills with different transforms on one rasterizer (union, shared state)
    "multi_fill": [([MOVE, QUADRATIC, LINE, CLOSE], [0.0, 0.0, 20.0, -10.0, 40.0, 0.0, 20.0, 30.0],
                    _rot(0.3, 1.5, 100.0, 50.0)),
                   ([LINE, CUBIC, CLOSE], [10.0, 10.0, 30.0, -20.0, 60.0, 40.0, 0.0, 30.0], _rot(-1.1, 0.8, 80.0, 90.0))],
    # raw commands (move_to / line_to / command) mixed with a transformed fill
    "raw_then_fill": [([MOVE, LINE, LINE], [3.5, 3.5, 70.25, 9.75, 40.0, 60.0], None),
                      ([QUADRATIC, CLOSE, MOVE, LINE, LINE], [0.0, 0.0, 5.0, 5.0, 50.0, 50.0, 90.0, 50.0, 70.0, 90.0],
                       _rot(0.0, 1.0, 0.0, 0.0))],
    "holes_and_overlap": [([MOVE, LINE, LINE, LINE, CLOSE, MOVE, LINE, LINE, LINE, CLOSE, MOVE, LINE, LINE, LINE, CLOSE],
                           [8.0, 8.0, 120.0, 8.0, 120.0, 100.0, 8.0, 100.0,
                            30.0, 30.0, 30.0, 70.0, 90.0, 70.0, 90.0, 30.0,
                            60.0, 20.0, 140.0, 20.0, 140.0, 60.0, 60.0, 60.0], IDENTITY)],
    # a long line and subpixel slivers
    "long_thin": [([MOVE, LINE, LINE, CLOSE], [1.3, 2.7, 1500.9, 250.1, 1500.2, 252.6], IDENTITY)],
    "tiny": [([MOVE, LINE, LINE, CLOSE], [5.1, 5.1, 5.3, 5.15, 5.2, 5.4], IDENTITY)],
    # figure eight: self-intersection with winding +1 and -1 lobes
    "figure_eight": [([MOVE, CUBIC, CUBIC, CLOSE],
                      [64.0, 64.0, 200.0, -60.0, 200.0, 190.0, 64.0, 64.0, -70.0, -60.0, -70.0, 190.0, 64.0, 64.0],
                      IDENTITY)],
}


# Rasters at the i16 limits (rasterizer.rs:78-79, 108-116): `floor(p) as i16`
# saturates at 32767 / -32768 and the walk's `x += x_dir` wraps (release-build
# integer arithmetic), so a walk that
# passes 32767 continues at -32768 (tiles at both ends of the i16 range, a span
# 65,520 px wide, a y wrap covering 16,390 tiles).  A batch of their own: none
# of them fits the fused kernel's grid, and the dense-canvas tests keep to
# small coordinates.
I16_CASES = {
    "i16_wrap_x": [([MOVE, LINE, LINE, LINE, CLOSE],
                    [32760.5, 10.5, 32775.5, 14.5, 32775.5, 30.5, 32760.5, 30.5], IDENTITY)],
    "i16_wrap_neg_x": [([MOVE, LINE, LINE, CLOSE], [-32765.5, 3.5, -32775.0, 9.0, -32760.0, 20.0], IDENTITY)],
    "i16_wrap_y": [([MOVE, QUADRATIC, LINE, CLOSE],
                    [100.25, 32758.0, 140.0, 32790.0, 120.0, 32762.5, 90.0, 32750.0], IDENTITY)],
    "i16_far_both": [([MOVE, LINE, LINE, CLOSE],
                      [-32766.0, -32766.0, -32760.0, -32771.0, -32770.0, -32760.0], IDENTITY)],
}


def _batch(cases):
    bb = BatchBuilder()
    for name, fills in cases.items():
        bb.begin_raster()
        for verbs, pts, xf in fills:
            bb.fill(verbs, pts, IDENTITY if xf is None else xf, raw=xf is None)
    return bb.build(), list(cases)


def edge_batch():
    return _batch(CASES)


def i16_batch():
    return _batch(I16_CASES)
