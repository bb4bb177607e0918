"""Stroke edge cases (Rasterizer::stroke, rasterizer.rs:169-171 with
path.rs:113-274): closed and open contours, sharp joins (two-point joins),
zero-length segments, the sticky `closed` flag after a Close, curves and a
conic, a path that starts with a Line, a lone Move, raw and transformed
strokes, and a stroke united with a fill in one rasterizer."""
import numpy as np

from ochre_gb300.batch import BatchBuilder

ROT = [0.8660254, -0.5, 0.5, 0.8660254, 40.25, 12.5]

# (name, [(verbs, pts, transform, raw, stroke_width or None)])
CASES = {
    "closed_rect": [([0, 1, 1, 1, 5], [10.5, 10.25, 50.5, 10.25, 50.5, 40.75, 10.5, 40.75], None, False, 4.0)],
    "open_polyline_sharp": [([0, 1, 1, 1], [5.5, 5.5, 60.25, 9.0, 8.0, 14.5, 62.0, 30.0], None, False, 3.0)],
    "cubic_open": [([0, 3], [4.0, 40.0, 20.0, 2.0, 60.0, 70.0, 76.0, 12.0], None, False, 2.5)],
    "quad_close_then_line": [([0, 2, 5, 1, 1], [10.0, 10.0, 40.0, 0.5, 60.0, 30.0, 20.0, 50.0, 70.0, 60.0],
                              None, False, 5.0)],
    "lone_move": [([0], [30.0, 30.0], None, False, 6.0)],
    "duplicate_points": [([0, 1, 1, 1, 1, 5], [10.0, 10.0, 10.0, 10.0, 40.0, 12.0, 40.0, 12.0, 30.0, 40.0],
                          None, False, 3.0)],
    "two_open_contours": [([0, 1, 1, 0, 1], [5.0, 5.0, 30.0, 5.5, 31.0, 30.0, 50.0, 50.0, 70.0, 20.0],
                           None, False, 2.0)],
    "conic": [([0, 4, 1], [10.0, 50.0, 40.0, 0.0, 70.0, 50.0, 0.7, 10.0, 50.0], None, False, 3.5)],
    "rotated": [([0, 1, 2, 5], [0.0, 0.0, 50.0, 0.0, 60.0, 40.0, 10.0, 30.0], ROT, False, 4.0)],
    "raw_stroke": [([0, 1, 1], [20.0, 20.0, 60.0, 22.0, 40.0, 60.0], None, True, 7.0)],
    "starts_with_line": [([1, 1, 1], [30.0, 10.0, 50.0, 40.0, 10.0, 40.0], None, False, 3.0)],
    "stroke_and_fill": [([0, 1, 1, 1, 5], [10.0, 10.0, 60.0, 10.0, 60.0, 60.0, 10.0, 60.0], None, False, None),
                        ([0, 1, 1, 1, 5], [20.0, 20.0, 50.0, 20.0, 50.0, 50.0, 20.0, 50.0], None, False, 6.0)],
    "hairline": [([0, 3, 5], [8.0, 8.0, 30.0, 90.0, 80.0, -20.0, 90.0, 70.0], None, False, 0.75)],
    "reversal": [([0, 1, 1], [10.0, 30.0, 70.0, 30.0, 20.0, 30.0], None, False, 4.0)],
}


def stroke_batch():
    bb = BatchBuilder()
    for fills in CASES.values():
        bb.begin_raster()
        for verbs, pts, xf, raw, width in fills:
            bb.fill(verbs, pts, xf, raw=raw, stroke_width=width)
    return bb.build(), list(CASES)
