"""CPU tests of the oracle: pinned against hand-derived answers of the
reference's semantics, against an independent Python restatement, and against
the committed golden fixtures."""
import numpy as np
import pytest

import oracle
import oracle_py
from golden.make_golden import NAMES, load
from ochre_gb300 import workloads as W


def _raster(r, i):
    t0, t1 = int(r["raster_tile_off"][i]), int(r["raster_tile_off"][i + 1])
    s0, s1 = int(r["raster_span_off"][i]), int(r["raster_span_off"][i + 1])
    return (r["tile_xy"][t0:t1], r["tile_alpha"][t0:t1], r["span_xy"][s0:s1], r["span_w"][s0:s1],
            r["span_tile"][s0:s1] - t0)


@pytest.mark.parametrize("name", NAMES)
def test_oracle_reproduces_golden(name):
    b, exp = load(name)
    r = oracle.run(b, want_cov=True)
    assert r["status"] == 0
    for k, v in exp.items():
        assert np.array_equal(r[k], v), k


def test_known_answer_empty_raster():
    # rasterizer.rs:194-208: no increments -> one all-zero tile at (0, 0)
    from ochre_gb300.batch import BatchBuilder
    b = BatchBuilder().begin_raster().build()
    r = oracle.run(b)
    assert r["tile_xy"].tolist() == [[0, 0]]
    assert not r["tile_alpha"].any()
    assert len(r["span_w"]) == 0


def test_known_answer_pixel_square():
    # Square (1,1)-(3,3): the right edge pushes area +1 per cell at x=3, the
    # left edge -1 at x=1; accum = -1 between them -> |.| = 1 -> 255.
    from ochre_gb300.batch import CLOSE, LINE, MOVE, BatchBuilder
    b = BatchBuilder().fill([MOVE, LINE, LINE, LINE, CLOSE], [1, 1, 3, 1, 3, 3, 1, 3], raw=True).build()
    r = oracle.run(b)
    expect = np.zeros((8, 8), np.uint8)
    expect[1:3, 1:3] = 255
    assert r["tile_xy"].tolist() == [[0, 0]]
    assert np.array_equal(r["tile_alpha"][0].reshape(8, 8), expect)


def test_known_answer_rectangle_spans():
    # Rectangle x 4..60, y 4..28: tile rows 0 and 3 are crossed by the
    # horizontal edges (zero-height increments still create tiles); rows 1, 2
    # hold only the left (tile 0) and right (tile 7) edge tiles.  Crossings of
    # tile-row boundaries: left edge (going up) -1 at tile_x 0, right edge
    # (going down) +1 at tile_x 7; the winding after tile (0, ty) is -1, so a
    # span of 6 tiles (48 px) follows tile 0 on rows 1 and 2.
    from ochre_gb300.batch import CLOSE, LINE, MOVE, BatchBuilder
    b = BatchBuilder().fill([MOVE, LINE, LINE, LINE, CLOSE], [4, 4, 60, 4, 60, 28, 4, 28]).build()
    r = oracle.run(b)
    xy, alpha, sxy, sw, st = _raster(r, 0)
    expect_tiles = ([(8 * i, 0) for i in range(8)] + [(0, 8), (56, 8), (0, 16), (56, 16)]
                    + [(8 * i, 24) for i in range(8)])
    assert [tuple(t) for t in xy.tolist()] == expect_tiles
    assert sxy.tolist() == [[8, 8], [8, 16]]
    assert sw.tolist() == [48, 48]
    assert st.tolist() == [8, 10]
    left = alpha[8].reshape(8, 8)
    right = alpha[9].reshape(8, 8)
    assert np.array_equal(left, np.tile([0, 0, 0, 0, 255, 255, 255, 255], (8, 1)))
    assert np.array_equal(right, np.tile([255, 255, 255, 255, 0, 0, 0, 0], (8, 1)))


def test_known_answer_half_pixel_edge():
    # A vertical edge at x = 2.5 from y=0 down to y=8 and back along x = 0:
    # cell x=2 gets area 0.5*h*((3-2.5)+(3-2.5)) = 0.5 per row -> |-1 + 0.5|
    # ... with accum -1 from the left edge: coverage 0.5 -> 128.
    from ochre_gb300.batch import CLOSE, LINE, MOVE, BatchBuilder
    b = BatchBuilder().fill([MOVE, LINE, LINE, LINE, CLOSE], [0, 0, 2.5, 0, 2.5, 8, 0, 8], raw=True).build()
    r = oracle.run(b)
    a = r["tile_alpha"][0].reshape(8, 8)
    assert np.array_equal(a, np.tile([255, 255, 128, 0, 0, 0, 0, 0], (8, 1)))


@pytest.mark.parametrize("verb,ctrl,n_curve", [
    # Quadratic (path.rs:49-58): |last - 2c + p| = |(0, -200)| = 200, so
    # dt = sqrt(4 * 0.1 / 200) = 0.04472; 22 steps reach 0.9839 and the 23rd
    # is clamped to 1: 23 lines.
    ("quad", [50, 100, 100, 0], 23),
    # Cubic (path.rs:59-74): a = -last + 3 c1 - 3 c2 + p = (-200, 0),
    # b = 3 (last - 2 c1 + c2) = (300, -300), conc = max(|b|, |a + b|)
    # = max(424.26, 316.23); dt = sqrt(sqrt(8) * 0.1 / 424.26) = 0.02582;
    # 38 steps reach 0.9812 and the 39th is clamped to 1: 39 lines.
    ("cubic", [0, 100, 100, 100, 100, 0], 39),
])
def test_known_answer_flatten_counts(verb, ctrl, n_curve):
    # Move (0, 0), the curve to (100, 0), Close: the curve's lines plus the
    # closing line (100, 0) -> (0, 0) that finish adds (rasterizer.rs:181-183),
    # each line starting where the previous one ended.
    from ochre_gb300.batch import CLOSE, CUBIC, MOVE, QUADRATIC, BatchBuilder
    v = {"quad": QUADRATIC, "cubic": CUBIC}[verb]
    b = BatchBuilder().fill([MOVE, v, CLOSE], [0, 0] + ctrl, raw=True).build()
    r = oracle.run(b, capture_lines=True)
    L = r["lines"][int(r["raster_line_off"][0]):int(r["raster_line_off"][1])]
    assert len(L) == n_curve + 1
    assert np.array_equal(L[1:, :2], L[:-1, 2:])
    assert L[0, :2].tolist() == [0, 0] and L[n_curve - 1, 2:].tolist() == [100, 0]
    assert L[n_curve].tolist() == [100, 0, 0, 0]


def test_known_answer_close_and_move_semantics():
    # Close is a no-op (rasterizer.rs:154): a Line after it starts at the
    # last point, so Move (0,0), Line (8,0), Line (8,8), Close, Line (0,8)
    # outlines the whole tile, and finish closes (0,8) -> (0,0); the edges on
    # x = 8 and y = 8 walk cells of the next tiles (floor(8) = 8), which get
    # coverage 0 (the right edge's area cancels the carry).  A Move
    # closes the contour before it when last != first (rasterizer.rs:62-64):
    # the second raster's Move (16,0) adds (8,8) -> (0,0) first, and its own
    # contour (16,0) -> (24,0) -> (24,8) is closed by finish.
    from ochre_gb300.batch import CLOSE, LINE, MOVE, BatchBuilder
    bb = BatchBuilder()
    bb.begin_raster()
    bb.fill([MOVE, LINE, LINE, CLOSE, LINE], [0, 0, 8, 0, 8, 8, 0, 8], raw=True)
    bb.begin_raster()
    bb.fill([MOVE, LINE, LINE, MOVE, LINE, LINE], [0, 0, 8, 0, 8, 8, 16, 0, 24, 0, 24, 8], raw=True)
    r = oracle.run(bb.build(), capture_lines=True)
    lines = [r["lines"][int(r["raster_line_off"][i]):int(r["raster_line_off"][i + 1])].tolist() for i in range(2)]
    assert lines[0] == [[0, 0, 8, 0], [8, 0, 8, 8], [8, 8, 0, 8], [0, 8, 0, 0]]
    assert lines[1] == [[0, 0, 8, 0], [8, 0, 8, 8], [8, 8, 0, 0],
                        [16, 0, 24, 0], [24, 0, 24, 8], [24, 8, 16, 0]]
    xy, alpha, _, sw, _ = _raster(r, 0)
    assert xy.tolist() == [[0, 0], [8, 0], [0, 8], [8, 8]] and len(sw) == 0
    assert (alpha[0] == 255).all() and not alpha[1:].any()


def test_known_answer_union_of_fills():
    # Several fills on one rasterizer add into one accumulation
    # (rasterizer.rs:161-165).  Raster 0: the square x 0..2.5, y 0..8 twice
    # in the same direction: coverage 2 in columns 0-1 and 2 * 0.5 = 1 in
    # column 2, alpha min(|S| * 256, 255) = 255 for all three (the cast
    # saturates).  Raster 1: the same square and its reverse: S = 0
    # everywhere, the tiles are still emitted (their cells had increments)
    # with alpha 0.
    from ochre_gb300.batch import CLOSE, LINE, MOVE, BatchBuilder
    fwd = [0, 0, 2.5, 0, 2.5, 8, 0, 8]
    rev = [0, 0, 0, 8, 2.5, 8, 2.5, 0]
    verbs = [MOVE, LINE, LINE, LINE, CLOSE]
    bb = BatchBuilder()
    bb.begin_raster()
    bb.fill(verbs, fwd, raw=True)
    bb.fill(verbs, fwd, raw=True)
    bb.begin_raster()
    bb.fill(verbs, fwd, raw=True)
    bb.fill(verbs, rev, raw=True)
    r = oracle.run(bb.build())
    xy0, a0, _, _, _ = _raster(r, 0)
    xy1, a1, _, _, _ = _raster(r, 1)
    assert xy0.tolist() == [[0, 0], [0, 8]] == xy1.tolist()
    assert np.array_equal(a0[0].reshape(8, 8), np.tile([255, 255, 255, 0, 0, 0, 0, 0], (8, 1)))
    assert not a0[1].any() and not a1.any()


@pytest.mark.parametrize("hole", [True, False])
def test_known_answer_nonzero_winding(hole):
    # Square x, y in [0, 64] with a second contour x, y in [16, 48] in the
    # same fill, reversed (a hole) or in the same direction (an overlap).
    # Tile rows 3-5 (y 24..47) hold only vertical edges: cells x = 0, 16, 48
    # and 64 put tiles at tile x 0, 2, 6 and 8.  Crossings of each tile-row
    # boundary add -1 at an up edge and +1 at a down edge, so the winding
    # after tile 0 is -1 (span over tile 1), after tile 2 is 0 for the hole
    # (no span over tiles 3-5) or -2 for the overlap (a 24-px span), after
    # tile 6 is -1 (span over tile 7) (rasterizer.rs:252-265).  Coverage:
    # tile 0 is 1, tile 2 is 0 (hole) or 2 (overlap, saturating to 255),
    # tile 6 is 1, tile 8 is 0.
    from ochre_gb300.batch import CLOSE, LINE, MOVE, BatchBuilder
    outer = [0, 0, 64, 0, 64, 64, 0, 64]
    inner = [16, 16, 16, 48, 48, 48, 48, 16] if hole else [16, 16, 48, 16, 48, 48, 16, 48]
    verbs = [MOVE, LINE, LINE, LINE, CLOSE] * 2
    r = oracle.run(BatchBuilder().fill(verbs, outer + inner, raw=True).build())
    xy, alpha, sxy, sw, st = _raster(r, 0)
    for ty in (3, 4, 5):
        rows = [i for i, (x, y) in enumerate(xy.tolist()) if y == 8 * ty]
        assert [xy[i][0] for i in rows] == [0, 16, 48, 64], ty
        full = [255, 0, 255, 0] if hole else [255, 255, 255, 0]
        for i, a in zip(rows, full):
            assert (alpha[i] == a).all(), (ty, int(xy[i][0]))
        spans = [(int(x), int(w), int(t)) for (x, y), w, t in zip(sxy.tolist(), sw, st) if y == 8 * ty]
        expect = [(8, 8, rows[0]), (56, 8, rows[2])] if hole else [(8, 8, rows[0]), (24, 24, rows[1]), (56, 8, rows[2])]
        assert spans == expect, ty


def test_known_answer_sloped_triangle():
    # Triangle (0.5, 0.5) -> (2.5, 2.5) -> (0.5, 2.5): the region
    # 0.5 <= x <= y <= 2.5.  Per pixel (x, y) the covered area is
    # (0,0) 1/8, (0,1) 1/2, (0,2) 1/4, (1,1) 1/2, (1,2) 1/2, (2,2) 1/8, else 0;
    # every term of the reference's sums is a multiple of 1/8, so the f32
    # coverage is exact and alpha = (area * 256) as u8 (rasterizer.rs:232-239).
    # The diagonal passes through pixel corners, where the walk steps x first
    # and adds zero-length increments (rasterizer.rs:108-116).
    from ochre_gb300.batch import CLOSE, LINE, MOVE, BatchBuilder
    b = BatchBuilder().fill([MOVE, LINE, LINE, CLOSE], [0.5, 0.5, 2.5, 2.5, 0.5, 2.5], raw=True).build()
    r = oracle.run(b)
    expect = np.zeros((8, 8), np.uint8)
    for (x, y), a in {(0, 0): 32, (0, 1): 128, (0, 2): 64, (1, 1): 128, (1, 2): 128, (2, 2): 32}.items():
        expect[y, x] = a
    assert r["tile_xy"].tolist() == [[0, 0]]
    assert np.array_equal(r["tile_alpha"][0].reshape(8, 8), expect)
    assert len(r["span_w"]) == 0


def test_known_answer_negative_coordinates():
    # Square x, y in [-12, -4]: cells and tiles use floor and div_euclid
    # (rasterizer.rs:66-68, 123-131), so pixel -12 is column 4 of tile -2
    # (x -16..-9) and pixel -5 column 3 of tile -1 (x -8..-1).  Four tiles in
    # (tile_y, tile_x) order, each a filled 4 x 4 quadrant; adjacent tiles on
    # a row leave no gap, so no span.
    from ochre_gb300.batch import CLOSE, LINE, MOVE, BatchBuilder
    b = BatchBuilder().fill([MOVE, LINE, LINE, LINE, CLOSE], [-12, -12, -4, -12, -4, -4, -12, -4], raw=True).build()
    r = oracle.run(b)
    assert r["tile_xy"].tolist() == [[-16, -16], [-8, -16], [-16, -8], [-8, -8]]
    quads = [(slice(4, 8), slice(4, 8)), (slice(4, 8), slice(0, 4)), (slice(0, 4), slice(4, 8)),
             (slice(0, 4), slice(0, 4))]
    for t, (rows, cols) in enumerate(quads):
        expect = np.zeros((8, 8), np.uint8)
        expect[rows, cols] = 255
        assert np.array_equal(r["tile_alpha"][t].reshape(8, 8), expect), t
    assert len(r["span_w"]) == 0


@pytest.mark.parametrize("gen,kw", [
    (W.readme_path, {}),
    (W.cubic_boxes, dict(n_paths=2)),
    (W.glyph_run, dict(n_paths=12)),
    (W.uneven_mix, dict(n_paths=3, max_seg=40)),
    (W.diff_scenes, dict(n_scenes=1, min_paths=3, max_paths=3, max_seg=12)),
])
def test_oracle_matches_python_restatement(gen, kw):
    b = gen(**kw)
    r = oracle.run(b)
    for i in range(b.n_rasters):
        tiles, spans, ninc = oracle_py.rasterize(oracle_py.commands_of_batch(b, i))
        xy, alpha, sxy, sw, st = _raster(r, i)
        assert [tuple(t) for t in xy.tolist()] == [t[:2] for t in tiles]
        assert np.array_equal(alpha, np.array([np.frombuffer(t[2], np.uint8) for t in tiles]).reshape(-1, 64))
        assert [(int(a), int(c), int(w), int(t)) for (a, c), w, t in zip(sxy.tolist(), sw, st)] == spans
        assert int(r["raster_stats"][i, 1]) == ninc


@pytest.mark.parametrize("which", ["edge_batch", "i16_batch"])
def test_edge_cases_match_python_restatement(which):
    import edge_cases
    b, names = getattr(edge_cases, which)()
    with np.errstate(all="ignore"):
        r = oracle.run(b)
    for i, name in enumerate(names):
        tiles, spans, _ = oracle_py.rasterize(oracle_py.commands_of_batch(b, i))
        xy, alpha, sxy, sw, st = _raster(r, i)
        assert [tuple(t) for t in xy.tolist()] == [t[:2] for t in tiles], name
        assert np.array_equal(alpha, np.array([np.frombuffer(t[2], np.uint8) for t in tiles]).reshape(-1, 64)), name
        assert [(int(a), int(c), int(w), int(t)) for (a, c), w, t in zip(sxy.tolist(), sw, st)] == spans, name


def test_oracle_threads_agree():
    b = W.glyph_run(n_paths=300)
    r1 = oracle.run(b, threads=1)
    r4 = oracle.run(b, threads=4)
    for k in ("tile_xy", "tile_alpha", "span_xy", "span_w", "span_tile", "raster_tile_off"):
        assert np.array_equal(r1[k], r4[k]), k


def test_oracle_line_capture_counts():
    b = W.cubic_boxes(n_paths=3)
    r = oracle.run(b, capture_lines=True)
    # every line ends where the next one starts within a raster
    for i in range(b.n_rasters):
        l0, l1 = int(r["raster_line_off"][i]), int(r["raster_line_off"][i + 1])
        L = r["lines"][l0:l1]
        assert np.array_equal(L[1:, :2], L[:-1, 2:])
    assert int(r["line_ninc"].sum()) == int(r["raster_stats"][:, 1].sum())


def test_stroke_matches_python_restatement():
    """The oracle's stroke preprocessing (path.rs:113-274) against the
    independent Python restatement, command by command and bit for bit."""
    import stroke_cases
    from ochre_gb300.batch import FLOATS_PER_VERB
    for name, fills in stroke_cases.CASES.items():
        for verbs, pts, _, _, width in fills:
            if width is None:
                continue
            v, p = oracle.stroke(verbs, pts, width)
            exp = oracle_py.stroke_polyline(oracle_py.path_polyline(np.array(verbs, np.uint8),
                                                                    np.array(pts, np.float32)), width)
            assert [int(x) for x in v] == [e[0] for e in exp], name
            got_pts = p.reshape(-1, 2)
            exp_pts = np.array([q for _, q in exp if q is not None], np.float32).reshape(-1, 2)
            assert np.array_equal(got_pts.view(np.uint32), exp_pts.view(np.uint32)), name


def test_stroke_known_answer_closed_rectangle():
    # forward side of a closed contour starts at its last point with a zero
    # previous normal (no miter at the first vertex), path.rs:170-212
    v, p = oracle.stroke([0, 1, 1, 1, 5], [10, 10, 50, 10, 50, 40, 10, 40], 4.0)
    assert v.tolist() == [0, 1, 1, 1, 1, 5, 0, 1, 1, 1, 1, 5]
    assert p.reshape(-1, 2).tolist()[:5] == [[12, 40], [12, 12], [48, 12], [48, 38], [10, 38]]


def test_stroke_rasters_match_python_restatement():
    import stroke_cases
    b, names = stroke_cases.stroke_batch()
    r = oracle.run(b)
    assert r["status"] == 0
    for i, name in enumerate(names):
        tiles, spans, _ = oracle_py.rasterize(oracle_py.commands_of_batch(b, i))
        xy, alpha, sxy, sw, st = _raster(r, i)
        assert [tuple(t) for t in xy.tolist()] == [t[:2] for t in tiles], name
        assert np.array_equal(alpha, np.array([np.frombuffer(t[2], np.uint8) for t in tiles]).reshape(-1, 64)), name
        assert [(int(a), int(c), int(w), int(t)) for (a, c), w, t in zip(sxy.tolist(), sw, st)] == spans, name


@pytest.mark.parametrize("seed,stroke_share,big_share",
                         [(11, 0.0, 0.1), (12, 0.0, 0.1), (13, 0.5, 0.1), (14, 0.0, 0.3), (15, 1.0, 0.15)])
def test_fuzz_oracle_matches_python_restatement(seed, stroke_share, big_share):
    """Random command sequences (every verb, any order, degenerate curves,
    repeated points, shears, raw commands, strokes, rasters eight times
    larger): both CPU restatements agree bit for bit, alpha included."""
    from fuzz_cases import fuzz_batch
    b = fuzz_batch(90, seed=seed, stroke_share=stroke_share, big_share=big_share)
    r = oracle.run(b)
    for i in range(b.n_rasters):
        tiles, spans, ninc = oracle_py.rasterize(oracle_py.commands_of_batch(b, i))
        xy, alpha, sxy, sw, st = _raster(r, i)
        assert [tuple(t) for t in xy.tolist()] == [t[:2] for t in tiles], i
        assert np.array_equal(alpha, np.array([np.frombuffer(t[2], np.uint8) for t in tiles]).reshape(-1, 64)), i
        assert [(int(a), int(c), int(w), int(t)) for (a, c), w, t in zip(sxy.tolist(), sw, st)] == spans, i


def test_oracle_struct_layouts_match_its_header(tmp_path):
    """The oracle wrapper's ctypes structures are oracle/ochre_oracle.h's."""
    import ctypes
    import os
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    pairs = [("ochre_oracle_batch", oracle._Batch), ("ochre_oracle_result", oracle._Result)]
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "ochre_oracle.h"', "int main(void) {"]
    for cname, cls in pairs:
        lines.append(f'    printf("{cname} %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            lines.append(f'    printf("{cname}.{fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", "-I", os.path.dirname(oracle.__file__), str(src), "-o", str(exe)], check=True)
    got = dict(line.rsplit(" ", 1) for line in subprocess.run([str(exe)], check=True, capture_output=True,
                                                              text=True).stdout.splitlines())
    for cname, cls in pairs:
        assert int(got[cname]) == ctypes.sizeof(cls), cname
        for fname, _ in cls._fields_:
            assert int(got[f"{cname}.{fname}"]) == getattr(cls, fname).offset, (cname, fname)


@pytest.mark.parametrize("name,expect", [
    ("readme_path", (70, 858, 50, 100, 23)),
    ("cubic_boxes", (1_104_367, 10_086_440, 561_524, 873_599, 170_315)),
    ("glyph_run", (7_825_524, 27_586_310, 1_235_618, 2_116_864, 253_952)),
    ("diff_union", (130_435, 290_234, 10_026, 8_635, 992)),
    ("stroke_run", (6_092_392, 76_028_159, 4_366_022, 5_825_432, 81_363)),
])
def test_configuration_counts(name, expect):
    """Exact lines, increments, crossings, tiles and spans of the seeded
    benchmark configurations (tests/golden/config_counts.py prints all of
    them): pins the workload generators and the oracle together."""
    import os
    from ochre_gb300 import workloads as W
    from golden.config_counts import counts
    c = counts(getattr(W, name)(), threads=os.cpu_count() or 1)
    assert (c["lines"], c["increments"], c["crossings"], c["tiles"], c["spans"]) == expect


def _side_step_local(pts, closed, reverse, width):
    """One offset side with every step's join computed on its own, the form
    the device walks 32 steps at a time: the point before step i is the
    side's point i - 1 (its first point at i = 0), and the normal before it
    is that of the nearest earlier step with a join."""
    F, ZERO, ONE = np.float32, np.float32(0.0), np.float32(1.0)
    half = F(0.5) * F(width)
    seq = pts[::-1] if reverse else pts
    first = pts[0] if closed == reverse else pts[-1]
    n = len(seq)
    normals = []   # per step: its normal when it has a join, else None
    for i in range(n + 1):
        nxt = seq[i] if i < n else first
        prv = seq[i - 1] if i > 0 else first
        if i < n and nxt[0] == prv[0] and nxt[1] == prv[1]:
            normals.append(None)
            continue
        tx, ty = nxt[0] - prv[0], nxt[1] - prv[1]
        nn = (-ty, tx)
        ln = np.sqrt(nn[0] * nn[0] + nn[1] * nn[1])
        normals.append((ZERO, ZERO) if ln == ZERO else (nn[0] * (ONE / ln), nn[1] * (ONE / ln)))
    res = []
    for i in range(n + 1):
        nn = normals[i]
        if nn is None:
            continue
        prv = seq[i - 1] if i > 0 else first
        earlier = [m for m in normals[:i] if m is not None]
        pn = earlier[-1] if earlier else (ZERO, ZERO)
        off = ONE / (ONE + (pn[0] * nn[0] + pn[1] * nn[1]))
        if abs(off) > F(2.0):
            res.append((prv[0] + half * pn[0], prv[1] + half * pn[1]))
            res.append((prv[0] + half * nn[0], prv[1] + half * nn[1]))
        else:
            k = half * off
            res.append((prv[0] + k * (pn[0] + nn[0]), prv[1] + k * (pn[1] + nn[1])))
    return res


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_stroke_joins_are_step_local(seed):
    """The reference's offset loop (path.rs:160-212) carries the previous
    distinct point and the previous join's normal; restated with every join
    computed from the point before its step and the nearest earlier join's
    normal (the device's 32-steps-per-round walk), it gives the same points
    bit for bit, on random contours with repeated points, open and closed."""
    rng = np.random.default_rng(seed)
    F = np.float32
    for _ in range(60):
        n = int(rng.integers(1, 40))
        raw = rng.normal(0, 30, size=(n, 2)).astype(F)
        pts = []
        for p in raw:
            pts.append((F(p[0]), F(p[1])))
            if rng.uniform() < 0.3:          # a repeated point
                pts.append(pts[-1])
            if rng.uniform() < 0.05 and len(pts) > 2:   # back to an earlier point
                pts.append(pts[int(rng.integers(0, len(pts) - 1))])
        closed = bool(rng.uniform() < 0.5)
        width = F(rng.uniform(0.25, 12.0))
        poly = [(0, pts[0])] + [(1, p) for p in pts[1:]] + ([(5, None)] if closed else [])
        want = oracle_py.stroke_polyline(poly, width)
        fwd = _side_step_local(pts, closed, False, width)
        bwd = _side_step_local(pts, closed, True, width)
        got = [(0 if j == 0 else 1, q) for j, q in enumerate(fwd)] + ([(5, None)] if closed else [])
        got += [(0 if (j == 0 and closed) else 1, q) for j, q in enumerate(bwd)] + [(5, None)]
        assert [v for v, _ in got] == [v for v, _ in want]
        for (_, a), (_, b) in zip(got, want):
            if a is not None:
                assert a[0] == b[0] and a[1] == b[1]
