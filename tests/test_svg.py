"""SVG input (path data parser, document reader) and end-to-end rendering
(rasterize + composite) against the oracle."""
import math

import numpy as np
import pytest

from ochre_gb300 import svg

SCENE = """<svg xmlns="http://www.w3.org/2000/svg" width="320" height="240">
  <rect x="0" y="0" width="320" height="240" fill="#f0f0e8"/>
  <g transform="translate(20,10) scale(1.5)">
    <path d="M10 20 C40 -10 90 60 120 20 S170 -20 190 40 L150 90 Q120 120 90 90 T40 90 Z"
          fill="rgb(200, 60, 40)" fill-opacity="0.8" stroke="#123" stroke-width="2.5"/>
    <circle cx="60" cy="120" r="25" fill="navy" opacity="0.6"/>
    <ellipse cx="140" cy="120" rx="30" ry="12" transform="rotate(30 140 120)" fill="#3a6" stroke="black"/>
  </g>
  <polyline points="10,230 60,180 110,220 160,170 210,230" fill="none" stroke="orange" stroke-width="6"/>
  <polygon points="250,20 300,60 280,120 230,100" style="fill: teal; stroke: #fff; stroke-width: 3"/>
  <line x1="230" y1="200" x2="310" y2="150" stroke="purple" stroke-width="4" stroke-opacity="0.5"/>
  <path d="M240 140 a20 10 30 1 0 40 0 a20 10 30 1 0 -40 0 z" fill="#c0c" fill-opacity="0.5"/>
</svg>"""


def _flat(cmds):
    return [(c.verb, [round(x, 6) for x in c.floats]) for c in cmds]


def test_path_data_commands():
    p = svg.parse_path("M10 20 l5-5h10v10 C 1 2 3 4 5 6 s 1 1 2 2 q1 0 2 2 t 3 3 a5 5 0 0110 10 z m1 1 2 2")
    got = _flat(p)
    assert got[:8] == [(0, [10, 20]), (1, [15, 15]), (1, [25, 15]), (1, [25, 25]), (3, [1, 2, 3, 4, 5, 6]),
                       (3, [7, 8, 6, 7, 7, 8]), (2, [8, 8, 9, 10]), (2, [10, 12, 12, 13])]
    # arc from (12,13) to (22,23): radius scaled up to a semicircle, two 90-degree conics
    assert got[8] == (4, [17, 8, 22, 13, round(math.cos(math.pi / 4), 6)])
    assert got[9][0] == 4 and got[9][1][2:4] == [22, 23]
    assert got[10] == (5, [])
    assert got[11:] == [(0, [11, 21]), (1, [13, 23])]


def test_drawing_after_closepath_starts_at_the_subpath_start():
    """After z the next drawing command starts a new subpath at the initial
    point (SVG 1.1 8.3.3): an explicit Move, since ochre's Close is a no-op."""
    assert _flat(svg.parse_path("M0 0 L10 0 L10 10 z L5 5")) == [
        (0, [0, 0]), (1, [10, 0]), (1, [10, 10]), (5, []), (0, [0, 0]), (1, [5, 5])]
    assert _flat(svg.parse_path("M0 0 L10 0 z l5 5 z m1 1"))[3:] == [
        (0, [0, 0]), (1, [5, 5]), (5, []), (0, [1, 1])]
    assert _flat(svg.parse_path("M0 0 L10 0 z M3 3 L4 4"))[3:] == [(0, [3, 3]), (1, [4, 4])]


def test_number_forms():
    p = svg.parse_path("M.5-1.5e1L1e-1.2 2,3-4.5.5")
    assert _flat(p) == [(0, [0.5, -15.0]), (1, [0.1, 0.2]), (1, [2, 3]), (1, [-4.5, 0.5])]
    with pytest.raises(ValueError):
        svg.parse_path("L1 2")
    with pytest.raises(ValueError):
        svg.parse_path("M1 2 L3")


@pytest.mark.parametrize("rx,ry,phi,large,sweep", [(30, 12, 25, 0, 1), (30, 12, 25, 1, 0), (5, 9, 110, 1, 1)])
def test_arc_conics_lie_on_the_ellipse(rx, ry, phi, large, sweep):
    x0, y0, x1, y1 = 10.0, 5.0, 40.0, 25.0
    cmds = svg._arc_to_conics(x0, y0, rx, ry, phi, bool(large), bool(sweep), x1, y1)
    assert 1 <= len(cmds) <= 4
    pts, last = [(x0, y0)], (x0, y0)
    for c in cmds:
        cx_, cy_, px, py, w = c.floats
        for t in (0.25, 0.5, 0.75, 1.0):
            b0, b1, b2 = (1 - t) ** 2, 2 * t * (1 - t) * w, t * t
            den = b0 + b1 + b2
            pts.append(((b0 * last[0] + b1 * cx_ + b2 * px) / den, (b0 * last[1] + b1 * cy_ + b2 * py) / den))
        last = (px, py)
    assert abs(last[0] - x1) < 1e-9 and abs(last[1] - y1) < 1e-9
    # all points on one ellipse with the arc's axis ratio and rotation (radii may be scaled up
    # uniformly when they are too small): in the ellipse frame, u^2/rx^2 + v^2/ry^2 - 2 u cu/rx^2
    # - 2 v cv/ry^2 + k = 0 is linear in (cu, cv, k)
    a = math.radians(phi)
    P = np.array(pts)
    u = math.cos(a) * P[:, 0] + math.sin(a) * P[:, 1]
    v = -math.sin(a) * P[:, 0] + math.cos(a) * P[:, 1]
    A = np.c_[-2 * u / rx ** 2, -2 * v / ry ** 2, np.ones(len(u))]
    rhs = -(u ** 2 / rx ** 2 + v ** 2 / ry ** 2)
    sol, *_ = np.linalg.lstsq(A, rhs, rcond=None)
    assert np.abs(A @ sol - rhs).max() < 1e-9 * np.abs(rhs).max()
    # the sweep direction: the signed area of the polygon of samples
    area = 0.5 * np.sum(P[:-1, 0] * P[1:, 1] - P[1:, 0] * P[:-1, 1])
    assert (area > 0) == bool(sweep)


def test_document_paints():
    paints, size = svg.load_svg(SCENE)
    assert size == (320.0, 240.0)
    kinds = [(p.rgba, p.stroke_width) for p in paints]
    assert kinds[0] == ((240, 240, 232, 255), None)
    assert kinds[1] == ((200, 60, 40, 204), None) and kinds[2] == ((17, 34, 51, 255), 2.5)
    assert kinds[3] == ((0, 0, 128, 153), None)
    assert paints[1].transform[0, 0] == 1.5 and paints[1].transform[0, 2] == 20.0
    assert kinds[-1][0] == (204, 0, 204, 128)
    polyline = [k for k in kinds if k[0][:3] == (255, 165, 0)]
    assert polyline == [((255, 165, 0, 255), 6.0)]


@pytest.mark.gpu
def test_render_svg_matches_oracle():
    import oracle
    paints, (w, h) = svg.load_svg(SCENE)
    batch, colors = svg.paints_to_batch(paints)
    img = svg.render_svg(SCENE)
    ref = oracle.composite(oracle.run(batch), batch.n_rasters, colors, int(w), int(h))
    assert img.shape == (240, 320, 4)
    # the GPU's alpha may differ from the oracle's by 1 LSB (summation order),
    # which can move a blended channel by a step
    diff = np.abs(img.astype(np.int16) - ref.astype(np.int16))
    assert diff.max() <= 2 and (diff > 0).mean() < 0.01, (int(diff.max()), float((diff > 0).mean()))
    # the scene actually drew something in each part of the canvas
    assert (img[:, :, :3] != 255).any(axis=2).mean() > 0.5


# The reference's own example documents (examples/res/*.svg): the parsed
# batches (this project's SVG reader, tests/golden/make_svg_docs.py) are the
# fixture tests/golden/svg_docs.npz, so these tests need no reference tree.
REF_DOCS = ["tiger", "calabi_yau", "lorem_ipsum"]


@pytest.mark.parametrize("name", REF_DOCS)
def test_reference_example_documents(name):
    import oracle
    import oracle_py
    from golden.make_svg_docs import load
    batch, colors, _, n_path_elements = load(name)
    # every <path> element became at least one paint (fill and/or stroke)
    assert batch.n_rasters >= n_path_elements and len(colors) == batch.n_rasters
    batch.validate()
    r = oracle.run(batch, threads=8)
    assert r["status"] == 0 and len(r["tile_xy"]) > 0
    # the independent numpy restatement agrees bit for bit on a sample
    step = max(1, batch.n_rasters // 24)
    for i in range(0, batch.n_rasters, step):
        tiles, spans, _ = oracle_py.rasterize(oracle_py.commands_of_batch(batch, i))
        a, b = int(r["raster_tile_off"][i]), int(r["raster_tile_off"][i + 1])
        assert [tuple(t) for t in r["tile_xy"][a:b].tolist()] == [t[:2] for t in tiles], (name, i)
        alpha = np.array([np.frombuffer(t[2], np.uint8) for t in tiles]).reshape(-1, 64)
        assert np.array_equal(r["tile_alpha"][a:b], alpha), (name, i)
        c, d = int(r["raster_span_off"][i]), int(r["raster_span_off"][i + 1])
        assert d - c == len(spans), (name, i)


@pytest.mark.gpu
@pytest.mark.parametrize("name", REF_DOCS)
def test_reference_example_documents_gpu(name):
    """GPU rasterization and compositing of the reference's example documents
    against the oracle: tiles and spans exact, composited image within two
    steps per channel on under 1 % of the pixels."""
    import torch

    import oracle
    from compare import compare
    from golden.make_svg_docs import load
    from ochre_gb300 import DeviceBatch, default_context
    batch, colors, (w, h), _ = load(name)
    ref = oracle.run(batch, threads=8)
    ctx = default_context()
    r = ctx.rasterize_device(DeviceBatch(batch))
    got = ctx.device_result_to_numpy(r, batch.n_rasters)
    compare(got, ref, batch.n_rasters)
    W, H = int(w or 1024), int(h or 1024)
    canvas = torch.full((H, W, 4), 255, dtype=torch.uint8, device="cuda:0")
    ctx.composite(r, batch.n_rasters, torch.as_tensor(colors, device=canvas.device), canvas)
    torch.cuda.synchronize()
    img = canvas.cpu().numpy()
    want = oracle.composite(ref, batch.n_rasters, colors, W, H)
    # alpha may differ by 1 LSB (summation order), which can move a blended
    # channel by a step per layer drawn over it
    diff = np.abs(img.astype(np.int16) - want.astype(np.int16))
    assert diff.max() <= 2 and (diff > 0).mean() < 0.01, (int(diff.max()), float((diff > 0).mean()))
    assert (img[:, :, :3] != 255).any(axis=2).mean() > 0.01   # the document drew something
