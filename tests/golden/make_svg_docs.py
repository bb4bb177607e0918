"""Regenerates tests/golden/svg_docs.npz from the reference's example
documents (examples/res/*.svg of glowcoil/ochre: the Ghostscript tiger, a
Calabi-Yau drawing and a page of lorem-ipsum glyphs).

Each document is read with this project's own SVG reader
(ochre_gb300/svg.py) into the batch the example renders (one rasterizer per
painted fill or stroke, examples/svg.rs:139-156): verbs, points, per-fill
transforms, flags and stroke widths, the RGBA8 colour of every raster and
the document's canvas size.  The fixture holds only those parsed arrays, so
the tests run without the reference tree (which the GPU machines do not
have); the expected outputs are computed by the oracle at test time.

Usage:  python tests/golden/make_svg_docs.py [reference examples/res directory]
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from ochre_gb300 import svg  # noqa: E402
from ochre_gb300.batch import Batch  # noqa: E402

DOCS = {"tiger": "Ghostscript_Tiger.svg", "calabi_yau": "calabi-yau.svg", "lorem_ipsum": "lorem-ipsum.svg"}
FIXTURE = os.path.join(HERE, "svg_docs.npz")


def build(src_dir: str) -> None:
    arrays = {}
    for key, fname in DOCS.items():
        with open(os.path.join(src_dir, fname)) as f:
            text = f.read()
        paints, (w, h) = svg.load_svg(text)
        b, colors = svg.paints_to_batch(paints)
        fw = getattr(b, "fill_width", None)
        arrays.update({
            f"{key}/verbs": b.verbs, f"{key}/pts": b.pts, f"{key}/fill_cmd_off": b.fill_cmd_off,
            f"{key}/fill_xf": b.fill_xf,
            f"{key}/fill_flags": b.fill_flags if b.fill_flags is not None else np.zeros(0, np.uint8),
            f"{key}/fill_width": fw if fw is not None else np.zeros(0, np.float32),
            f"{key}/raster_fill_off": (b.raster_fill_off if b.raster_fill_off is not None
                                       else np.zeros(0, np.uint32)),
            f"{key}/n_rasters": np.array(b.n_rasters), f"{key}/colors": colors,
            f"{key}/size": np.array([w, h], np.float64), f"{key}/n_path_elements": np.array(text.count("<path")),
        })
        print(f"{fname}: {b.n_rasters} rasters, {b.n_cmds} commands, canvas {w} x {h}")
    np.savez_compressed(FIXTURE, **arrays)


def load(key: str):
    """(Batch, colours [n, 4] u8, (width, height), <path> element count) of one document."""
    z = np.load(FIXTURE)
    g = lambda k: z[f"{key}/{k}"]
    fl, fw, ro = g("fill_flags"), g("fill_width"), g("raster_fill_off")
    b = Batch(g("verbs"), g("pts"), g("fill_cmd_off"), g("fill_xf"), fl if len(fl) else None,
              ro if len(ro) else None, int(g("n_rasters")))
    if len(fw):
        b.fill_width = fw
    w, h = (float(v) for v in g("size"))
    return b, g("colors"), (w, h), int(g("n_path_elements"))


if __name__ == "__main__":
    build(sys.argv[1] if len(sys.argv) > 1 else "/root/reference/examples/res")
