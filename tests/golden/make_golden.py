"""Regenerates the golden fixtures in tests/golden/*.npz.

The Rust reference cannot run on these machines and ships no recorded
outputs, so the fixtures hold the oracle's output (oracle/ochre_oracle.c,
cross-checked against tests/oracle_py.py and hand-derived answers in
tests/test_oracle.py) together with the exact inputs, so that the GPU path,
the oracle and any later build are compared on identical bytes.

Usage:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

import oracle  # noqa: E402
from ochre_gb300 import workloads as W  # noqa: E402
from ochre_gb300.batch import Batch  # noqa: E402


def cases():
    import edge_cases
    eb, _ = edge_cases.edge_batch()
    ib, _ = edge_cases.i16_batch()
    return {
        "readme": W.readme_path(),
        "edge_cases": eb,
        "i16_limits": ib,
        "cubic_boxes_2": W.cubic_boxes(n_paths=2),
        "glyph_run_48": W.glyph_run(n_paths=48),
        "uneven_mix_4": W.uneven_mix(n_paths=4, max_seg=120),
        "diff_union_6": W.diff_union(n_paths=6),
        "diff_scenes_1": W.diff_scenes(n_scenes=1, min_paths=6, max_paths=6, max_seg=24),
    }


def save(name: str, b: Batch) -> None:
    with np.errstate(all="ignore"):
        r = oracle.run(b, want_cov=True)
    assert r["status"] == 0, (name, r["status"])
    arrays = {
        "verbs": b.verbs, "pts": b.pts, "fill_cmd_off": b.fill_cmd_off, "fill_xf": b.fill_xf,
        "fill_flags": b.fill_flags if b.fill_flags is not None else np.zeros(0, np.uint8),
        "has_fill_flags": np.array(b.fill_flags is not None),
        "raster_fill_off": b.raster_fill_off if b.raster_fill_off is not None else np.zeros(0, np.uint32),
        "has_raster_fill_off": np.array(b.raster_fill_off is not None),
        "n_rasters": np.array(b.n_rasters),
    }
    for k in ("tile_xy", "tile_alpha", "tile_cov", "span_xy", "span_w", "span_tile", "raster_tile_off",
              "raster_span_off", "raster_stats"):
        arrays["out_" + k] = r[k]
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
    print(f"{name}: {b.n_rasters} rasters, {len(r['tile_xy'])} tiles, {len(r['span_w'])} spans")


def load(name: str):
    """(Batch, expected-output dict) of a fixture."""
    z = np.load(os.path.join(HERE, name + ".npz"))
    b = Batch(z["verbs"], z["pts"], z["fill_cmd_off"], z["fill_xf"],
              z["fill_flags"] if bool(z["has_fill_flags"]) else None,
              z["raster_fill_off"] if bool(z["has_raster_fill_off"]) else None, int(z["n_rasters"]))
    out = {k[4:]: z[k] for k in z.files if k.startswith("out_")}
    return b, out


NAMES = ["readme", "edge_cases", "i16_limits", "cubic_boxes_2", "glyph_run_48", "uneven_mix_4", "diff_union_6", "diff_scenes_1"]

if __name__ == "__main__":
    for name, b in cases().items():
        save(name, b)
