"""Exact intermediate counts of every seeded benchmark configuration, from the
oracle (test infrastructure): paths, flattened lines L, pixel-cell
increments I, tile-row crossings, tiles T and spans N.  Prints a markdown
table.  Usage: python tests/golden/config_counts.py [--scenes N] [--threads K]
(the dense-scenes configuration is the heaviest; --scenes limits it)."""
from __future__ import annotations

import argparse
import os
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from ochre_gb300 import workloads as W  # noqa: E402


def counts(batch, threads: int) -> dict:
    r = oracle.run(batch, threads=threads)
    if r["status"] != 0:
        raise RuntimeError(f"oracle status {r['status']}")
    st = r["raster_stats"]
    return {"rasters": batch.n_rasters, "fills": batch.n_fills, "commands": batch.n_cmds,
            "lines": int(st[:, 0].sum()), "increments": int(st[:, 1].sum()), "crossings": int(st[:, 2].sum()),
            "tiles": int(r["tile_xy"].shape[0]), "spans": int(r["span_w"].shape[0])}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--scenes", type=int, default=4096)
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    a = ap.parse_args()
    configs = [
        ("README path (smoke)", W.readme_path),
        ("cubic boxes: 1,000 paths x 16 cubics", W.cubic_boxes),
        ("glyph run: 100,000 paths", W.glyph_run),
        ("uneven mix: 20,000 paths", W.uneven_mix),
        ("differentiable union: 256 x 32 cubics, one raster", W.diff_union),
        (f"dense scenes: {a.scenes:,} scenes of 512^2", lambda: W.diff_scenes(n_scenes=a.scenes)),
        ("stroke run: 20,000 stroked paths", W.stroke_run),
    ]
    print("| configuration | rasters | fills | commands | lines L | increments I | crossings | tiles T | spans N | oracle s |")
    print("|---|---|---|---|---|---|---|---|---|---|")
    for name, make in configs:
        b = make()
        t0 = time.time()
        c = counts(b, a.threads)
        print(f"| {name} | {c['rasters']:,} | {c['fills']:,} | {c['commands']:,} | {c['lines']:,} | "
              f"{c['increments']:,} | {c['crossings']:,} | {c['tiles']:,} | {c['spans']:,} | {time.time() - t0:.1f} |",
              flush=True)


if __name__ == "__main__":
    main()
