"""Comparison of a GPU result with the oracle's (test infrastructure).

The bar: tile positions, tile counts per raster, span positions/widths and
the tile each span follows are bit-exact; every alpha byte is within 1 LSB
(the reference's unstable sorts leave the f32 summation order inside a tile
unspecified, so 1 LSB is the tightest meaningful bound).
"""
from __future__ import annotations

import numpy as np

ALPHA_TOL_LSB = 1


def compare(gpu: dict, ref: dict, n_rasters: int) -> dict:
    """Raises AssertionError on any structural mismatch or alpha > 1 LSB;
    returns diff statistics."""
    for k in ("raster_tile_off", "raster_span_off"):
        g = np.asarray(gpu[k], dtype=np.int64)
        r = np.asarray(ref[k], dtype=np.int64)
        assert g.shape == r.shape == (n_rasters + 1,), (k, g.shape, r.shape)
        if not np.array_equal(g, r):
            bad = int(np.flatnonzero(g != r)[0])
            raise AssertionError(f"{k} differs first at raster {bad}: gpu {g[bad]} oracle {r[bad]}")
    assert gpu["tile_xy"].shape == ref["tile_xy"].shape, (gpu["tile_xy"].shape, ref["tile_xy"].shape)
    if not np.array_equal(gpu["tile_xy"], ref["tile_xy"]):
        bad = int(np.flatnonzero(np.any(gpu["tile_xy"] != ref["tile_xy"], axis=1))[0])
        raise AssertionError(f"tile position differs at tile {bad}: gpu {gpu['tile_xy'][bad]} oracle {ref['tile_xy'][bad]}")
    for k in ("span_xy", "span_w", "span_tile"):
        g, r = np.asarray(gpu[k]), np.asarray(ref[k])
        assert g.shape == r.shape, (k, g.shape, r.shape)
        if not np.array_equal(g.astype(np.int64), r.astype(np.int64)):
            bad = int(np.flatnonzero((g != r).reshape(len(g), -1).any(axis=1))[0])
            raise AssertionError(f"{k} differs at span {bad}: gpu {g[bad]} oracle {r[bad]}")
    ga_all, ra_all = gpu["tile_alpha"], ref["tile_alpha"]
    assert ga_all.shape == ra_all.shape, (ga_all.shape, ra_all.shape)
    # in slices of tiles, so that full-size results (tens of millions of
    # tiles) need no second full-size copy
    max_lsb, n_diff = 0, 0
    CH = 1 << 22
    for a in range(0, len(ra_all), CH):
        ga = ga_all[a:a + CH].astype(np.int16)
        ra = ra_all[a:a + CH].astype(np.int16)
        d = np.abs(ga - ra)
        m = int(d.max()) if d.size else 0
        if m > ALPHA_TOL_LSB:
            t, c = np.unravel_index(int(np.argmax(d)), d.shape)
            raise AssertionError(f"alpha differs by {m} LSB at tile {a + t} cell {c} "
                                 f"(gpu {ga[t, c]} oracle {ra[t, c]}, tile at {ref['tile_xy'][a + t]})")
        max_lsb = max(max_lsb, m)
        n_diff += int(np.count_nonzero(d))
    stats = {
        "tiles": int(len(ra_all)),
        "spans": int(len(ref["span_w"])),
        "max_lsb": max_lsb,
        "diff_fraction": n_diff / ra_all.size if ra_all.size else 0.0,
    }
    if "tile_cov" in gpu and "tile_cov" in ref:
        r = ref["tile_cov"].astype(np.float64)
        e = np.abs(gpu["tile_cov"].astype(np.float64) - r)
        stats["cov_max_abs_vs_oracle_f32"] = float(e.max()) if e.size else 0.0
        # relative to |S| where it exceeds 1 (the f32 sums' rounding scales with them)
        stats["cov_max_rel_vs_oracle_f32"] = float((e / np.maximum(1.0, np.abs(r))).max()) if e.size else 0.0
    return stats
