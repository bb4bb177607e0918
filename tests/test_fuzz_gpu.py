"""Seeded random rasters (tests/fuzz_cases.py) on every execution form and
through a CUDA-graph replay, against the oracle."""
import numpy as np
import pytest

import oracle
from compare import compare
from fuzz_cases import fuzz_batch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed,big_share", [(1, 0.0), (2, 0.0), (3, 0.1), (4, 0.3)])
def test_fuzz_matches_oracle(any_ctx, seed, big_share):
    b = fuzz_batch(1500, seed=seed, big_share=big_share)
    ref = oracle.run(b, threads=16)
    got = any_ctx.rasterize(b)
    st = compare(got, ref, b.n_rasters)
    assert st["diff_fraction"] < 0.01, st


def test_fuzz_fused_form_is_used(gpu_ctx):
    """Without large rasters the fuzz batches run on the fused kernel (so the
    test above covers it)."""
    for seed in (1, 2):
        gpu_ctx.rasterize(fuzz_batch(1500, seed=seed, big_share=0.0))
        assert gpu_ctx.stats()["fused"] == 1, seed


@pytest.mark.parametrize("seed", [21, 22])
def test_fuzz_strokes_match_oracle(any_ctx, seed):
    b = fuzz_batch(1200, seed=seed, big_share=0.05, stroke_share=0.5)
    assert b.has_strokes
    st = compare(any_ctx.rasterize(b), oracle.run(b, threads=16), b.n_rasters)
    assert st["diff_fraction"] < 0.01, st


@pytest.mark.parametrize("big_share", [0.0, 0.2])
def test_fuzz_graph_replay(gpu_ctx, big_share):
    from ochre_gb300 import DeviceBatch
    b = fuzz_batch(600, seed=7, big_share=big_share)
    g = gpu_ctx.graph(DeviceBatch(b))
    try:
        compare(g.rasterize(), oracle.run(b, threads=16), b.n_rasters)
    finally:
        g.close()
