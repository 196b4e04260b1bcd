"""Autotuner (bpgb_plan_autotune / bpgb_batch_autotune): the choice runs, is never slower
than the untuned default by more than timing noise, validates its bin windows, and is
served from the cache (file round trip included) without timing anything."""
from __future__ import annotations

import numpy as np
import pytest

from backprojector_gb300 import capi, synthetic
from oracle import oracle

pytestmark = pytest.mark.gpu


def test_plan_autotune_choice_runs_and_is_cached(cuda, tmp_path):
    import torch

    capi.tune_cache_clear()
    c = synthetic.make_capture("octree_256", seed=5, small=True)
    dH = torch.from_numpy(c.H).to(cuda)
    dV = torch.empty(tuple(int(v) for v in c.voxels_per_side), device=cuda)
    tuned, rep = capi.autotune_plan(c.pairs, c.T, c.voxels_per_side, c.zero, c.inc, c.t0,
                                    c.deltaT, dH, dV)
    assert rep["cache_hit"] == 0 and rep["candidates"] > 10
    assert capi.tune_cache_size() == 1
    assert rep["best_ms"] > 0 and rep["default_ms"] > 0
    assert rep["best_ms"] <= rep["default_ms"] * 1.05
    ref = oracle.bp_gpu_f64(c.H, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT)
    with capi.Plan(c.pairs, c.T, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT, checked=1,
                   **tuned) as p:
        p.execute(dH, dV)
        assert p.check() == 0
        info = p.info()
    assert info["algo"] == "fast"
    assert oracle.rel_l2(dV.cpu().numpy(), ref) < 5e-3
    # a second call is a cache hit, also after a save / clear / load round trip
    tuned2, rep2 = capi.autotune_plan(c.pairs, c.T, c.voxels_per_side, c.zero, c.inc, c.t0,
                                      c.deltaT, dH, dV)
    assert rep2["cache_hit"] == 1 and rep2["candidates"] == 0 and tuned2 == tuned
    path = tmp_path / "tune.txt"
    capi.tune_cache_save(path)
    capi.tune_cache_clear()
    capi.tune_cache_load(path)
    tuned3, rep3 = capi.autotune_plan(c.pairs, c.T, c.voxels_per_side, c.zero, c.inc, c.t0,
                                      c.deltaT, dH, dV)
    assert rep3["cache_hit"] == 1 and tuned3 == tuned
    capi.tune_cache_clear()


def test_batch_autotune_choice_runs(cuda):
    import torch

    capi.tune_cache_clear()
    caps = synthetic.make_batch(8, seed=11, grids=(8, 16), Ts=(512, 1024), voxels=(16, 32),
                                exhaustive_grid=4)
    scales = synthetic.fp16_scales(caps)
    geo = synthetic.batch_geometry(caps, scales)
    with capi.Batch(geo, h_dtype=capi.DTYPE_F16) as b0:
        info = b0.info()
        H = synthetic.pack_batch(caps, b0.row_offsets, info["pitch"], np.float16, scales)
    dH = torch.from_numpy(H).to(cuda)
    dV = torch.empty(info["total_voxels"], device=cuda)
    tuned, rep = capi.autotune_batch(geo, dH, dV, h_dtype=capi.DTYPE_F16)
    assert rep["cache_hit"] == 0 and rep["candidates"] > 7
    assert rep["best_ms"] <= rep["default_ms"] * 1.05
    with capi.Batch(geo, h_dtype=capi.DTYPE_F16, checked=1, **tuned) as b:
        assert b.row_offsets == b0.row_offsets and b.info()["pitch"] == info["pitch"]
        b.execute(dH, dV)
        assert b.check() == 0
        flat = dV.cpu().numpy()
    for i, c in enumerate(caps):
        o = b.voxel_offsets[i]
        vol = flat[o:o + c.nvox].reshape(tuple(int(v) for v in c.voxels_per_side))
        r = b.row_offsets[i]
        Hc = H[r:r + c.P, :c.T].astype(np.float32) * scales[i]
        ref = oracle.bp_gpu_f64(Hc, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT)
        assert oracle.rel_l2(vol, ref) < (5e-3 if c.P >= 256 else 2e-2), i
    _, rep2 = capi.autotune_batch(geo, dH, dV, h_dtype=capi.DTYPE_F16)
    assert rep2["cache_hit"] == 1
    capi.tune_cache_clear()
