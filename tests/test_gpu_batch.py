"""Batched persistent launch (bpgb_batch_*): many uneven captures in one kernel launch,
checked per capture against single-capture plans and the FP64 oracle.

Tolerances: against a plan on the same stored rows the batch has the same bins and
summation order (rel-L2 <= 1e-6).  FP16 rows dequantised with the per-capture scale feed
the FP64 oracle, so the batch differs from it by FAST binning only: rel-L2 <= 1e-3 on
captures of >= 1024 pairs (as for plans) and <= 2e-2 on the 16-256-pair captures of these
small batches, where one bin placed one bin over moves a voxel by about 1/P of its sum.
"""
from __future__ import annotations

import numpy as np
import pytest

from backprojector_gb300 import capi, synthetic
from oracle import oracle

pytestmark = pytest.mark.gpu


def small_batch(n=10, seed=3, exhaustive_frac=0.3):
    return synthetic.make_batch(n, seed=seed, grids=(4, 6, 8), Ts=(512, 1024),
                                voxels=(12, 16, 20), exhaustive_frac=exhaustive_frac,
                                exhaustive_grid=4)


def tol(c):
    # rel-L2 against the FP64 oracle is set by a handful of .5-boundary bins on small
    # captures: one flipped bin moves a voxel by ~1/P of its sum.  Measured on the 256-pair
    # lasers x SPADs captures: mis-binned fraction 2-4e-5 for both the factored and the
    # per-pair form, rel-L2 up to 1.06e-2.
    return 1e-3 if c.P >= 1024 else 2e-2


def upload(cuda, caps, batch, dtype, scales):
    import torch

    info = batch.info()
    H = synthetic.pack_batch(caps, batch.row_offsets, info["pitch"], dtype, scales)
    dH = torch.from_numpy(H).to(cuda)
    dV = torch.full((info["total_voxels"],), float("nan"), dtype=torch.float32, device=cuda)
    return H, dH, dV


def volumes(caps, batch, flat):
    out = []
    for i, c in enumerate(caps):
        o = batch.voxel_offsets[i]
        out.append(flat[o:o + c.nvox].reshape(tuple(int(v) for v in c.voxels_per_side)))
    return out


def dequantised(c, H, batch, i, scale):
    r = batch.row_offsets[i]
    return H[r:r + c.P, :c.T].astype(np.float32) * np.float32(scale)


@pytest.mark.parametrize("dtype", ["f16", "f32"])
def test_batch_matches_plans_and_oracle(cuda, dtype):
    caps = small_batch()
    np_dtype = np.float16 if dtype == "f16" else np.float32
    h_dtype = capi.DTYPE_F16 if dtype == "f16" else capi.DTYPE_F32
    scales = synthetic.fp16_scales(caps) if dtype == "f16" else np.ones(len(caps), np.float32)
    geo = synthetic.batch_geometry(caps, scales)
    with capi.Batch(geo, h_dtype=h_dtype, checked=1) as b:
        info = b.info()
        assert info["captures"] == len(caps) and info["planar"] == 1
        assert info["updates"] == sum(c.updates for c in caps)
        H, dH, dV = upload(cuda, caps, b, np_dtype, scales)
        b.execute(dH, dV)
        assert b.check() == 0
        vols = volumes(caps, b, dV.cpu().numpy())
    import torch

    for i, c in enumerate(caps):
        assert np.all(np.isfinite(vols[i]))
        # the same capture alone through a plan, on the same stored rows (lasers x SPADs
        # captures take the factored form in both)
        r = b.row_offsets[i]
        dHc = torch.from_numpy(np.ascontiguousarray(H[r:r + c.P, :c.T])).to(cuda)
        dVc = torch.empty(tuple(int(v) for v in c.voxels_per_side), dtype=torch.float32,
                          device=cuda)
        with capi.Plan(c.pairs, c.T, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT,
                       algo=capi.ALGO_FAST, h_dtype=h_dtype, h_scale=float(scales[i])) as p:
            p.execute(dHc, dVc)
            p.check()
            single = dVc.cpu().numpy()
        assert oracle.rel_l2(vols[i], single) < 1e-6, i
        Hc = dequantised(c, H, b, i, scales[i])
        ref = oracle.bp_gpu_f64(Hc, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT)
        assert oracle.rel_l2(vols[i], ref) < tol(c), i


@pytest.mark.parametrize("frac", [0.0, 1.0])
def test_batch_of_one_kind(cuda, frac):
    """Only single-laser captures (one persistent launch, per-pair legs) or only lasers x
    SPADs captures (one persistent launch, factored legs); the unfactored option runs every
    capture per pair."""
    import torch

    caps = small_batch(n=5, seed=6, exhaustive_frac=frac)
    geo = synthetic.batch_geometry(caps)
    outs = []
    for unf in (0, 1):
        with capi.Batch(geo, h_dtype=capi.DTYPE_F32, checked=1, unfactored=unf) as b:
            H, dH, dV = upload(cuda, caps, b, np.float32, None)
            launches = capi.launch_count()
            b.execute(dH, dV)
            torch.cuda.synchronize()
            # one persistent launch, plus one reduction per capture split over pair ranges
            assert 1 <= capi.launch_count() - launches <= 1 + len(caps)
            assert b.check() == 0
            outs.append(volumes(caps, b, dV.cpu().numpy()))
    for i, c in enumerate(caps):
        ref = oracle.bp_gpu_f64(c.H, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT)
        for vols in outs:
            assert oracle.rel_l2(vols[i], ref) < tol(c), i
        if frac == 0.0:  # nothing to factor: both runs are the same launch
            assert np.array_equal(outs[0][i], outs[1][i])


@pytest.mark.parametrize("splits", [1, 3])
def test_batch_pair_splits_option(cuda, splits):
    """Every capture's units split over `splits` pair ranges (partial sums added after the
    launch in range order) or none: the same volumes within summation order."""
    caps = small_batch(n=6, seed=7)
    geo = synthetic.batch_geometry(caps)
    outs = []
    for sp in (splits, 0):
        with capi.Batch(geo, h_dtype=capi.DTYPE_F32, checked=1, pair_splits=sp) as b:
            H, dH, dV = upload(cuda, caps, b, np.float32, None)
            b.execute(dH, dV)
            assert b.check() == 0
            outs.append(volumes(caps, b, dV.cpu().numpy()))
    for i, c in enumerate(caps):
        assert oracle.rel_l2(outs[0][i], outs[1][i]) < 1e-6, i
        ref = oracle.bp_gpu_f64(c.H, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT)
        assert oracle.rel_l2(outs[0][i], ref) < tol(c), i


def test_batch_graph_replays_and_recaptures(cuda):
    import torch

    caps = small_batch(n=6, seed=4)
    scales = synthetic.fp16_scales(caps)
    with capi.Batch(synthetic.batch_geometry(caps, scales), h_dtype=capi.DTYPE_F16) as b:
        H, dH, dV = upload(cuda, caps, b, np.float16, scales)
        b.execute(dH, dV)
        torch.cuda.synchronize()
        first = dV.cpu().numpy()
        dV.fill_(float("nan"))
        b.graph_launch(dH, dV)
        b.check()
        assert np.array_equal(dV.cpu().numpy(), first)
        # the graph re-reads the buffer on every replay
        keep = dH.clone()
        dH.zero_()
        torch.cuda.synchronize()
        b.graph_launch(dH, dV)
        b.check()
        assert np.all(dV.cpu().numpy() == 0)
        dH.copy_(keep)
        torch.cuda.synchronize()
        for _ in range(3):
            b.graph_launch(dH, dV)
        b.check()
        assert np.array_equal(dV.cpu().numpy(), first)
        # new buffers: the graph is captured again
        dH2 = keep.clone()
        dV2 = torch.full_like(dV, float("nan"))
        torch.cuda.synchronize()
        b.graph_launch(dH2, dV2)
        b.check()
        assert np.array_equal(dV2.cpu().numpy(), first)


def test_batch_non_planar_capture(cuda):
    """One capture with SPADs off the wall plane switches the batch to the general form."""
    caps = small_batch(n=4, seed=5, exhaustive_frac=0.0)
    jitter = np.random.default_rng(8).uniform(-0.02, 0.02, caps[1].P).astype(np.float32)
    caps[1].pairs = caps[1].pairs.copy()
    caps[1].pairs["camera_point"][:, 1] += jitter
    geo = synthetic.batch_geometry(caps)
    with capi.Batch(geo, h_dtype=capi.DTYPE_F32, checked=1) as b:
        assert b.info()["planar"] == 0
        H, dH, dV = upload(cuda, caps, b, np.float32, None)
        b.execute(dH, dV)
        assert b.check() == 0
        vols = volumes(caps, b, dV.cpu().numpy())
    for i, c in enumerate(caps):
        ref = oracle.bp_gpu_f64(c.H, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT)
        assert oracle.rel_l2(vols[i], ref) < tol(c), i


def test_batch_confocal_and_single_capture(cuda):
    c = synthetic.make_capture("precision_64", seed=7, small=True, confocal=True)
    with capi.Batch(synthetic.batch_geometry([c]), h_dtype=capi.DTYPE_F32, checked=1) as b:
        H, dH, dV = upload(cuda, [c], b, np.float32, None)
        b.execute(dH, dV)
        assert b.check() == 0
        out = volumes([c], b, dV.cpu().numpy())[0]
    ref = oracle.bp_gpu_f64(c.H, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT)
    assert oracle.rel_l2(out, ref) < 5e-3


def test_batch_rejections(cuda):
    caps = small_batch(n=2, seed=6)
    geo = synthetic.batch_geometry(caps)
    with pytest.raises(capi.BackprojectorError) as e:
        capi.Batch(geo, h_dtype=capi.DTYPE_BF16)
    assert e.value.status == capi.ERR_UNSUPPORTED
    with pytest.raises(capi.BackprojectorError) as e:
        capi.Batch(geo, accum=capi.ACCUM_KAHAN)
    assert e.value.status == capi.ERR_UNSUPPORTED
    with pytest.raises(capi.BackprojectorError) as e:
        capi.Batch([], h_dtype=capi.DTYPE_F32)
    assert e.value.status == capi.ERR_INVALID_ARGUMENT
    bad = [dict(g) for g in geo]
    bad[1]["deltaT"] = float("nan")
    with pytest.raises(capi.BackprojectorError) as e:
        capi.Batch(bad)
    assert e.value.status == capi.ERR_INVALID_ARGUMENT
    assert "capture 1" in str(e.value)
