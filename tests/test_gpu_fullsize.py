"""Parity at the full benchmark shapes, against the FP64 oracle on seeded voxel samples
drawn uniformly over each volume (empty space included, not only occupied voxels):

* octree_256 dense: 1 laser x 128 x 128 SPADs, T = 4096, 256^3 (2.75e11 updates) -- FAST on
  FP32 rows and on FP16 rows with a per-capture scale;
* phasor_128: the pulse (bpgb_phasor_pulse on the GPU, bit-identical to the oracle's on
  sampled rows) then the complex FAST pass, complex64 rows and FP16 (re, im) rows;
* batch_64: the 64 uneven captures (grids up to 96^2, T up to 2048, volumes up to 96^3,
  16^2 x 16^2 lasers x SPADs captures) in the persistent batch launches, sampled voxels in
  every capture.

Tolerance: rel-L2 <= 1e-3 on the sampled voxels wherever P >= 1024 (the accuracy target
for FP32 arithmetic), FP16-stored rows scored against the oracle on the same
dequantised rows; mis-binned fraction of (voxel, pair) bins against the FP64 oracle's
<= 1e-3 on the dense capture.
"""
from __future__ import annotations

import numpy as np
import pytest

from backprojector_gb300 import capi, synthetic
from oracle import oracle

pytestmark = pytest.mark.gpu

SAMPLE = 512


def sample_ids(nvox, n=SAMPLE, seed=0):
    return np.sort(np.random.default_rng(seed).choice(nvox, size=min(n, nvox), replace=False))


@pytest.fixture(scope="module")
def dense_capture():
    return synthetic.make_capture("octree_256", seed=11)


@pytest.mark.parametrize("rows", ["f32", "f16"])
def test_dense_256_full_size(cuda, dense_capture, rows):
    import torch

    c = dense_capture
    N = tuple(int(v) for v in c.voxels_per_side)
    H = c.H
    opt = dict(algo=capi.ALGO_FAST, checked=1)
    if rows == "f16":
        scale = float(np.abs(H).max()) / 16384.0
        h16 = (H / np.float32(scale)).astype(np.float16)
        dH = torch.from_numpy(h16).to(cuda)
        H = h16.astype(np.float32) * np.float32(scale)  # what the kernel sums
        opt.update(h_dtype=capi.DTYPE_F16, h_scale=scale)
    else:
        dH = torch.from_numpy(H).to(cuda)
    dV = torch.full(N, float("nan"), device=cuda)
    with capi.Plan(c.pairs, c.T, N, c.zero, c.inc, c.t0, c.deltaT, **opt) as plan:
        plan.execute(dH, dV)
        assert plan.check() == 0
        out = dV.cpu().numpy().reshape(-1)
        ids = sample_ids(c.nvox)
        assert np.isfinite(out).all()
        ref = oracle.bp_gpu_f64(H, c.pairs, N, c.zero, c.inc, c.t0, c.deltaT, voxels=ids)
        rel = oracle.rel_l2(out[ids], ref)
        print(f"[octree_256 dense {rows}] rel-L2 vs FP64 oracle on {len(ids)} voxels {rel:.3e}")
        assert rel < 1e-3, rel
        if rows == "f32":
            bid = ids[:32]
            d = torch.empty((len(bid), c.P), dtype=torch.int32, device=cuda)
            plan.dump_bins(bid, d)
            b64 = oracle.bins(c.pairs, c.T, N, c.zero, c.inc, c.t0, c.deltaT, bid, 0)
            mis = oracle.misbinned_fraction(d.cpu().numpy(), b64)
            print(f"[octree_256 dense f32] mis-binned fraction {mis:.3e} ({len(bid)} x {c.P})")
            assert mis < 1e-3, mis


@pytest.fixture(scope="module")
def phasor_capture():
    return synthetic.make_capture("phasor_128", seed=12)


@pytest.mark.parametrize("rows", ["c64", "c32"])
def test_phasor_128_full_size(cuda, phasor_capture, rows):
    import torch

    c = phasor_capture
    N = tuple(int(v) for v in c.voxels_per_side)
    dH = torch.from_numpy(c.H).to(cuda)
    dHc = torch.empty(c.H.shape, dtype=torch.complex64, device=cuda)
    capi.phasor_pulse_device(dH, c.P, c.T, c.T, c.wavelength, c.deltaT, dHc, c.T)
    torch.cuda.synchronize()
    Hc = dHc.cpu().numpy()
    rows_chk = np.random.default_rng(1).choice(c.P, 24, replace=False)
    assert np.array_equal(Hc[rows_chk], oracle.phasor_pulse(c.H[rows_chk], c.wavelength, c.deltaT))
    opt = dict(algo=capi.ALGO_FAST, checked=1, h_dtype=capi.DTYPE_C64)
    src, Href = dHc, Hc
    if rows == "c32":
        flat = torch.view_as_real(dHc)
        scale = float(flat.abs().max()) / 16384.0
        src = (flat / scale).half().contiguous()
        Href = (src.float() * scale).cpu().numpy().view(np.complex64).reshape(c.P, c.T)
        opt.update(h_dtype=capi.DTYPE_C32, h_scale=scale)
    dV = torch.full(N, complex("nan"), dtype=torch.complex64, device=cuda)
    with capi.Plan(c.pairs, c.T, N, c.zero, c.inc, c.t0, c.deltaT, **opt) as plan:
        plan.execute(src, dV)
        assert plan.check() == 0
    out = dV.cpu().numpy().reshape(-1)
    ids = sample_ids(c.nvox, seed=2)
    ref = oracle.bp_gpu_c64(Href, c.pairs, N, c.zero, c.inc, c.t0, c.deltaT, voxels=ids)
    rel = oracle.rel_l2(out[ids], ref)
    print(f"[phasor_128 {rows}] rel-L2 vs FP64 oracle on {len(ids)} voxels {rel:.3e}")
    assert rel < 1e-3, rel


def test_batch_64_full_shapes(cuda):
    """Every capture of the 64-capture batch: 8 seeded voxels each against the FP64 oracle
    on the dequantised FP16 rows; P >= 1024 captures to 1e-3 on their samples, all samples
    together to 1e-3."""
    import torch

    caps = synthetic.make_batch(64, seed=0)
    scales = synthetic.fp16_scales(caps)
    geo = synthetic.batch_geometry(caps, scales)
    with capi.Batch(geo, h_dtype=capi.DTYPE_F16, checked=1) as b:
        info = b.info()
        Hh = synthetic.pack_batch(caps, b.row_offsets, info["pitch"], np.float16, scales)
        dH = torch.from_numpy(Hh).to(cuda)
        dV = torch.full((info["total_voxels"],), float("nan"), device=cuda)
        b.execute(dH, dV)
        assert b.check() == 0
        flat = dV.cpu().numpy()
        got_all, ref_all, big = [], [], 0
        for i, c in enumerate(caps):
            r, o = b.row_offsets[i], b.voxel_offsets[i]
            Hq = Hh[r:r + c.P, :c.T].astype(np.float32) * np.float32(scales[i])
            ids = sample_ids(c.nvox, n=8, seed=100 + i)
            ref = oracle.bp_gpu_f64(Hq, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0,
                                    c.deltaT, voxels=ids)
            got = flat[o:o + c.nvox][ids]
            assert np.isfinite(got).all()
            if c.P >= 1024 and np.linalg.norm(ref) > 0:
                big += 1
                assert oracle.rel_l2(got, ref) < 1e-3, (i, c.P, oracle.rel_l2(got, ref))
            got_all.append(got)
            ref_all.append(ref)
        assert big >= 16
        rel = oracle.rel_l2(np.concatenate(got_all), np.concatenate(ref_all))
        print(f"[batch_64] rel-L2 vs FP64 oracle on 8 voxels x 64 captures {rel:.3e}; "
              f"{big} captures with P >= 1024 each within 1e-3")
        assert rel < 1e-3, rel
