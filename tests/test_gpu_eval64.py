"""bpgb_eval_f64_voxels (the GPU's FP64 evaluation used by the bench to score FP32
results) against the FP64 CPU oracle: the same operations in the same order, so the
values must be identical bit for bit, real and complex rows, small and full-size
captures."""
from __future__ import annotations

import numpy as np
import pytest

from backprojector_gb300 import capi, synthetic
from oracle import oracle

pytestmark = pytest.mark.gpu


def gpu_eval(cuda, H, pairs, N, zero, inc, t0, dT, ids):
    import torch

    cplx = np.iscomplexobj(H)
    dH = torch.from_numpy(np.ascontiguousarray(H.astype(np.complex64 if cplx else np.float32))).to(cuda)
    dP = torch.from_numpy(pairs.view(np.uint8).copy()).to(cuda)
    dI = torch.from_numpy(np.asarray(ids, np.int64)).to(cuda)
    dO = torch.empty(len(ids) * (2 if cplx else 1), dtype=torch.float64, device=cuda)
    capi.eval_f64_voxels(dH, H.shape[-1], dP, len(pairs), N, zero, inc, t0, dT, dI, dO,
                         is_complex=cplx)
    torch.cuda.synchronize()
    out = dO.cpu().numpy()
    return out.view(np.complex128) if cplx else out


@pytest.mark.parametrize("name,kw", [
    ("precision_64", dict(small=True)),
    ("dense_exhaustive_16", dict(small=True)),
    ("octree_256", dict()),
])
def test_eval_f64_bitwise_vs_oracle(cuda, name, kw):
    c = synthetic.make_capture(name, seed=4, **kw)
    ids = np.random.default_rng(6).choice(c.nvox, size=min(384, c.nvox), replace=False)
    got = gpu_eval(cuda, c.H, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT, ids)
    ref = oracle.bp_gpu_f64(c.H, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT,
                            voxels=ids)
    assert np.array_equal(got, ref), np.abs(got - ref).max()


def test_eval_f64_complex_bitwise_vs_oracle(cuda):
    c = synthetic.make_capture("phasor_128", seed=4, small=True)
    Hc = oracle.phasor_pulse(c.H, c.wavelength, c.deltaT)
    ids = np.arange(0, c.nvox, 7)
    got = gpu_eval(cuda, Hc, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT, ids)
    ref = oracle.bp_gpu_c64(Hc, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT,
                            voxels=ids)
    assert np.array_equal(got, ref)
