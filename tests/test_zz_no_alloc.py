"""The allocation-free entry point, bpgb_backproject_noalloc.

Callers that cannot allocate device memory while they reconstruct (a service on a fixed
memory pool, a host application whose allocator belongs to another framework) use this
call: it keeps its working memory in one static device array instead of cudaMalloc.
This test calls it through the C ABI twice in a row and checks each result against the
FAST plan path (bpgb_plan_execute) within the parity tolerance the other GPU tests use
for FAST results (rel-L2 5e-3 against the FP64 oracle; here the two paths run the same
kernel, so they must agree to 1e-6).  The file sorts last so that a run stopping at the
first failure has already run every other test.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from backprojector_gb300 import capi, synthetic
from oracle import oracle

pytestmark = pytest.mark.gpu


def noalloc(cap, dH, dP, dV, num_lasers, num_spads, confocal=False):
    import torch

    n = np.asarray(cap.voxels_per_side, np.uint32)
    st = capi.lib().bpgb_backproject_noalloc(
        C.c_void_p(dH.data_ptr()), cap.T, 0, C.c_void_p(dP.data_ptr()), num_lasers, num_spads,
        1 if confocal else 0, capi.u32ptr(n), capi.fptr(cap.zero), capi.fptr(cap.inc), cap.t0,
        cap.deltaT, C.c_void_p(dV.data_ptr()), C.c_void_p(torch.cuda.current_stream().cuda_stream))
    capi.check(st, "bpgb_backproject_noalloc")
    return dV.cpu().numpy()


def plan_result(cap, dH):
    import torch

    dV = torch.empty(tuple(int(v) for v in cap.voxels_per_side), dtype=torch.float32, device=dH.device)
    # the no-alloc call runs the per-pair form of the FAST kernel (lasers x SPADs captures
    # included), so it is compared with plans that do too
    with capi.Plan(cap.pairs, cap.T, cap.voxels_per_side, cap.zero, cap.inc, cap.t0, cap.deltaT,
                   algo=capi.ALGO_FAST, unfactored=1) as plan:
        plan.execute(dH, dV)
        plan.check()
    return dV.cpu().numpy()


@pytest.mark.parametrize("name,kw,L", [
    ("precision_64", dict(), 1),
    ("dense_exhaustive_16", dict(laser_grid=(4, 4), spad_grid=(8, 8), voxels=16), 16),
])
def test_noalloc_matches_plan_path_twice(cuda, name, kw, L):
    import torch

    caps = [synthetic.make_capture(name, seed=s, small=True, **kw) for s in (21, 22)]
    for cap in caps:  # two calls in a row, different captures: no stale scratch
        dH = torch.from_numpy(cap.H).to(cuda)
        dP = torch.from_numpy(cap.pairs.view(np.uint8).copy()).to(cuda)
        dV = torch.full(tuple(int(v) for v in cap.voxels_per_side), float("nan"), device=cuda)
        got = noalloc(cap, dH, dP, dV, L, cap.P // L)
        want = plan_result(cap, dH)
        assert np.isfinite(got).all()
        assert oracle.rel_l2(got, want) < 1e-6
        ref = oracle.bp_gpu_f64(cap.H, cap.pairs, cap.voxels_per_side, cap.zero, cap.inc, cap.t0,
                                cap.deltaT)
        assert oracle.rel_l2(got, ref) < 5e-3


def test_noalloc_large_volume_direct_store(cuda):
    """A 256^3 volume (67 MB of FP32) leaves no room for per-split partial sums in the
    16 MiB array: the call runs unsplit and stores straight into the volume.  Checked
    against the FP64 oracle on seeded voxels and against a plan, whose own split count
    may differ (sums in another order, hence 1e-5)."""
    import torch

    cap = synthetic.make_capture("octree_256", seed=31, spad_grid=(16, 16))
    dH = torch.from_numpy(cap.H).to(cuda)
    dP = torch.from_numpy(cap.pairs.view(np.uint8).copy()).to(cuda)
    dV = torch.full(tuple(int(v) for v in cap.voxels_per_side), float("nan"), device=cuda)
    for _ in range(2):
        got = noalloc(cap, dH, dP, dV, 1, cap.P)
        assert np.isfinite(got).all()
        assert oracle.rel_l2(got, plan_result(cap, dH)) < 1e-5
    ids = np.random.default_rng(3).choice(cap.nvox, 2048, replace=False)
    ref = oracle.bp_gpu_f64(cap.H, cap.pairs, cap.voxels_per_side, cap.zero, cap.inc, cap.t0,
                            cap.deltaT, voxels=ids)
    assert oracle.rel_l2(got.reshape(-1)[ids], ref) < 5e-3


def test_noalloc_rejects_bad_requests(cuda):
    import torch

    cap = synthetic.make_capture("precision_64", seed=23, small=True)
    dH = torch.from_numpy(cap.H).to(cuda)
    dP = torch.from_numpy(cap.pairs.view(np.uint8).copy()).to(cuda)
    dV = torch.zeros(tuple(int(v) for v in cap.voxels_per_side), device=cuda)
    # tables beyond the static array
    too_many = (16 << 20) // 16
    with pytest.raises(capi.BackprojectorError) as e:
        noalloc(cap, dH, dP, dV, 1, too_many)
    assert e.value.status == capi.ERR_INVALID_ARGUMENT
    # a stated factorisation the pair list does not have
    with pytest.raises(capi.BackprojectorError) as e:
        noalloc(cap, dH, dP, dV, 2, cap.P // 2)
    assert e.value.status == capi.ERR_INVALID_ARGUMENT
    # the next call still works
    got = noalloc(cap, dH, dP, dV, 1, cap.P)
    assert oracle.rel_l2(got, plan_result(cap, dH)) < 1e-6
