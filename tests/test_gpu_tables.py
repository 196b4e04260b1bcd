"""FAST plan tables are built on the GPU in FP64 (tables_fp64_kernel): they must equal,
bit for bit, the FP64 restatement below of the same arithmetic (the pair precompute keeps
its wall legs in double, backproject.hpp:356-418; the frame is the voxel basis normalised,
backproject.hpp:820-839), for single-laser, lasers x SPADs, confocal and rotated-basis
captures, and at full size."""
from __future__ import annotations

import numpy as np
import pytest

from backprojector_gb300 import capi, synthetic

pytestmark = pytest.mark.gpu


def expected_tables(pairs, zero, inc, t0, dT, L, S, confocal):
    """FP64 tables, each operation rounded separately in the kernel's order."""
    inc = np.asarray(inc, np.float32).reshape(3, 3).astype(np.float64)
    h = np.sqrt((inc[:, 0] * inc[:, 0] + inc[:, 1] * inc[:, 1]) + inc[:, 2] * inc[:, 2])
    u = inc / h[:, None]
    z = np.asarray(zero, np.float32).astype(np.float64)
    dT = np.float64(np.float32(dT))
    t0 = np.float64(np.float32(t0))

    def frame(pts):
        d = pts.astype(np.float64) - z[None, :]
        return np.stack([(u[r, 0] * d[:, 0] + u[r, 1] * d[:, 1]) + u[r, 2] * d[:, 2]
                         for r in range(3)], axis=1)

    sp = pairs[:S]
    cw = sp["camera_wall"].astype(np.float64)
    cs = (cw + sp["laser_wall"].astype(np.float64)) / dT if confocal else cw / dT
    spad = np.concatenate([frame(sp["camera_point"]), cs[:, None]], axis=1)
    heads = pairs[np.arange(L) * S]
    if confocal:
        las = np.zeros((1, 4))
        las[0, 3] = (-t0) / dT
    else:
        c = (-t0) / dT + heads["laser_wall"].astype(np.float64) / dT
        las = np.concatenate([frame(heads["laser_point"]), c[:, None]], axis=1)
    return np.concatenate([spad, las]).astype(np.float32)


CASES = {
    "single_laser": dict(name="precision_64", small=True),
    "lasers_x_spads": dict(name="dense_exhaustive_16", small=True),
    "confocal": dict(name="precision_64", small=True, confocal=True),
    "full_128x128": dict(name="octree_256", small=False),
}


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("rotated", [False, True])
def test_device_tables_bitwise(cuda, case, rotated):
    kw = dict(CASES[case])
    cap = synthetic.make_capture(kw.pop("name"), seed=5, render=False, **kw)
    zero, inc = cap.zero, cap.inc
    if rotated:  # a wall normal off the axes: a rotated voxel basis, non-planar lines
        zero, inc = capi.volume_basis(cap.volume_position, cap.volume_size, cap.voxels_per_side,
                                      wall_normal=(0.3, -1.0, 0.2))
    opts = [dict()]
    if case == "lasers_x_spads":
        opts.append(dict(unfactored=1))
    for o in opts:
        with capi.Plan(cap.pairs, cap.T, cap.voxels_per_side, zero, inc, cap.t0, cap.deltaT,
                       algo=capi.ALGO_FAST, **o) as plan:
            info = plan.info()
            L, S = int(info["num_lasers"]), int(info["num_spads"])
            got = plan.tables()
        confocal = bool(kw.get("confocal"))
        want = expected_tables(cap.pairs, zero, inc, cap.t0, cap.deltaT, L, S, confocal)
        assert got.shape == want.shape
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (
            int((got.view(np.uint32) != want.view(np.uint32)).sum()))
