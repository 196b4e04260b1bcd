"""The capture-level time window: the reference's semantics (get_time_limits' corner
bound and the unfloored chunked_t0, backproject.hpp:617-674, :847 -- t0_mode 4) against
the intended ones (a bound over every grid point, floored offset -- t0_mode 1), measured
per (voxel, pair) bin on the original time axis.

Two effects separate them.  (1) The corner bound's minimum is not a lower bound on the
path length (the shortest paths run through interior grid points), so the reference's
crop drops the earliest bins a voxel reaches: those bins read as out of range.  (2) The
fractional chunk offset frac(m) shifts every remaining bin's rounding point, so a fraction
of about frac(m) of them moves by one bin."""
from __future__ import annotations

import numpy as np
import pytest

from backprojector_gb300 import capi, synthetic

pytestmark = pytest.mark.gpu


def original_bins(cuda, c, T, t0, frm, ids):
    import torch

    with capi.Plan(c.pairs, T, c.voxels_per_side, c.zero, c.inc, t0, c.deltaT,
                   algo=capi.ALGO_FAST, h_pitch=(T + 3) // 4 * 4) as plan:
        d = torch.empty((len(ids), c.P), dtype=torch.int32, device=cuda)
        plan.dump_bins(ids, d)
        b = d.cpu().numpy().astype(np.int64)
    o = np.where(b >= 0, b + frm, -1)
    # bins outside the capture's [0, T) read zeros in every form: out of range
    return np.where((o >= 0) & (o < c.T), o, -1)


@pytest.mark.parametrize("name,small", [("precision_64", False), ("dense_exhaustive_16", False),
                                        ("octree_256", False)])
def test_reference_window_vs_intended(cuda, name, small):
    c = synthetic.make_capture(name, seed=2, small=small, render=False)
    args = (c.camera_grid, c.laser_grid, c.camera_position, c.laser_position, c.t0, c.deltaT,
            False, c.volume_position, c.volume_size)
    fr4, ln4, ct4 = capi.capture_window(*args, t0_mode=4)
    fr1, ln1, ct1 = capi.capture_window(*args, t0_mode=1)
    mc, _ = capi.time_limits(c.laser_position, c.laser_grid, c.camera_position, c.camera_grid,
                             c.volume_position, c.volume_size, c.t0, c.deltaT, corners=True)
    ids = np.sort(np.random.default_rng(3).choice(c.nvox, size=min(256, c.nvox), replace=False))
    ref = original_bins(cuda, c, ln4, ct4, fr4, ids)
    want = original_bins(cuda, c, ln1, ct1, fr1, ids)
    # the intended window keeps every bin the uncropped capture has
    full = original_bins(cuda, c, c.T, c.t0, 0, ids)
    assert np.mean(want != full) < 1e-3
    reached = want >= 0
    dropped = float(np.mean(reached & (ref < 0)))
    both = reached & (ref >= 0)
    shifted = float(np.mean(ref[both] != want[both])) if both.any() else 0.0
    frac = mc - np.floor(mc)
    print(f"\n[{name}{' small' if small else ''}] corner m {mc:.3f} (all-points window starts at "
          f"{fr1}); reference-exact vs intended: dropped {dropped:.4f} of the reached bins, "
          f"{shifted:.4f} of the rest one bin off (frac(m) = {frac:.3f})")
    # kept bins move by one bin at most, for about frac(m) of them
    assert both.mean() > 0.05
    assert np.all(np.abs(ref[both] - want[both]) <= 1)
    assert abs(shifted - frac) < 0.05 or abs(shifted - (1 - frac)) < 0.05
