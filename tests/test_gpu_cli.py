"""The command-line tool (bpgb_backprojector) on datasets written as .npz: its volumes
equal the nlosbpy binding's for the same capture (same library path, same arithmetic)."""
from __future__ import annotations

import subprocess

import numpy as np
import pytest

from backprojector_gb300 import build, octree, synthetic
from tests.test_cpu import write_dataset

pytestmark = pytest.mark.gpu


def run(*args):
    r = subprocess.run([str(build.CLI_PATH), *map(str, args)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return r.stdout


def test_cli_dense_and_bounces_match_binding(cuda, tmp_path):
    from backprojector_gb300 import load_nlosbpy

    nl = load_nlosbpy()
    c = synthetic.make_capture("dense_exhaustive_16", seed=3, small=True,
                               laser_grid=(4, 4), spad_grid=(8, 8), voxels=16)
    write_dataset(tmp_path / "cap.npz", c)
    out = run(tmp_path / "cap.npz", "-r", 16, 16, 16, "-o", tmp_path / "vol.npy")
    assert "Backprojected to" in out
    vol = np.load(tmp_path / "vol.npy")
    ref = nl.backproject(c.transient_array(), c.camera_grid, c.laser_grid, c.camera_position,
                         c.laser_position, c.t0, c.deltaT, False, c.volume_position,
                         c.volume_size, c.voxels_per_side, np.zeros(3, np.float32),
                         assume_row_major=True)
    assert vol.dtype == np.float32 and vol.shape == (16, 16, 16)
    assert np.array_equal(vol, ref)
    # a bounce axis: slices of bounce 3..-b are summed (bounce 5 is left out at -b 4)
    H = c.transient_array()
    stacked = np.stack([0.25 * H, 0.75 * H, 100.0 * H], axis=-2)
    write_dataset(tmp_path / "b.npz", c, data=stacked, bounces=np.array([3, 4, 5]))
    run(tmp_path / "b.npz", "-r", 16, 16, 16, "-b", 4, "-o", tmp_path / "vb.npy")
    assert np.allclose(np.load(tmp_path / "vb.npy"), ref, rtol=1e-5, atol=1e-5 * np.abs(ref).max())
    # default output name and aspect-scaled resolution (equal -r values follow the size)
    write_dataset(tmp_path / "flat.npz", c, hidden_volume_size=np.array([0.5, 0.25, 0.5],
                                                                          np.float32))
    run(tmp_path / "flat.npz", "-r", 16, 16, 16)
    assert np.load(tmp_path / "flat_recon.npy").shape == (16, 8, 16)


def test_cli_phasor_magnitude_matches_binding(cuda, tmp_path):
    from backprojector_gb300 import load_nlosbpy

    nl = load_nlosbpy()
    c = synthetic.make_capture("phasor_128", seed=4, small=True)
    write_dataset(tmp_path / "ph.npz", c)
    n = int(c.voxels_per_side[0])
    run(tmp_path / "ph.npz", "--phasor", "-w", c.wavelength, "-r", n, n, n, "-o",
        tmp_path / "ph.npy")
    ref = nl.phasor(c.transient_array(), c.camera_grid, c.laser_grid, c.camera_position,
                    c.laser_position, c.t0, c.deltaT, False, c.volume_position, c.volume_size,
                    c.voxels_per_side, c.wavelength, assume_row_major=True)
    got = np.load(tmp_path / "ph.npy")
    assert np.allclose(got, np.abs(ref), rtol=1e-6, atol=1e-6 * np.abs(ref).max())


@pytest.mark.parametrize("fp16", [False, True])
def test_cli_learned_octree_runs(cuda, tmp_path, fp16):
    c = synthetic.make_capture("octree_256", seed=5, small=True)
    write_dataset(tmp_path / "oc.npz", c)
    args = [tmp_path / "oc.npz", "--octree", "--weights", octree.WEIGHTS, "-r", 32, 32, 32,
            "-o", tmp_path / "oc.npy"]
    out = run(*args, *(["--fp16"] if fp16 else []))
    assert "tiles at full resolution" in out
    vol = np.load(tmp_path / "oc.npy")
    assert vol.shape == (32, 32, 32) and np.all(np.isfinite(vol)) and vol.max() > 0
