"""Generates the golden fixtures: outputs of the reference's own kernel.

The reference (mjgalindo/backprojector) has no tests or golden vectors.  This script pins
the oracle and the CUDA path to the reference itself: it builds small seeded captures,
runs the reference's unmodified kernel cuda_backprojection_impl<float | cuComplex>
(backproject_cuda.cu:117-175, compiled from its sources into
oracle/_ref/backproject_cuda_ref.cubin by backprojector_gb300/build.py) through
oracle/ref_harness.cu with the reference launcher's policy, and stores inputs and
outputs as compressed .npz files.

Needs a GPU (run on the GB300 machine):
    python tests/golden/make_golden.py [out_dir]
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from backprojector_gb300 import build, capi, synthetic  # noqa: E402
from oracle import oracle  # noqa: E402


def save(out: Path, name: str, cap_or_inputs: dict, ref_vol, block: int, ms: float, note: str):
    d = dict(cap_or_inputs)
    d["ref_volume"] = ref_vol
    d["ref_block"] = np.int32(block)
    d["ref_ms"] = np.float64(ms)
    d["note"] = np.array(note)
    np.savez_compressed(out / f"{name}.npz", **d)
    print(f"{name}: block={block} ms={ms:.2f} |V|max={np.abs(ref_vol).max():.4g}")


def inputs(H, pairs, N, zero, inc, t0, dT):
    return dict(H=H, pairs=pairs.view(np.uint8).reshape(len(pairs), 32),
                N=np.asarray(N, np.uint32), zero=np.asarray(zero, np.float32),
                inc=np.asarray(inc, np.float32), t0=np.float32(t0), dT=np.float32(dT))


def run(H, pairs, N, zero, inc, t0, dT):
    return oracle.reference_gpu(H, pairs, N, zero, inc, t0, dT)


def main(out: Path) -> None:
    build.build_all()
    out.mkdir(parents=True, exist_ok=True)

    # exhaustive: 4x4 lasers x 4x4 SPADs (P = 256), Poisson counts, 16^3
    cap = synthetic.make_capture("dense_exhaustive_16", seed=11, small=True, laser_grid=(4, 4),
                                 spad_grid=(4, 4), voxels=16)
    a = inputs(cap.H, cap.pairs, cap.voxels_per_side, cap.zero, cap.inc, cap.t0, cap.deltaT)
    v, b, ms = run(cap.H, cap.pairs, cap.voxels_per_side, cap.zero, cap.inc, cap.t0, cap.deltaT)
    save(out, "exhaustive_p256_n16", a, v, b, ms, "integer counts; exhaustive 4x4 x 4x4")

    # single laser: 16x16 SPADs (P = 256), Poisson counts, T = 1024, 24^3
    cap = synthetic.make_capture("precision_64", seed=12, small=True)
    a = inputs(cap.H, cap.pairs, cap.voxels_per_side, cap.zero, cap.inc, cap.t0, cap.deltaT)
    v, b, ms = run(cap.H, cap.pairs, cap.voxels_per_side, cap.zero, cap.inc, cap.t0, cap.deltaT)
    save(out, "single_p256_n24", a, v, b, ms, "integer counts; one laser, 16x16 SPADs")

    # same geometry, H[p, t] = t + 1: exact integer sums of bin indices
    ramp = np.broadcast_to(np.arange(1, cap.T + 1, dtype=np.float32), cap.H.shape).copy()
    v, b, ms = run(ramp, cap.pairs, cap.voxels_per_side, cap.zero, cap.inc, cap.t0, cap.deltaT)
    a = inputs(np.zeros((0,), np.float32), cap.pairs, cap.voxels_per_side, cap.zero, cap.inc,
               cap.t0, cap.deltaT)
    a["H_kind"] = np.array("ramp")
    a["T"] = np.int32(cap.T)
    save(out, "single_ramp_n24", a, v, b, ms, "H[p,t] = t + 1 (regenerated in the test)")

    # ragged P (15 x 20 SPADs = 300 pairs): the reference drops P mod blockDim pairs
    cap = synthetic.make_capture("precision_64", seed=13, small=True, spad_grid=(15, 20), voxels=16)
    a = inputs(cap.H, cap.pairs, cap.voxels_per_side, cap.zero, cap.inc, cap.t0, cap.deltaT)
    v, b, ms = run(cap.H, cap.pairs, cap.voxels_per_side, cap.zero, cap.inc, cap.t0, cap.deltaT)
    save(out, "ragged_p300_n16", a, v, b, ms, "300 pairs: the reference uses the first 256")

    # N = 40 (not a multiple of 16): the reference's voxel cursor skips voxels
    cap = synthetic.make_capture("precision_64", seed=14, small=True, spad_grid=(8, 8), voxels=40,
                                 T=512)
    a = inputs(cap.H, cap.pairs, cap.voxels_per_side, cap.zero, cap.inc, cap.t0, cap.deltaT)
    v, b, ms = run(cap.H, cap.pairs, cap.voxels_per_side, cap.zero, cap.inc, cap.t0, cap.deltaT)
    save(out, "single_p64_n40", a, v, b, ms, "N=40: unvisited voxels stay 0")

    # complex64 (phasor): pulse-convolved rows, 8x8 SPADs, T = 512, 16^3
    cap = synthetic.make_capture("phasor_128", seed=15, small=True, spad_grid=(8, 8), T=512,
                                 voxels=16)
    Hc = oracle.phasor_pulse(cap.H, cap.wavelength, cap.deltaT)
    a = inputs(Hc, cap.pairs, cap.voxels_per_side, cap.zero, cap.inc, cap.t0, cap.deltaT)
    v, b, ms = run(Hc, cap.pairs, cap.voxels_per_side, cap.zero, cap.inc, cap.t0, cap.deltaT)
    save(out, "complex_p64_n16", a, v, b, ms, "complex64 phasor rows")

    # real-valued, noise-free rendering (non-integer sums), 16x16 SPADs, 20^3
    cap = synthetic.make_capture("octree_256", seed=16, small=True, voxels=20)
    a = inputs(cap.H, cap.pairs, cap.voxels_per_side, cap.zero, cap.inc, cap.t0, cap.deltaT)
    v, b, ms = run(cap.H, cap.pairs, cap.voxels_per_side, cap.zero, cap.inc, cap.t0, cap.deltaT)
    save(out, "objects_p256_n20", a, v, b, ms, "float radiance, no noise")
    print("golden fixtures written to", out, "with", capi.__name__)


if __name__ == "__main__":
    main(Path(sys.argv[1]) if len(sys.argv) > 1 else Path(__file__).resolve().parent)
