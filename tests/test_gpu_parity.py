"""GPU parity: the CUDA path (through the C ABI) against the reference kernel's outputs
(golden fixtures) and the FP64 CPU oracle.

Tolerances (vs the FP64 oracle, on real-valued renderings):
  EXACT  rel-L2 <= 2e-3: FP32 geometry flips ~0.1% of bins (the reference's own rate);
  FAST   rel-L2 <= 1e-3 where P >= 1024 (FP32, Kahan and FP16 rows), 5e-3 / 6e-3 below
         (one flipped bin moves a voxel by 1/P of its sum), BF16 2e-2; mis-binned
         fraction <= 1%;
against the reference kernel (golden): EXACT bit-identical on integer-valued H, FAST
rel-L2 <= 5e-3 with <= 1e-3 of its bins differing from the reference's.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

from backprojector_gb300 import capi, synthetic
from oracle import oracle

GOLDEN = Path(__file__).resolve().parent / "golden"

pytestmark = pytest.mark.gpu


def golden(name):
    p = GOLDEN / f"{name}.npz"
    if not p.exists():
        pytest.skip(f"golden fixture {name} not generated")
    z = np.load(p)
    d = {k: z[k] for k in z.files}
    d["pairs"] = np.ascontiguousarray(d["pairs"]).view(capi.PAIR_DTYPE).reshape(-1)
    if str(d.get("H_kind", "")) == "ramp":
        T = int(d["T"])
        d["H"] = np.broadcast_to(np.arange(1, T + 1, dtype=np.float32), (len(d["pairs"]), T)).copy()
    return d


def run_plan(cuda, H, pairs, N, zero, inc, t0, dT, **opt):
    import torch

    cplx = np.iscomplexobj(H)
    dtype = opt.get("h_dtype", capi.DTYPE_C64 if cplx else capi.DTYPE_F32)
    opt["h_dtype"] = dtype
    Hn = np.ascontiguousarray(H)
    if dtype == capi.DTYPE_F16:
        dH = torch.from_numpy(Hn.astype(np.float32)).to(cuda).half()
    elif dtype == capi.DTYPE_BF16:
        dH = torch.from_numpy(Hn.astype(np.float32)).to(cuda).bfloat16()
    elif dtype == capi.DTYPE_C32:
        # interleaved FP16 (re, im) with a per-capture scale
        flat = Hn.astype(np.complex64).view(np.float32)
        scale = float(np.abs(flat).max()) / 16384.0 or 1.0
        opt["h_scale"] = scale
        dH = (torch.from_numpy(flat / np.float32(scale)).to(cuda)).half()
    elif cplx:
        dH = torch.from_numpy(Hn.astype(np.complex64)).to(cuda)
    else:
        dH = torch.from_numpy(Hn.astype(np.float32)).to(cuda)
    shape = tuple(int(v) for v in N)
    dV = torch.full(shape, float("nan"), dtype=torch.complex64 if cplx else torch.float32,
                    device=cuda)
    with capi.Plan(pairs, H.shape[-1], N, zero, inc, t0, dT, **opt) as plan:
        plan.execute(dH, dV)
        viol = plan.check()
        info = plan.info()
        out = dV.cpu().numpy()
    return out, info, viol


# ---------------------------------------------------------------- vs the reference kernel

@pytest.mark.parametrize("name", ["exhaustive_p256_n16", "single_p256_n24", "single_ramp_n24"])
def test_exact_bit_identical_to_reference_kernel(cuda, name):
    g = golden(name)
    out, info, _ = run_plan(cuda, g["H"], g["pairs"], g["N"], g["zero"], g["inc"], float(g["t0"]),
                            float(g["dT"]), algo=capi.ALGO_EXACT)
    assert info["algo"] == "exact"
    # integer-valued H: every partial sum is exact, so equal bins <=> equal volumes
    assert np.array_equal(out, g["ref_volume"]), np.abs(out - g["ref_volume"]).max()


def test_exact_float_rows_vs_reference_kernel(cuda):
    g = golden("objects_p256_n20")
    out, _, _ = run_plan(cuda, g["H"], g["pairs"], g["N"], g["zero"], g["inc"], float(g["t0"]),
                         float(g["dT"]), algo=capi.ALGO_EXACT)
    # same bins, different summation order only
    assert oracle.rel_l2(out, g["ref_volume"]) < 1e-6


def test_exact_complex_vs_reference_kernel(cuda):
    g = golden("complex_p64_n16")
    out, _, _ = run_plan(cuda, g["H"], g["pairs"], g["N"], g["zero"], g["inc"], float(g["t0"]),
                         float(g["dT"]), algo=capi.ALGO_EXACT)
    assert oracle.rel_l2(out, g["ref_volume"]) < 1e-6


def test_ragged_pairs_reference_drops_tail(cuda):
    """P = 300: the reference loops i < P / blockDim and ignores the last 44 pairs
    (backproject_cuda.cu:150); this engine uses all of them."""
    g = golden("ragged_p300_n16")
    block = int(g["ref_block"])
    kept = (len(g["pairs"]) // block) * block
    assert kept < len(g["pairs"])
    out_kept, _, _ = run_plan(cuda, g["H"][:kept], g["pairs"][:kept], g["N"], g["zero"], g["inc"],
                              float(g["t0"]), float(g["dT"]), algo=capi.ALGO_EXACT)
    assert np.array_equal(out_kept, g["ref_volume"])
    out_all, _, _ = run_plan(cuda, g["H"], g["pairs"], g["N"], g["zero"], g["inc"], float(g["t0"]),
                             float(g["dT"]), algo=capi.ALGO_EXACT)
    ref_all = oracle.bp_gpu_f64(g["H"], g["pairs"], g["N"], g["zero"], g["inc"], float(g["t0"]),
                                float(g["dT"]))
    assert oracle.rel_l2(out_all, ref_all) < 2e-3


def test_n40_every_voxel_visited(cuda):
    """N = 40 (not a multiple of 16): the reference's voxel cursor wraps
    (backproject_cuda.cu:65-80) and recomputes some voxels; every voxel it writes matches
    this engine exactly."""
    g = golden("single_p64_n40")
    out, _, _ = run_plan(cuda, g["H"], g["pairs"], g["N"], g["zero"], g["inc"], float(g["t0"]),
                         float(g["dT"]), algo=capi.ALGO_EXACT)
    seen = oracle.reference_visited(g["N"])
    assert np.array_equal(out[seen], g["ref_volume"][seen])
    assert np.all(g["ref_volume"][~seen] == 0)
    ref = oracle.bp_gpu_f64(g["H"], g["pairs"], g["N"], g["zero"], g["inc"], float(g["t0"]),
                            float(g["dT"]))
    assert oracle.rel_l2(out, ref) < 2e-3


GOLDEN_ALL = ["exhaustive_p256_n16", "single_p256_n24", "single_ramp_n24", "objects_p256_n20",
              "complex_p64_n16", "ragged_p300_n16", "single_p64_n40"]


@pytest.mark.parametrize("name", GOLDEN_ALL)
def test_fast_vs_reference_kernel_golden(cuda, name):
    """The default (FAST) algorithm against the reference kernel's own volumes, and its
    bins against the reference's: EXACT's bins, which are the reference kernel's (the
    integer-row fixtures above are bit-identical).  Tolerance: rel-L2 <= 5e-3 at these
    pair counts (P <= 300: one flipped bin moves a voxel by 1/P of its sum), mis-binned
    fraction <= 1e-3."""
    import torch

    g = golden(name)
    H, pairs = g["H"], g["pairs"]
    if name == "ragged_p300_n16":  # the reference used the first P - P mod blockDim pairs
        kept = (len(pairs) // int(g["ref_block"])) * int(g["ref_block"])
        H, pairs = H[:kept], pairs[:kept]
    args = (pairs, g["N"], g["zero"], g["inc"], float(g["t0"]), float(g["dT"]))
    out, info, viol = run_plan(cuda, H, *args, algo=capi.ALGO_FAST, checked=1)
    assert info["algo"] == "fast" and viol == 0
    ref = g["ref_volume"]
    seen = oracle.reference_visited(g["N"]) if name == "single_p64_n40" else np.ones(ref.shape, bool)
    rel = oracle.rel_l2(out[seen], ref[seen])
    assert rel < 5e-3, rel
    nvox = int(np.prod(g["N"].astype(np.int64)))
    ids = np.flatnonzero(seen.reshape(-1))
    bins = {}
    for algo in (capi.ALGO_FAST, capi.ALGO_EXACT):
        opt = dict(algo=algo)
        if np.iscomplexobj(H):
            opt["h_dtype"] = capi.DTYPE_C64
        with capi.Plan(pairs, H.shape[-1], *args[1:], **opt) as plan:
            d = torch.empty((len(ids), len(pairs)), dtype=torch.int32, device=cuda)
            plan.dump_bins(ids, d)
            bins[algo] = d.cpu().numpy()
    mis = oracle.misbinned_fraction(bins[capi.ALGO_FAST], bins[capi.ALGO_EXACT])
    print(f"[{name}] FAST vs reference kernel: rel-L2 {rel:.3e}, mis-binned {mis:.3e}")
    assert mis < 1e-3, mis
    assert len(ids) <= nvox


# ---------------------------------------------------------------- vs the FP64 oracle

CASES = [
    ("dense_exhaustive_16", dict(laser_grid=(4, 4), spad_grid=(8, 8), voxels=16)),
    ("precision_64", dict()),
    ("octree_256", dict()),
]


def _cap(name, kw, seed=5):
    return synthetic.make_capture(name, seed=seed, small=True, **kw)


@pytest.mark.parametrize("name,kw", CASES)
def test_exact_vs_fp64_oracle_and_misbinned(cuda, name, kw):
    import torch

    c = _cap(name, kw)
    ref = oracle.bp_gpu_f64(c.H, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT)
    out, _, _ = run_plan(cuda, c.H, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT,
                         algo=capi.ALGO_EXACT)
    assert oracle.rel_l2(out, ref) < 2e-3
    ids = np.random.default_rng(0).choice(c.nvox, size=min(64, c.nvox), replace=False)
    with capi.Plan(c.pairs, c.T, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT,
                   algo=capi.ALGO_EXACT) as plan:
        d = torch.empty((len(ids), c.P), dtype=torch.int32, device=cuda)
        plan.dump_bins(ids, d)
        gpu_bins = d.cpu().numpy()
    b64 = oracle.bins(c.pairs, c.T, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT, ids, 0)
    b32 = oracle.bins(c.pairs, c.T, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT, ids, 1)
    assert oracle.misbinned_fraction(gpu_bins, b64) < 5e-3
    # the CPU FP32 emulation differs from norm3df only next to .5 boundaries
    assert oracle.misbinned_fraction(gpu_bins, b32) < 1e-3


FAST_VARIANTS = [
    dict(h_dtype=capi.DTYPE_F32, accum=capi.ACCUM_F32),
    dict(h_dtype=capi.DTYPE_F32, accum=capi.ACCUM_KAHAN),
    dict(h_dtype=capi.DTYPE_F16, accum=capi.ACCUM_F32),
    dict(h_dtype=capi.DTYPE_BF16, accum=capi.ACCUM_KAHAN),
]


@pytest.mark.parametrize("name,kw", CASES)
@pytest.mark.parametrize("var", FAST_VARIANTS, ids=["f32", "kahan", "f16", "bf16kahan"])
def test_fast_vs_fp64_oracle(cuda, name, kw, var):
    c = _cap(name, kw)
    ref = oracle.bp_gpu_f64(c.H, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT)
    H = c.H
    scale = 1.0
    if var["h_dtype"] in (capi.DTYPE_F16, capi.DTYPE_BF16):
        scale = float(np.abs(H).max()) / 1024.0 or 1.0
        H = H / scale
    out, info, viol = run_plan(cuda, H, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT,
                               algo=capi.ALGO_FAST, checked=1, h_scale=scale, **var)
    assert info["algo"] == "fast"
    assert viol == 0
    # 1e-3 wherever P >= 1024 (FP32 / FP16 rows); below that one flipped bin moves a voxel
    # by 1/P of its sum
    tol = {capi.DTYPE_F32: 5e-3, capi.DTYPE_F16: 6e-3, capi.DTYPE_BF16: 2e-2}[var["h_dtype"]]
    if c.P >= 1024 and var["h_dtype"] != capi.DTYPE_BF16:
        tol = 1e-3
    assert oracle.rel_l2(out, ref) < tol


@pytest.mark.parametrize("name,kw", CASES)
def test_fast_misbinned_fraction(cuda, name, kw):
    import torch

    c = _cap(name, kw)
    ids = np.random.default_rng(1).choice(c.nvox, size=min(64, c.nvox), replace=False)
    with capi.Plan(c.pairs, c.T, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT,
                   algo=capi.ALGO_FAST) as plan:
        d = torch.empty((len(ids), c.P), dtype=torch.int32, device=cuda)
        plan.dump_bins(ids, d)
        gpu_bins = d.cpu().numpy()
    b64 = oracle.bins(c.pairs, c.T, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT, ids, 0)
    assert oracle.misbinned_fraction(gpu_bins, b64) < 1e-2


def test_fast_matches_its_own_bin_dump(cuda):
    """The FAST volume equals the sum of H at the bins its dump reports (same arithmetic)."""
    import torch

    c = _cap("precision_64", {})
    out, _, _ = run_plan(cuda, c.H, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT,
                         algo=capi.ALGO_FAST)
    ids = np.arange(0, c.nvox, 97)
    with capi.Plan(c.pairs, c.T, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT,
                   algo=capi.ALGO_FAST) as plan:
        d = torch.empty((len(ids), c.P), dtype=torch.int32, device=cuda)
        plan.dump_bins(ids, d)
        b = d.cpu().numpy()
    rows = np.arange(c.P)[None, :]
    vals = np.where(b >= 0, c.H[rows, np.clip(b, 0, c.T - 1)], 0.0).astype(np.float64).sum(1)
    assert np.allclose(out.ravel()[ids], vals, rtol=1e-5, atol=1e-3)


def _dump(cuda, c, ids, **opt):
    import torch

    with capi.Plan(c.pairs, c.T, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT,
                   algo=capi.ALGO_FAST, **opt) as plan:
        d = torch.empty((len(ids), c.P), dtype=torch.int32, device=cuda)
        plan.dump_bins(ids, d)
        return d.cpu().numpy(), plan.info()


@pytest.mark.parametrize("chunk,splits", [(0, 0), (4, 1), (12, 3), (64, 7)])
def test_factored_exhaustive_vs_oracle(cuda, chunk, splits):
    """Lasers x SPADs captures take the factored form (legs per voxel and laser / SPAD,
    reused across the other grid); partial laser groups (12-row stages = 3 lasers over 16)
    and pair splits that start inside a SPAD block included."""
    c = _cap("dense_exhaustive_16", dict(laser_grid=(4, 4), spad_grid=(8, 8), voxels=16))
    ref = oracle.bp_gpu_f64(c.H, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT)
    opt = dict(chunk=chunk, pair_splits=splits)
    out, info, viol = run_plan(cuda, c.H, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0,
                               c.deltaT, algo=capi.ALGO_FAST, checked=1, **opt)
    assert info["factored"] == 1 and info["geometry"] == "exhaustive" and viol == 0
    assert oracle.rel_l2(out, ref) < 5e-3
    plain, _, _ = run_plan(cuda, c.H, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0,
                           c.deltaT, algo=capi.ALGO_FAST, **opt)
    assert np.array_equal(plain, out)  # the checked variant changes nothing in range
    unf, uinfo, _ = run_plan(cuda, c.H, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0,
                             c.deltaT, algo=capi.ALGO_FAST, unfactored=1, **opt)
    assert uinfo["factored"] == 0 and oracle.rel_l2(unf, ref) < 5e-3
    # the volume is the sum of H at the bins the dump reports (same arithmetic), and those
    # bins match the FP64 oracle's
    ids = np.arange(0, c.nvox, 13)
    b, dinfo = _dump(cuda, c, ids, **opt)
    assert dinfo["factored"] == 1
    rows = np.arange(c.P)[None, :]
    vals = np.where(b >= 0, c.H[rows, np.clip(b, 0, c.T - 1)], 0.0).astype(np.float64).sum(1)
    assert np.allclose(out.ravel()[ids], vals, rtol=1e-5, atol=1e-3)
    b64 = oracle.bins(c.pairs, c.T, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT, ids, 0)
    assert oracle.misbinned_fraction(b, b64) < 1e-2


def test_factored_exhaustive_full_size(cuda):
    """The 16x16 lasers x 16x16 SPADs capture at 32^3 (65,536 pairs): FP32 and FP16 rows
    against the volume's own bin dump and the FP64 oracle's bins on sampled voxels."""
    c = synthetic.make_capture("dense_exhaustive_16", seed=3)
    ids = np.random.default_rng(2).choice(c.nvox, size=48, replace=False)
    b, info = _dump(cuda, c, ids)
    assert info["factored"] == 1
    b64 = oracle.bins(c.pairs, c.T, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT, ids, 0)
    assert oracle.misbinned_fraction(b, b64) < 1e-2
    rows = np.arange(c.P)[None, :]
    vals = np.where(b >= 0, c.H[rows, np.clip(b, 0, c.T - 1)], 0.0).astype(np.float64).sum(1)
    out, _, viol = run_plan(cuda, c.H, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0,
                            c.deltaT, algo=capi.ALGO_FAST, checked=1)
    assert viol == 0
    assert np.allclose(out.ravel()[ids], vals, rtol=1e-5, atol=1e-3)
    scale = float(np.abs(c.H).max()) / 1024.0
    h16 = (c.H / scale).astype(np.float16)
    out16, info16, _ = run_plan(cuda, h16.astype(np.float32), c.pairs, c.voxels_per_side, c.zero,
                                c.inc, c.t0, c.deltaT, algo=capi.ALGO_FAST,
                                h_dtype=capi.DTYPE_F16, h_scale=scale)
    assert info16["factored"] == 1
    # FP16 rows align windows to 16 bytes = 8 bins, which moves the legs' constants: a few
    # .5-boundary bins may differ from the FP32 dump
    vals16 = np.where(b >= 0, h16.astype(np.float64)[rows, np.clip(b, 0, c.T - 1)], 0.0).sum(1)
    assert oracle.rel_l2(out16.ravel()[ids], vals16 * scale) < 1e-3
    assert oracle.rel_l2(out16, out) < 5e-3


def test_fast_complex_vs_oracle(cuda):
    c = _cap("phasor_128", {})
    Hc = oracle.phasor_pulse(c.H, c.wavelength, c.deltaT)
    ref = oracle.bp_gpu_c64(Hc, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT)
    out, info, viol = run_plan(cuda, Hc, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT,
                               algo=capi.ALGO_FAST, checked=1)
    assert info["algo"] == "fast" and viol == 0
    assert oracle.rel_l2(out, ref) < 5e-3


@pytest.mark.parametrize("accum", ["plain", "kahan"])
def test_fast_complex_fp16_rows_vs_oracle(cuda, accum):
    """Complex rows stored as FP16 (re, im) pairs with a per-capture scale: same bins and
    FP32 sums as complex64 rows; only the rows' rounding differs."""
    c = _cap("phasor_128", {})
    Hc = oracle.phasor_pulse(c.H, c.wavelength, c.deltaT)
    ref = oracle.bp_gpu_c64(Hc, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT)
    acc = capi.ACCUM_KAHAN if accum == "kahan" else capi.ACCUM_F32
    for checked in (1, 0):
        out, info, viol = run_plan(cuda, Hc, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0,
                                   c.deltaT, algo=capi.ALGO_FAST, h_dtype=capi.DTYPE_C32,
                                   accum=acc, checked=checked)
        assert info["algo"] == "fast" and viol == 0
        assert out.dtype == np.complex64
        assert oracle.rel_l2(out, ref) < 5e-3


def test_fp16_complex_rows_refused_by_exact(cuda):
    c = _cap("phasor_128", {})
    with pytest.raises(capi.BackprojectorError):
        capi.Plan(c.pairs, c.T, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT,
                  algo=capi.ALGO_EXACT, h_dtype=capi.DTYPE_C32)


def test_fast_non_planar_wall_vs_oracle(cuda):
    """SPADs off the wall plane (depth jitter): the general (non-planar) FAST arithmetic."""
    c = _cap("precision_64", {}, seed=9)
    pairs = c.pairs.copy()
    jitter = np.random.default_rng(3).uniform(-0.02, 0.02, len(pairs)).astype(np.float32)
    pairs["camera_point"][:, 1] += jitter
    ref = oracle.bp_gpu_f64(c.H, pairs, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT)
    for checked in (1, 0):
        out, info, viol = run_plan(cuda, c.H, pairs, c.voxels_per_side, c.zero, c.inc, c.t0,
                                   c.deltaT, algo=capi.ALGO_FAST, checked=checked)
        assert info["algo"] == "fast" and viol == 0
        assert oracle.rel_l2(out, ref) < 5e-3


def test_confocal_fast_vs_oracle(cuda):
    c = synthetic.make_capture("precision_64", seed=7, small=True, confocal=True)
    ref = oracle.bp_gpu_f64(c.H, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT)
    out, info, viol = run_plan(cuda, c.H, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0,
                               c.deltaT, algo=capi.ALGO_FAST, checked=1)
    assert info["geometry"] == "confocal" and viol == 0
    assert oracle.rel_l2(out, ref) < 5e-3


@pytest.mark.parametrize("splits", [1, 3, 7])
def test_fast_pair_splits_deterministic(cuda, splits):
    c = _cap("precision_64", {})
    a, ia, _ = run_plan(cuda, c.H, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT,
                        algo=capi.ALGO_FAST, pair_splits=splits)
    b, _, _ = run_plan(cuda, c.H, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT,
                       algo=capi.ALGO_FAST, pair_splits=splits)
    assert ia["pair_splits"] == splits
    assert np.array_equal(a, b)
    ref = oracle.bp_gpu_f64(c.H, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT)
    assert oracle.rel_l2(a, ref) < 5e-3


def test_plans_sharing_a_kernel_stay_launchable(cuda):
    """Plans of one kernel variant with different shared memory footprints, created in
    either order, all launch (the per-kernel limit is only ever raised)."""
    import torch

    caps = [_cap("precision_64", {}), _cap("octree_256", {}), _cap(*CASES[0])]
    plans = [capi.Plan(c.pairs, c.T, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT,
                       algo=capi.ALGO_FAST) for c in caps]
    smem = [p.info()["smem_bytes"] for p in plans]
    assert len(set(smem)) > 1, smem
    for p, c in reversed(list(zip(plans, caps))):
        dH = torch.from_numpy(c.H).to(cuda)
        dV = torch.empty(tuple(int(v) for v in c.voxels_per_side), device=cuda)
        p.execute(dH, dV)
        p.check()
        ref = oracle.bp_gpu_f64(c.H, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT)
        assert oracle.rel_l2(dV.cpu().numpy(), ref) < 5e-3
        p.close()


@pytest.mark.parametrize("tile", list(range(6)))
def test_fast_tile_presets(cuda, tile):
    c = _cap("octree_256", {})
    ref = oracle.bp_gpu_f64(c.H, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT)
    out, info, viol = run_plan(cuda, c.H, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0,
                               c.deltaT, algo=capi.ALGO_FAST, tile=tile, checked=1)
    assert viol == 0
    assert oracle.rel_l2(out, ref) < 5e-3


# ---------------------------------------------------------------- other kernels

def test_phasor_pulse_bit_identical_to_oracle(cuda):
    import torch

    c = _cap("phasor_128", {})
    ref = oracle.phasor_pulse(c.H, c.wavelength, c.deltaT)
    dH = torch.from_numpy(c.H).to(cuda)
    dO = torch.empty(c.H.shape, dtype=torch.complex64, device=cuda)
    capi.phasor_pulse_device(dH, c.P, c.T, c.T, c.wavelength, c.deltaT, dO, c.T)
    torch.cuda.synchronize()
    assert np.array_equal(dO.cpu().numpy(), ref)


def test_pairs_fp64_bit_identical(cuda):
    c = _cap("dense_exhaustive_16", dict(laser_grid=(4, 4), spad_grid=(8, 8), voxels=16))
    got = capi.precompute_pairs(c.laser_position, c.laser_grid, c.camera_position, c.camera_grid)
    ref = oracle.precompute_distances(c.laser_position, c.laser_grid, c.camera_position,
                                      c.camera_grid)
    assert got.tobytes() == ref.tobytes()
    assert got.tobytes() == c.pairs.tobytes()


def test_dropin_host_call_matches_plan(cuda):
    c = _cap("precision_64", {})
    a = capi.backproject_host(c.H, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT,
                              algo=capi.ALGO_EXACT)
    b, _, _ = run_plan(cuda, c.H, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT,
                       algo=capi.ALGO_EXACT)
    assert np.array_equal(a, b)
    # ragged T (not a multiple of 4): the host call pads rows for the TMA path
    H = np.ascontiguousarray(c.H[:, :1021])
    f = capi.backproject_host(H, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT)
    ref = oracle.bp_gpu_f64(H, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT)
    assert oracle.rel_l2(f, ref) < 5e-3


def test_dropin_host_call_reuses_plan_only_for_same_geometry(cuda):
    """The host call keeps its last plan per thread: repeated calls with new transient data
    reuse it, and any change of pairs, grid, t0, deltaT or options builds a new one."""
    c = _cap("precision_64", {})
    args = (c.voxels_per_side, c.zero, c.inc)

    def fresh(H, pairs, t0, dT, **opt):
        return run_plan(cuda, H, pairs, *args, t0, dT, **opt)[0]

    first = capi.backproject_host(c.H, c.pairs, *args, c.t0, c.deltaT)
    assert np.array_equal(first, fresh(c.H, c.pairs, c.t0, c.deltaT))
    H2 = np.ascontiguousarray(c.H[::-1])  # new data, same geometry: cached plan
    again = capi.backproject_host(H2, c.pairs, *args, c.t0, c.deltaT)
    assert np.array_equal(again, fresh(H2, c.pairs, c.t0, c.deltaT))
    moved = c.pairs.copy()
    moved["camera_point"][5, 0] += 0.01
    for pairs, t0, dT, opt in ((moved, c.t0, c.deltaT, {}),
                               (c.pairs, c.t0 + 3 * c.deltaT, c.deltaT, {}),
                               (c.pairs, c.t0, c.deltaT * 1.01, {}),
                               (c.pairs, c.t0, c.deltaT, dict(accum=capi.ACCUM_KAHAN)),
                               (c.pairs, c.t0, c.deltaT, {})):
        got = capi.backproject_host(c.H, pairs, *args, t0, dT, **opt)
        assert np.array_equal(got, fresh(c.H, pairs, t0, dT, **opt))
    grid = (c.voxels_per_side[0], c.voxels_per_side[1], c.voxels_per_side[2] - 4)
    got = capi.backproject_host(c.H, c.pairs, grid, c.zero, c.inc, c.t0, c.deltaT)
    assert np.array_equal(got, run_plan(cuda, c.H, c.pairs, grid, c.zero, c.inc, c.t0,
                                        c.deltaT)[0])


def test_empty_and_out_of_range(cuda):
    c = _cap("precision_64", {})
    empty = capi.backproject_host(np.zeros((0, c.T), np.float32), c.pairs[:0], c.voxels_per_side,
                                  c.zero, c.inc, c.t0, c.deltaT)
    assert np.all(empty == 0)
    # every bin beyond T: the volume is zero on both paths
    for algo in (capi.ALGO_EXACT, capi.ALGO_FAST):
        out = capi.backproject_host(c.H, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0 + 100.0,
                                    c.deltaT, algo=algo)
        assert np.all(out == 0)
    ones = np.ones_like(c.H)
    out = capi.backproject_host(ones, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT,
                                algo=capi.ALGO_EXACT)
    b = oracle.bins(c.pairs, c.T, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT,
                    np.arange(c.nvox), 1)
    # all-ones H: each voxel counts its in-range pairs
    assert np.abs(out.ravel() - (b >= 0).sum(1)).max() <= 2


def test_errors_are_status_codes(cuda):
    c = _cap("precision_64", {})
    bad = c.pairs.copy()
    bad["camera_point"][3, 1] = np.nan
    with pytest.raises(capi.BackprojectorError) as e:
        capi.backproject_host(c.H, bad, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT)
    assert e.value.status == capi.ERR_INVALID_ARGUMENT
    L = capi.lib()
    n = np.asarray(c.voxels_per_side, np.uint32)
    out = np.zeros(c.nvox, np.float32)
    st = L.bpgb_backproject_f32(capi.vptr(c.H), c.H.size - 1, c.T, capi.vptr(c.pairs), c.P,
                                capi.vptr(out), capi.u32ptr(n), capi.fptr(c.zero), capi.fptr(c.inc),
                                c.t0, c.deltaT)
    assert st == capi.ERR_INVALID_ARGUMENT
    with pytest.raises(capi.BackprojectorError) as e:
        capi.backproject_host(c.H, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT,
                              algo=capi.ALGO_EXACT, h_dtype=capi.DTYPE_F16)
    assert e.value.status == capi.ERR_UNSUPPORTED


def test_bounded_wait_reports_timeout(cuda):
    """A wait on a barrier nothing arrives on gives up and reports; the context stays
    usable for the next call."""
    assert capi.lib().bpgb_diag_wait_timeout(64) == capi.ERR_TIMEOUT
    c = _cap("precision_64", {})
    out = capi.backproject_host(c.H, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT)
    assert np.isfinite(out).all()


# ---------------------------------------------------------------- whole reconstructions

def test_nlosbpy_backproject_matches_oracle_pipeline(cuda):
    from backprojector_gb300 import load_nlosbpy

    nl = load_nlosbpy()
    c = _cap("dense_exhaustive_16", dict(laser_grid=(4, 4), spad_grid=(8, 8), voxels=16))
    vol = nl.backproject(c.transient_array(), c.camera_grid, c.laser_grid, c.camera_position,
                         c.laser_position, c.t0, c.deltaT, False, c.volume_position, c.volume_size,
                         c.voxels_per_side, np.zeros(3, np.float32), assume_row_major=True)
    m, M = capi.time_limits(c.laser_position, c.laser_grid, c.camera_position, c.camera_grid,
                            c.volume_position, c.volume_size, c.t0, c.deltaT)
    lo, hi = int(np.floor(m)), int(np.ceil(M))
    chunk = np.zeros((c.P, hi - lo), np.float32)
    s0, s1 = max(lo, 0), min(c.T, hi)
    chunk[:, s0 - lo:s1 - lo] = c.H[:, s0:s1]
    ct0 = np.float32(c.t0) + np.float32(m) * np.float32(c.deltaT)
    ref = oracle.bp_gpu_f64(chunk, c.pairs, c.voxels_per_side, c.zero, c.inc, float(ct0), c.deltaT)
    assert vol.shape == tuple(c.voxels_per_side)
    assert oracle.rel_l2(vol, ref) < 5e-3
    # column-major inputs (the binding's default) are the same arrays with axes reversed
    vol_cm = nl.backproject(c.transient_array().T, c.camera_grid.T, c.laser_grid.T,
                            c.camera_position, c.laser_position, c.t0, c.deltaT, False,
                            c.volume_position, c.volume_size, c.voxels_per_side,
                            np.zeros(3, np.float32))
    assert np.array_equal(vol_cm, vol)
    with pytest.raises(Exception):
        nl.backproject(c.transient_array(), c.camera_grid, c.laser_grid, c.camera_position,
                       c.laser_position, c.t0, c.deltaT, False, c.volume_position, c.volume_size,
                       c.voxels_per_side, np.zeros(3, np.float32), assume_row_major=True,
                       use_cpu=True)


def test_nlosbpy_phasor_matches_oracle_pipeline(cuda):
    from backprojector_gb300 import load_nlosbpy

    nl = load_nlosbpy()
    c = _cap("phasor_128", {})
    vol = nl.phasor(c.transient_array(), c.camera_grid, c.laser_grid, c.camera_position,
                    c.laser_position, c.t0, c.deltaT, False, c.volume_position, c.volume_size,
                    c.voxels_per_side, c.wavelength, assume_row_major=True)
    m, M = capi.time_limits(c.laser_position, c.laser_grid, c.camera_position, c.camera_grid,
                            c.volume_position, c.volume_size, c.t0, c.deltaT)
    lo, hi = int(m), int(M)
    chunk = np.zeros((c.P, hi - lo), np.float32)
    s0, s1 = max(lo, 0), min(c.T, hi)
    chunk[:, s0 - lo:s1 - lo] = c.H[:, s0:s1]
    Hc = oracle.phasor_pulse(chunk, c.wavelength, c.deltaT)
    ct0 = np.float32(c.t0) + np.float32(lo) * np.float32(c.deltaT)
    ref = oracle.bp_gpu_c64(Hc, c.pairs, c.voxels_per_side, c.zero, c.inc, float(ct0), c.deltaT)
    assert vol.dtype == np.complex64
    assert oracle.rel_l2(vol, ref) < 5e-3


def test_reference_kernel_speed_on_256_capture(cuda):
    """The reference's own kernel (built from its sources, its launcher's policy) against
    the FAST plan on the 256^3 capture, on the same GPU; prints both rates."""
    import torch

    if not oracle.REF_LIB.exists():
        pytest.skip("reference kernel not built (reference sources absent at build time)")
    c = synthetic.make_capture("octree_256", seed=0)
    _, block, ref_ms = oracle.reference_gpu(c.H, c.pairs, c.voxels_per_side, c.zero, c.inc,
                                            c.t0, c.deltaT)
    dH = torch.from_numpy(c.H).to(cuda)
    dV = torch.empty(tuple(int(v) for v in c.voxels_per_side), device=cuda)
    with capi.Plan(c.pairs, c.T, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT,
                   algo=capi.ALGO_FAST) as p:
        p.execute(dH, dV)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(3):
            p.execute(dH, dV)
        e1.record()
        e1.synchronize()
        ms = e0.elapsed_time(e1) / 3
    print(f"\n[octree_256 dense] reference kernel (block {block}) {ref_ms:.1f} ms = "
          f"{c.updates / ref_ms * 1e3:.3e} updates/s; FAST {ms:.2f} ms = "
          f"{c.updates / ms * 1e3:.3e} updates/s; ratio {ref_ms / ms:.1f}")
    assert ms * 10 < ref_ms


def test_device_crop_reproduces_capture_call(cuda):
    """A device-resident capture cropped on the GPU (bpgb_capture_window + bpgb_rows_crop)
    and backprojected by a plan equals bpgb_backproject_capture (which crops while copying
    from the host) bit for bit."""
    import torch

    from backprojector_gb300 import load_nlosbpy

    nl = load_nlosbpy()
    c = _cap("dense_exhaustive_16", dict(laser_grid=(4, 4), spad_grid=(8, 8), voxels=16))
    ref = nl.backproject(c.transient_array(), c.camera_grid, c.laser_grid, c.camera_position,
                         c.laser_position, c.t0, c.deltaT, False, c.volume_position, c.volume_size,
                         c.voxels_per_side, np.zeros(3, np.float32), assume_row_major=True)
    fr, ln, ct = capi.capture_window(c.camera_grid, c.laser_grid, c.camera_position,
                                     c.laser_position, c.t0, c.deltaT, False, c.volume_position,
                                     c.volume_size, t0_mode=0)
    pitch = (ln + 3) // 4 * 4
    dH = torch.from_numpy(c.H).to(cuda)
    crop = torch.full((c.P, pitch), float("nan"), device=cuda)
    capi.rows_crop(dH, c.P, c.T, c.T, fr, ln, crop, pitch)
    dV = torch.empty(tuple(int(v) for v in c.voxels_per_side), device=cuda)
    pairs = capi.precompute_pairs(c.laser_position, c.laser_grid, c.camera_position,
                                  c.camera_grid)  # the capture call's FP64 pair list
    with capi.Plan(pairs, ln, c.voxels_per_side, c.zero, c.inc, ct, c.deltaT,
                   h_pitch=pitch) as p:
        p.execute(crop, dV)
        p.check()
    assert np.array_equal(dV.cpu().numpy(), ref)
    host = crop.cpu().numpy()
    lo, hi = max(fr, 0), min(c.T, fr + ln)
    assert np.array_equal(host[:, lo - fr:hi - fr], c.H[:, lo:hi])
    assert np.all(host[:, ln:] == 0) and np.all(host[:, :lo - fr] == 0)
