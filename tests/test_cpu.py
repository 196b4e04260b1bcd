"""CPU tests (no GPU): the oracle against the reference kernel's golden outputs and known
answers, the host-side helpers of the C ABI, and the library's exported symbols."""
from __future__ import annotations

import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from backprojector_gb300 import capi, synthetic
from oracle import oracle

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        txt = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(bpgb_[a-z0-9_]+)\s*\(", txt))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    L = capi.lib()
    names = declared_symbols()
    assert len(names) >= 20
    for n in names:
        assert hasattr(L, n), n
        assert n in capi.SIGNATURES, f"{n} has no ctypes signature"


def test_library_exports_reference_cpp_entry_points():
    out = subprocess.run(["nm", "-DC", "--defined-only", str(capi.LIB_PATH)], capture_output=True,
                         text=True).stdout
    for fn in ("call_cuda_backprojection(", "call_cuda_complex_backprojection(",
               "call_cuda_octree_backprojection("):
        assert fn in out, fn


def test_cnn_line_planes_sizes_and_shape_checks():
    """Host arithmetic of the tensor-core CNN entry points (no GPU needed): line-planes
    tensor bytes = (batch (n0+2)(n1+2) + 16 tail lines) x planes x (32 + 2 zpad) rows x
    16 B; weight images 9 (two-plane input) or 5 (one plane, taps paired) groups of
    1536 B; volumes that are not 32-voxel z-lines or whose n1 is not a multiple of 8 are
    refused (0 bytes)."""
    assert capi.cnn_lp_bytes(16, 0, (32, 32, 32), 16) == (16 * 34 * 34 + 16) * 2 * 32 * 16
    assert capi.cnn_lp_bytes(1, 1, (32, 32, 32), 16) == (16 * 34 * 34 + 16) * 1 * 34 * 16
    assert capi.cnn_lp_bytes(2, 0, (3, 8, 32), 2) == (2 * 5 * 10 + 16) * 1 * 32 * 16
    assert capi.cnn_lp_bytes(16, 0, (32, 32, 16), 1) == 0  # z-lines must be 32 voxels
    assert capi.cnn_lp_bytes(16, 0, (32, 12, 32), 1) == 0  # n1 % 8 != 0
    assert capi.cnn_lp_bytes(17, 0, (32, 32, 32), 1) == 0  # at most 16 channels
    assert capi.cnn_lp_bytes(16, 2, (32, 32, 32), 1) == 0  # zpad 0 or 1
    assert capi.cnn_tc_weight_bytes(16) == 9 * 1536 and capi.cnn_tc_weight_bytes(9) == 9 * 1536
    assert capi.cnn_tc_weight_bytes(2) == 5 * 1536 and capi.cnn_tc_weight_bytes(1) == 5 * 1536
    assert capi.cnn_tc_weight_bytes(0) == 0 and capi.cnn_tc_weight_bytes(17) == 0
    with pytest.raises(capi.BackprojectorError):  # null tensors: refused before any launch
        capi.cnn_tc_conv3d(None, 16, 0, (32, 32, 32), 1, None, None, 16, True, d_Y=None)


def test_abi_version_and_status_strings():
    L = capi.lib()
    assert L.bpgb_abi_version() == capi.ABI_VERSION == 2
    assert L.bpgb_status_string(capi.ERR_TIMEOUT) == b"device wait timed out"
    o = capi.options()
    assert o.algo == capi.ALGO_AUTO and o.h_scale == 1.0 and o.tile == -1


def test_options_mirror_matches_the_c_struct():
    """bpgb_options_default writes exactly the mirrored bytes: a sentinel right after the
    ctypes Options stays untouched, and the defaults land in the named fields."""
    import ctypes as C

    class Guarded(C.Structure):
        _fields_ = [("o", capi.Options), ("guard", C.c_uint8 * 64)]

    g = Guarded()
    C.memset(C.byref(g), 0xAB, C.sizeof(g))
    capi.lib().bpgb_options_default(C.byref(g.o))
    assert bytes(g.guard) == b"\xab" * 64
    assert g.o.unfactored == 0 and list(g.o.reserved) == [0, 0, 0, 0]
    assert g.o.h_dtype == capi.DTYPE_F32 and g.o.accum == capi.ACCUM_F32
    assert C.sizeof(capi.Options) == 16 * 4


def test_volume_basis_axis_aligned_and_wall_normal():
    zero, inc = capi.volume_basis((0, 1, 0), (1, 2, 3), (11, 21, 31))
    assert np.allclose(zero, [-0.5, 0.0, -1.5])
    assert np.allclose(inc.reshape(3, 3), np.diag([0.1, 0.1, 0.1]))
    # wall_normal (0,-1,0): y = -n = (0,1,0), x = y cross z = (1,0,0), z = y cross x = (0,0,-1)
    zero, inc = capi.volume_basis((0, 1, 0), (1, 1, 1), (3, 3, 3), (0, -1, 0))
    assert np.allclose(inc.reshape(3, 3), [[0.5, 0, 0], [0, 0.5, 0], [0, 0, -0.5]])
    with pytest.raises(capi.BackprojectorError):
        capi.volume_basis((0, 1, 0), (1, 1, 1), (1, 3, 3))


def test_phasor_taps_match_oracle_bit_for_bit():
    for wl, dT in ((0.063, 0.0005), (0.04, 0.001), (0.005, 0.0003)):
        a = capi.phasor_taps(wl, dT)
        b = oracle.phasor_taps(wl, dT)
        assert a.shape == b.shape and np.array_equal(a, b)
    assert capi.phasor_taps(0.063, 0.0005).shape[1] == int(np.float32(4) * np.float32(0.063) / np.float32(0.0005))


def test_time_limits_bracket_every_path():
    c = synthetic.make_capture("dense_exhaustive_16", seed=2, small=True, render=False)
    m, M = capi.time_limits(c.laser_position, c.laser_grid, c.camera_position, c.camera_grid,
                            c.volume_position, c.volume_size, c.t0, c.deltaT)
    b = oracle.bins(c.pairs, 10**7, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT,
                    np.arange(0, c.nvox, 7), 0)
    assert m < b[b >= 0].min() and M > b.max()


def test_synthetic_render_deterministic_and_matches_paths():
    a = synthetic.make_capture("precision_64", seed=4, small=True)
    b = synthetic.make_capture("precision_64", seed=4, small=True)
    assert np.array_equal(a.H, b.H)
    # pair list from numpy equals the oracle's restatement of precompute_distances
    ref = oracle.precompute_distances(a.laser_position, a.laser_grid, a.camera_position, a.camera_grid)
    assert ref.tobytes() == a.pairs.tobytes()
    # Poisson counts are integers and scaled to the requested peak
    assert np.all(a.H == np.round(a.H)) and abs(a.H.max() - 1e4) < 500


def test_oracle_known_answers():
    # single pair, delta transient at bin b: voxels whose FP64 bin is b light up
    c = synthetic.make_capture("precision_64", seed=5, small=True, spad_grid=(2, 2), render=False)
    pairs = c.pairs[:1]
    bins = oracle.bins(pairs, c.T, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT,
                       np.arange(c.nvox), 0)[:, 0]
    b0 = int(np.median(bins[bins >= 0]))
    H = np.zeros((1, c.T), np.float32)
    H[0, b0] = 1.0
    vol = oracle.bp_gpu_f64(H, pairs, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT)
    assert np.array_equal(vol.ravel() == 1.0, bins == b0) and (bins == b0).any()
    # linearity and pair-permutation invariance
    c = synthetic.make_capture("precision_64", seed=6, small=True, spad_grid=(6, 6))
    args = (c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT)
    v1 = oracle.bp_gpu_f64(c.H, c.pairs, *args)
    v2 = oracle.bp_gpu_f64(2 * c.H, c.pairs, *args)
    assert np.allclose(v2, 2 * v1)
    perm = np.random.default_rng(0).permutation(c.P)
    v3 = oracle.bp_gpu_f64(c.H[perm], c.pairs[perm], *args)
    assert np.allclose(v3, v1, rtol=1e-12)
    # a single point scatterer: the argmax sits next to the scatterer's voxel
    c = synthetic.make_capture("precision_64", seed=8, small=True, spad_grid=(16, 16), voxels=24,
                               render=False)
    q = (c.zero + c.inc.reshape(3, 3).T @ np.array([12.0, 9.0, 14.0])).astype(np.float32)
    H = capi.synth_render(c.pairs, c.T, c.t0, c.deltaT, q[None, :], np.ones(1, np.float32))
    H = (H > 0).astype(np.float32)
    vol = oracle.bp_gpu_f64(H, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT)
    am = np.array(np.unravel_index(np.argmax(vol), vol.shape))
    assert np.abs(am - np.array([12, 9, 14])).max() <= 1


def test_reference_cursor_emulation():
    assert oracle.reference_visited((32, 32, 32)).all()
    assert oracle.reference_visited((16, 8, 5)).all()
    # sizes that are not multiples of 16 wrap the cursor (some voxels are computed twice);
    # every voxel is still written once at least
    for n in (17, 20, 40, (20, 30, 40)):
        assert oracle.reference_visited((n, n, n) if isinstance(n, int) else n).all()


def test_classic_cpu_path_runs_and_is_close_to_gpu_semantics():
    c = synthetic.make_capture("precision_64", seed=9, small=True)
    v = oracle.classic(c.H, c.pairs, c.voxels_per_side, c.volume_position, c.volume_size, c.t0,
                       c.deltaT)
    assert v.shape == tuple(c.voxels_per_side) and np.isfinite(v).all() and v.max() > 0


def golden_files():
    return sorted(GOLDEN.glob("*.npz"))


@pytest.mark.skipif(not golden_files(), reason="golden fixtures not generated")
def test_oracle_pinned_to_reference_kernel_outputs():
    """FP64 oracle and FP32 emulation against the reference kernel's own outputs."""
    for f in golden_files():
        z = np.load(f)
        pairs = np.ascontiguousarray(z["pairs"]).view(capi.PAIR_DTYPE).reshape(-1)
        if str(z["H_kind"]) == "ramp" if "H_kind" in z.files else False:
            T = int(z["T"])
            H = np.broadcast_to(np.arange(1, T + 1, dtype=np.float32), (len(pairs), T)).copy()
        else:
            H = z["H"]
        args = (z["N"], z["zero"], z["inc"], float(z["t0"]), float(z["dT"]))
        ref = z["ref_volume"]
        block = int(z["ref_block"])
        mask = oracle.reference_visited(z["N"])
        if np.iscomplexobj(H):
            o64 = oracle.bp_gpu_c64(H, pairs, *args, ref_block=block)
            assert oracle.rel_l2(o64[mask], ref[mask]) < 2e-2, f.name
            continue
        emu = oracle.bp_gpu_f32emu(H, pairs, *args, ref_block=block)
        o64 = oracle.bp_gpu_f64(H, pairs, *args, ref_block=block)
        if np.all(H == np.round(H)):
            # integer rows: sums are exact, so a voxel differs only where one of its
            # updates is binned differently (norm3df vs the correctly rounded norm next
            # to a .5 boundary): at most 0.1% of voxels
            assert np.mean(emu[mask] != ref[mask]) <= 1e-3, f.name
        else:
            assert oracle.rel_l2(emu[mask], ref[mask]) < 1e-4, f.name
        assert oracle.rel_l2(o64[mask], ref[mask]) < 2e-2, f.name
        assert np.all(ref[~mask] == 0), f.name


def test_tune_cache_file_round_trip(tmp_path):
    """The autotuner's cache file: load merges entries, save writes them back, bad lines
    are rejected with the line number (no device needed)."""
    capi.tune_cache_clear()
    src = tmp_path / "tune.txt"
    src.write_text("plan/GB300/sm152/dt0/acc0/P16384/T4096/n256x256x256 3 16 4 0 88.5\n"
                   "batch/GB300/sm152/dt1/n64/shapeabc 1 32 3 0 140.25\n")
    capi.tune_cache_load(src)
    assert capi.tune_cache_size() == 2
    out = tmp_path / "saved.txt"
    capi.tune_cache_save(out)
    lines = sorted(out.read_text().split("\n")[:-1])
    assert lines == sorted(src.read_text().split("\n")[:-1])
    capi.tune_cache_load(tmp_path / "missing.txt")  # no file yet: not an error
    bad = tmp_path / "bad.txt"
    bad.write_text("key 99 16 4 0 1.0\n")
    with pytest.raises(capi.BackprojectorError) as e:
        capi.tune_cache_load(bad)
    assert e.value.status == capi.ERR_INVALID_ARGUMENT and ":1:" in str(e.value)
    assert capi.tune_cache_size() == 2
    capi.tune_cache_clear()
    assert capi.tune_cache_size() == 0


def test_native_octree_weights_file_errors(tmp_path):
    """bpgb_octree_create reads its weights with the library's own .npz reader: missing,
    malformed, compressed and mis-shaped files are rejected before any device work."""
    c = synthetic.make_capture("octree_256", small=True, render=False)
    args = (c.pairs, c.T, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT)
    cases = {"missing.npz": "cannot open"}
    (tmp_path / "junk.npz").write_bytes(b"not a zip archive at all, just some bytes")
    cases["junk.npz"] = "end-of-directory"
    np.savez_compressed(tmp_path / "packed.npz", w0=np.zeros((32, 16), np.float32))
    cases["packed.npz"] = "compressed"
    np.savez(tmp_path / "shape.npz", w0=np.zeros((3, 3), np.float32), in_channels=np.int64(2),
             p_lo=np.float64(0.1))
    for name, msg in cases.items():
        with pytest.raises(capi.BackprojectorError) as e:
            capi.NativeOctree(*args, tmp_path / name)
        assert e.value.status == capi.ERR_INVALID_ARGUMENT and msg in str(e.value), str(e.value)
    # a well-formed file gets past the reader (then needs a device for its plans)
    with pytest.raises(capi.BackprojectorError) as e:
        capi.NativeOctree(*args, tmp_path / "shape.npz")
    assert "cannot open" not in str(e.value) and "zip" not in str(e.value)


def _cli():
    from backprojector_gb300 import build

    return str(build.CLI_PATH)


def write_dataset(path, c, **override):
    """A capture in the command-line tool's .npz layout."""
    arrays = dict(data=c.transient_array(), camera_grid_positions=c.camera_grid,
                  laser_grid_positions=c.laser_grid, camera_position=c.camera_position,
                  laser_position=c.laser_position, t0=np.float32(c.t0),
                  deltat=np.float32(c.deltaT), is_confocal=np.int64(1 if c.spec.confocal else 0),
                  hidden_volume_position=c.volume_position, hidden_volume_size=c.volume_size)
    arrays.update(override)
    arrays = {k: v for k, v in arrays.items() if v is not None}
    np.savez(path, **arrays)


def test_cli_arguments_and_dataset_checks(tmp_path):
    """bpgb_backprojector rejects bad flags and malformed datasets before touching a GPU."""
    def run(*args):
        return subprocess.run([_cli(), *map(str, args)], capture_output=True, text=True)

    r = run("--help")
    assert r.returncode == 0 and "usage: bpgb_backprojector" in r.stderr
    assert run().returncode == 2
    assert run("x.npz", "--bogus").returncode == 2
    r = run("x.npz", "--cpu")
    assert r.returncode == 1 and "no CPU path" in r.stderr
    r = run(tmp_path / "missing.npz")
    assert r.returncode == 1 and "cannot open" in r.stderr
    c = synthetic.make_capture("dense_exhaustive_16", small=True, render=False)
    write_dataset(tmp_path / "no_t0.npz", c, t0=None)
    r = run(tmp_path / "no_t0.npz")
    assert r.returncode == 1 and "missing array 't0'" in r.stderr
    write_dataset(tmp_path / "shape.npz", c, data=np.zeros((2, 2, 2), np.float32))
    r = run(tmp_path / "shape.npz")
    assert r.returncode == 1 and "data must be" in r.stderr
    write_dataset(tmp_path / "bounce.npz", c, data=np.zeros((*c.transient_array().shape[:4], 2, c.T),
                                                              np.float32))
    r = run(tmp_path / "bounce.npz")
    assert r.returncode == 1 and "bounce" in r.stderr
    r = run(tmp_path / "shape.npz", "--octree")
    assert r.returncode == 1


def test_capture_window_matches_time_limits():
    c = synthetic.make_capture("dense_exhaustive_16", small=True, render=False)
    m, M = capi.time_limits(c.laser_position, c.laser_grid, c.camera_position, c.camera_grid,
                            c.volume_position, c.volume_size, c.t0, c.deltaT)
    args = (c.camera_grid, c.laser_grid, c.camera_position, c.laser_position, c.t0, c.deltaT,
            False, c.volume_position, c.volume_size)
    fr, ln, ct = capi.capture_window(*args, t0_mode=0)
    assert fr == int(np.floor(m)) and ln == int(np.ceil(M)) - int(np.floor(m))
    assert ct == float(np.float32(c.t0) + np.float32(m) * np.float32(c.deltaT))
    fr1, ln1, ct1 = capi.capture_window(*args, t0_mode=1)
    assert (fr1, ln1) == (fr, ln)
    assert ct1 == float(np.float32(c.t0) + np.float32(fr) * np.float32(c.deltaT))
    fr2, ln2, _ = capi.capture_window(*args, t0_mode=2)
    assert fr2 == int(m) and ln2 == int(M) - int(m)
    with pytest.raises(capi.BackprojectorError):
        capi.capture_window(*args, t0_mode=3)
    # + 4: the reference's corner bound
    mc, Mc = capi.time_limits(c.laser_position, c.laser_grid, c.camera_position, c.camera_grid,
                              c.volume_position, c.volume_size, c.t0, c.deltaT, corners=True)
    fr4, ln4, ct4 = capi.capture_window(*args, t0_mode=4)
    assert fr4 == int(np.floor(mc)) and ln4 == int(np.ceil(Mc)) - int(np.floor(mc))
    assert ct4 == float(np.float32(c.t0) + np.float32(mc) * np.float32(c.deltaT))


@pytest.mark.parametrize("name", ["dense_exhaustive_16", "precision_64", "octree_256", "phasor_128"])
def test_time_limits_corners_match_oracle(name):
    """bpgb_time_limits_corners restates get_time_limits (backproject.hpp:617-674) with its
    corner semantics; the oracle's restatement gives the same floats."""
    for small in (True, False):
        c = synthetic.make_capture(name, small=small, render=False)
        args = (c.laser_position, c.laser_grid, c.camera_position, c.camera_grid,
                c.volume_position, c.volume_size, c.t0, c.deltaT)
        got = capi.time_limits(*args, corners=True)
        want = oracle.time_limits_corners(*args)
        assert np.float32(got[0]) == np.float32(want[0]) and np.float32(got[1]) == np.float32(want[1])
        # the bound over every grid point and the volume box is never looser on the low side
        # by more than the grids' corner geometry allows: both cover [t0-relative min, max]
        m, M = capi.time_limits(*args)
        assert m < M and got[0] < got[1]


def _max_worker(rank, world, port, q):
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        q.put((rank, bench.max_over_ranks(1.5 + rank, "cpu")))
    finally:
        dist.destroy_process_group()


def test_bench_max_over_ranks_gloo():
    """Replica runs time every rank and report the slowest (2 gloo ranks on the CPU)."""
    import socket

    import torch.multiprocessing as mp

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_max_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got == [(0, 2.5), (1, 2.5)]
    import bench

    assert bench.max_over_ranks(3.0, "cpu") == 3.0  # no process group: the value itself


def test_bench_reference_arm_two_ranks():
    """--impl reference under torchrun with 2 ranks: rank 0 alone runs and prints one JSON
    line, rank 1 exits 0 without work."""
    import json
    import socket
    import sys

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    root = Path(__file__).resolve().parents[1]
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
                        "--nproc-per-node", "2", "--master-addr", "127.0.0.1", "--master-port",
                        str(port), str(root / "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "1", "--workload", "dense_exhaustive_16",
                        "--ref-sample", "8"], capture_output=True, text=True, timeout=600,
                       cwd=root)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0


@pytest.mark.parametrize("name", ["dense_exhaustive_16", "precision_64", "octree_256"])
def test_oracle_synth_backend_matches_product(name):
    """The bench's reference arm builds its captures with oracle.SynthBackend (no product
    library); they must equal the product backend's bit for bit (basis, rows, noise)."""
    from backprojector_gb300 import synthetic

    a = synthetic.make_capture(name, seed=13, small=True)
    b = synthetic.make_capture(name, seed=13, small=True, backend=oracle.SynthBackend)
    assert a.H.tobytes() == b.H.tobytes()
    assert a.zero.tobytes() == b.zero.tobytes() and a.inc.tobytes() == b.inc.tobytes()
    assert a.pairs.tobytes() == b.pairs.tobytes() and a.t0 == b.t0
