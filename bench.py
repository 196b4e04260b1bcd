"""Benchmark: voxel-pair updates/s of the dense backprojection on one GB300.

Workload (default): the learned-octree target capture at its dense form -- one laser,
128 x 128 SPADs on a 2 x 2 m wall, T = 4096 bins (deltaT 1.5 mm), 256^3 voxels over a
1.5 m cube; P = 16384 pairs, 2.75e11 voxel-pair updates per reconstruction.  One step =
one full reconstruction of a seeded synthetic capture (see backprojector_gb300/synthetic.py).

JSON line keys beyond the contract's: roofline (the FAST kernel against the GB300's
reciprocal-square-root issue rate, one MUFU op per update), cpu_baseline (the
reference's OpenMP CPU path restated in C, timed on a bounded voxel sample on the host
cores), e2e (the drop-in host-buffer C ABI call, host<->device copies included).
The reference's own GPU kernel, built from its sources, is timed on the same GPU by
tests/test_gpu_parity.py::test_reference_kernel_speed_on_256_capture.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOADS = {
    "octree_256": "dense, 1 laser x 128x128 SPADs, T=4096, dT=1.5mm, 256^3 over a 1.5 m cube",
    "precision_64": "dense, 1 laser x 64x64 SPADs, T=2048, dT=1mm, 64^3 over a 1 m cube",
    "dense_exhaustive_16": "dense, 16x16 lasers x 16x16 SPADs, T=512, dT=3mm, 32^3 over 0.5 m",
    "phasor_128": "phasor complex64, 1 laser x 128x128 SPADs, T=4096, dT=0.5mm, 128^3 over 1.5 m",
    "octree_256_learned": "learned octree on the octree_256 capture shape: 32^3 coarse pass, "
                          "BF16 tensor-core occupancy CNN, trilinear fill, block-sparse 8^3 "
                          "fine pass; FP16 rows; dense-equivalent updates/s (V x P / time)",
    "batch_64": "64 uneven captures in one persistent launch replayed from a CUDA graph: SPAD "
                "grids {16,32,48,64,96}^2 (1 laser, or 16^2 x 16^2 exhaustive for a quarter), "
                "T {512,1024,2048}, volumes {32,48,64,96}^3, 4-40 scatterers, FP16 rows with a "
                "per-capture scale, FP32 accumulate",
}
MUFU_PER_SM_PER_CLK = 16  # reciprocal square root throughput of one SM (Blackwell SFU)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x: float, device) -> float:
    """The largest x over the ranks of the initialised process group (x itself without
    one): the step time of a replica run is its slowest rank's."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi samples during the timed region."""

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.samples = []
        self.proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 8:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.15)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=2)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[4 + i] == "Active"})
        pw = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "power_w_max": max(pw) if pw else None, "samples": len(self.samples)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return json.loads(p.read_text())
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


def cpu_baseline(cap, sample_voxels: int, seed: int = 0):
    """The reference's OpenMP CPU path (classic_backprojection, backproject.hpp:138-216,
    restated in oracle/oracle.c) on a seeded voxel sample, all host threads."""
    from oracle import oracle

    rng = np.random.default_rng(seed)
    ids = rng.choice(cap.nvox, size=min(sample_voxels, cap.nvox), replace=False)
    t = time.perf_counter()
    oracle.classic(cap.H, cap.pairs, cap.voxels_per_side, cap.volume_position, cap.volume_size,
                   cap.t0, cap.deltaT, voxels=ids)
    dt = time.perf_counter() - t
    return len(ids) * cap.P / dt, dt, len(ids), oracle.num_threads()


def cpu_sample_for(rate: float, pairs: int, seconds: float, lo: int, hi: int) -> int:
    """Voxels a CPU sample needs to last about `seconds` at `rate` updates/s."""
    return int(min(hi, max(lo, seconds * rate / max(pairs, 1))))


def cpu_baseline_timed(cap, seconds: float, probe: int, seed: int = 0):
    """cpu_baseline on a sample sized to about `seconds` of CPU work (a `probe`-voxel run
    calibrates the rate first)."""
    r, dt, n, cores = cpu_baseline(cap, probe, seed)
    want = cpu_sample_for(r, cap.P, seconds, probe, cap.nvox)
    if want > n:
        r, dt, n, cores = cpu_baseline(cap, want, seed)
    return r, dt, n, cores


def run_reference_arm(args):
    """--impl reference: the reference's CPU implementation of the path on host cores."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from backprojector_gb300 import synthetic
    from oracle import oracle

    if args.workload == "batch_64":
        return run_reference_arm_batch(args)
    name = "octree_256" if args.workload == "octree_256_learned" else args.workload
    # inputs built without the product library (oracle.SynthBackend: the same captures)
    cap = synthetic.make_capture(name, seed=args.seed, backend=oracle.SynthBackend)
    # each step: a seeded voxel sample sized (during warm-up) to about --ref-seconds
    sample = args.ref_sample
    for _ in range(args.warmup):
        r, _, _, _ = cpu_baseline(cap, sample, seed=1)
        sample = cpu_sample_for(r, cap.P, args.ref_seconds, args.ref_sample, cap.nvox)
    secs = []
    cores = None
    for k in range(args.steps):
        r, dt, n, cores = cpu_baseline(cap, sample, seed=100 + k)
        secs.append(dt)
    value = float(sample * cap.P * args.steps / np.sum(secs))
    args.ref_sample = sample
    line = {
        "impl": "reference", "metric": "voxel-pair updates/s", "value": value, "unit": "updates/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": float(np.mean(secs) * 1e3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{args.workload}: {WORKLOADS[args.workload]}",
                   "sample": f"{args.ref_sample} seeded random voxels x all {cap.P} pairs per step"},
        "cpu_baseline": {"value": value, "unit": "updates/s", "cores": cores, "kind": "port",
                         "sample": f"{args.ref_sample} voxels x {cap.P} pairs per step; "
                                   "classic_backprojection restated in C (OpenMP)"},
        "e2e": {"value": value, "unit": "updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_reference_arm_batch(args):
    """--impl reference on batch_64: each step reconstructs a seeded voxel sample of every
    capture of the batch with the reference's CPU path."""
    from backprojector_gb300 import synthetic
    from oracle import oracle

    caps = synthetic.make_batch(64, seed=args.seed, backend=oracle.SynthBackend)
    per = max(1, args.ref_sample // 4)
    for _ in range(args.warmup):
        r, _, _, _ = cpu_baseline_batch(caps, per, seed=1)
        per = cpu_sample_for(r, sum(c.P for c in caps), args.ref_seconds,
                             max(1, args.ref_sample // 4), min(c.nvox for c in caps))
    upd, secs, cores = 0.0, [], None
    for k in range(args.steps):
        r, dt, _, cores = cpu_baseline_batch(caps, per, seed=100 + k)
        upd += r * dt
        secs.append(dt)
    value = float(upd / np.sum(secs))
    sample = (f"{per} seeded random voxels of each of the 64 captures x all their pairs per "
              "step; classic_backprojection restated in C (OpenMP)")
    line = {
        "impl": "reference", "metric": "voxel-pair updates/s", "value": value, "unit": "updates/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": float(np.mean(secs) * 1e3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"batch_64: {WORKLOADS['batch_64']}", "sample": sample},
        "cpu_baseline": {"value": value, "unit": "updates/s", "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import ctypes as C

    import torch

    from backprojector_gb300 import capi, synthetic

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    over = {"voxels": args.voxels} if args.voxels else {}
    cap = synthetic.make_capture(args.workload, seed=args.seed + rank, **over)
    phasor = args.workload == "phasor_128"
    N = tuple(int(v) for v in cap.voxels_per_side)
    stream = torch.cuda.Stream(device=dev)
    opt = dict(algo=capi.ALGO_FAST if args.algo == "fast" else capi.ALGO_EXACT)
    if args.dtype == "f16":
        opt["h_dtype"] = capi.DTYPE_F16
    if args.kahan:
        opt["accum"] = capi.ACCUM_KAHAN
    if args.tile is not None:
        opt["tile"] = args.tile
    prep = None  # per-step work ahead of the backprojection (the phasor pulse)
    if phasor:
        # A step is the whole phasor-field reconstruction of resident raw rows: the pulse
        # convolution (bpgb_phasor_pulse), for FP16 (re, im) rows the device-scaled
        # conversion, the complex backprojection, and the scale back.
        Hraw = torch.from_numpy(cap.H).to(dev)
        Hc = torch.empty(cap.H.shape, dtype=torch.complex64, device=dev)
        dH = Hc
        opt["h_dtype"] = capi.DTYPE_C64
        dV = torch.empty(N, dtype=torch.complex64, device=dev)
        amax = torch.ones(1, dtype=torch.float32, device=dev)
        if args.dtype == "f16":
            dH = torch.empty((cap.P, cap.T, 2), dtype=torch.float16, device=dev)
            opt["h_dtype"] = capi.DTYPE_C32

        def prep(st):
            capi.phasor_pulse_device(Hraw, cap.P, cap.T, cap.T, cap.wavelength, cap.deltaT, Hc,
                                     cap.T, stream=st)
            if args.dtype == "f16":
                capi.rows_absmax(Hc, cap.P, 2 * cap.T, 2 * cap.T, amax, st)
                capi.rows_to_half(Hc, cap.P, 2 * cap.T, 2 * cap.T, capi.DTYPE_F16, dH, 2 * cap.T,
                                  d_absmax=amax, target=16384.0, stream=st)

        def post(st):
            if args.dtype == "f16":
                capi.volume_scale(dV, 2 * cap.nvox, d_absmax=amax, target=16384.0, stream=st)

        prep(stream)
        stream.synchronize()
    else:
        dH = torch.from_numpy(cap.H).to(dev)
        scale = 1.0
        if args.dtype == "f16":
            scale = float(cap.H.max()) / 1024.0 or 1.0
            dH = (dH / scale).half()
            opt["h_scale"] = scale
        dV = torch.empty(N, dtype=torch.float32, device=dev)
        post = None
    tune_rep = None
    if not args.no_tune and args.tile is None and args.algo == "fast":
        t = time.perf_counter()
        tuned, tune_rep = capi.autotune_plan(cap.pairs, cap.T, N, cap.zero, cap.inc, cap.t0,
                                             cap.deltaT, dH, dV, **opt)
        tune_rep["seconds"] = time.perf_counter() - t
        opt.update(tuned)
    # Gate: the bounds-checked kernel variant must see every bin inside its staged window
    # before the unchecked variant runs.
    with capi.Plan(cap.pairs, cap.T, N, cap.zero, cap.inc, cap.t0, cap.deltaT, checked=1,
                   **opt) as gate:
        gate.execute(dH, dV)
        if gate.check() != 0:
            raise RuntimeError("window check failed: bins outside the staged windows")
    plan = capi.Plan(cap.pairs, cap.T, N, cap.zero, cap.inc, cap.t0, cap.deltaT, **opt)
    info = plan.info()
    # events around the backprojection of every step (the kernel the roofline is about)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]

    def step(k=None):
        if prep is not None:
            prep(stream)
        if k is not None:
            evs[k][0].record(stream)
        plan.execute(dH, dV, stream)
        if k is not None:
            evs[k][1].record(stream)
        if post is not None:
            post(stream)

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step()
    stream.synchronize()
    plan.check()
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    launches0 = capi.launch_count()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record(stream)
        for k in range(args.steps):
            step(k)
        e1.record(stream)
        e1.synchronize()
    torch.cuda.synchronize()
    launches = capi.launch_count() - launches0
    ms = e0.elapsed_time(e1) / args.steps
    bp_ms = float(np.mean([a.elapsed_time(b) for a, b in evs]))
    plan.check()
    ms = max_over_ranks(ms, dev)
    updates = cap.updates
    value = updates * ws / (ms * 1e-3)

    # e2e: the reference-facing calls on host buffers, copies inside the timed region
    e2e = None
    variants = {}
    L = capi.lib()
    n = np.asarray(N, np.uint32)
    if not phasor and args.dtype == "f32":
        o = capi.options(**{k: v for k, v in opt.items() if k != "h_scale"})

        def host_call(H, V):
            st = L.bpgb_backproject_host(C.c_void_p(H.ctypes.data if isinstance(H, np.ndarray)
                                                    else H.data_ptr()), cap.P * cap.T, cap.T,
                                         capi.vptr(cap.pairs), cap.P,
                                         C.c_void_p(V.ctypes.data if isinstance(V, np.ndarray)
                                                    else V.data_ptr()),
                                         capi.u32ptr(n), capi.fptr(cap.zero), capi.fptr(cap.inc),
                                         cap.t0, cap.deltaT, C.byref(o))
            capi.check(st, "bpgb_backproject_host")

        # first call from a fresh host thread (its plan cache and device buffers empty) on
        # pageable numpy buffers: plan build, table kernel, allocation, copies, kernel
        pageable_V = np.empty(N, np.float32)
        box = {}

        def first():
            torch.cuda.set_device(local)
            t = time.perf_counter()
            host_call(cap.H, pageable_V)
            box["s"] = time.perf_counter() - t
            t = time.perf_counter()
            for _ in range(max(1, args.steps // 2)):
                host_call(cap.H, pageable_V)
            box["cached"] = (time.perf_counter() - t) / max(1, args.steps // 2)

        th = threading.Thread(target=first)
        th.start()
        th.join()
        variants["pageable_first_call"] = {"ms": box["s"] * 1e3,
                                           "value": updates * ws / box["s"]}
        variants["pageable_cached"] = {"ms": box["cached"] * 1e3,
                                       "value": updates * ws / box["cached"]}
        hH = torch.from_numpy(cap.H).pin_memory()
        hV = torch.empty(N, dtype=torch.float32).pin_memory()
        for _ in range(max(1, args.warmup // 2)):
            host_call(hH, hV)
        t = time.perf_counter()
        for _ in range(args.steps):
            host_call(hH, hV)
        e2e_s = (time.perf_counter() - t) / args.steps
        e2e = {"value": updates * ws / e2e_s, "unit": "updates/s",
               "h2d_bytes_per_step": int(cap.H.nbytes), "d2h_bytes_per_step": int(cap.nvox * 4),
               "ms_per_step": e2e_s * 1e3,
               "path": "bpgb_backproject_host (the call_cuda_backprojection drop-in) on pinned "
                       "buffers, the thread's cached plan: H2D + kernel + D2H, synchronous",
               "variants": variants}
    elif phasor and args.dtype == "f32":
        # bp::phasor_reconstruction's replacement on host buffers: time window, FP64 pairs,
        # plan (tables on the GPU), pulse, complex backprojection, volume back -- per call
        traw = np.ascontiguousarray(cap.transient_array())
        out = np.empty(cap.nvox * 2, np.float32)
        lg = np.ascontiguousarray(cap.laser_grid, np.float32)
        cg = np.ascontiguousarray(cap.camera_grid, np.float32)
        po = capi.options(algo=capi.ALGO_FAST)

        def phasor_call():
            st = L.bpgb_phasor_capture(capi.fptr(traw), cap.T, capi.fptr(cg), cg.shape[0],
                                       cg.shape[1], capi.fptr(lg), lg.shape[0], lg.shape[1],
                                       capi.fptr(capi.f32(cap.camera_position)),
                                       capi.fptr(capi.f32(cap.laser_position)), cap.t0,
                                       cap.deltaT, 0, capi.fptr(capi.f32(cap.volume_position)),
                                       capi.fptr(capi.f32(cap.volume_size)), capi.u32ptr(n),
                                       capi.fptr(np.zeros(3, np.float32)), cap.wavelength,
                                       C.byref(po), capi.fptr(out))
            capi.check(st, "bpgb_phasor_capture")

        phasor_call()
        t = time.perf_counter()
        for _ in range(args.steps):
            phasor_call()
        e2e_s = (time.perf_counter() - t) / args.steps
        e2e = {"value": updates * ws / e2e_s, "unit": "updates/s",
               "h2d_bytes_per_step": int(traw.nbytes), "d2h_bytes_per_step": int(out.nbytes),
               "ms_per_step": e2e_s * 1e3,
               "path": "bpgb_phasor_capture (bp::phasor_reconstruction's replacement) on "
                       "pageable host buffers: window crop, FP64 pairs, plan with GPU tables, "
                       "pulse, complex backprojection, D2H -- everything per call"}

    clocks = clk.summary()
    esz = {"f32": 4, "f16": 2}[args.dtype] * (2 if phasor else 1)
    algo_bytes = cap.P * cap.T * esz + cap.nvox * (8 if phasor else 4)
    factored = bool(info.get("factored"))
    roofline = roofline_for(updates / (bp_ms * 1e-3), bp_ms, algo_bytes, phasor, clocks, dev,
                            ("bp_fact_kernel" if factored else "bp_fast_kernel")
                            if info["algo"] == "fast" else "bp_exact_kernel",
                            1.0 if factored else 0.0)
    roofline["kernel_ms"] = bp_ms
    tr = ROOT / "profiles" / f"traffic_{args.workload}.json"
    if tr.exists():
        try:
            roofline["traffic"] = json.loads(tr.read_text()).get("dram_bytes_per_launch")
        except Exception:
            pass

    line = {
        "metric": "voxel-pair updates/s", "value": value, "unit": "updates/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": {"f32": "f32", "f16": "f16 storage, f32 accumulate"}[args.dtype] if not phasor
        else {"f32": "complex64", "f16": "complex f16 storage, complex64 accumulate"}[args.dtype],
        "data": "synthetic (seeded scene rendered per pair; no dataset available)",
        "config": {"workload": f"{args.workload}: {WORKLOADS[args.workload]}", "P": cap.P,
                   "T": cap.T, "voxels": list(N), "updates_per_step": updates,
                   "l2": f"inputs larger than L2 (H = {cap.H.nbytes / 1e6:.0f} MB > 129 MB)",
                   "plan": info, "autotune": tune_rep,
                   "step": "pulse + backprojection" if phasor else "backprojection",
                   "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU"},
        "roofline": roofline,
        "e2e": e2e,
        "gpu_launches": int(launches),
        "clocks": clocks,
    }
    if phasor:
        line["stage_ms"] = {"backprojection": bp_ms, "pulse_and_conversion": ms - bp_ms}
    plan.close()
    if args.workload == "octree_256" and not args.no_octree:
        # the headline comparison: the learned octree against this dense pass, in the
        # same process (measure_octree)
        with ClockSampler(local) as oclk:
            m = measure_octree(args, dev)
        o = {k: v for k, v in m.items() if not k.startswith("_")}
        o["ms_per_recon"]["dense_fp32_tuned"] = ms
        o["speedup_vs_dense_fp32_tuned"] = ms / m["_ms"]
        o["clocks"] = oclk.summary()
        line["octree"] = o
    if rank == 0 and not args.no_cpu_baseline:
        r, dt, nvs, cores = cpu_baseline_timed(cap, args.cpu_seconds, args.cpu_sample)
        line["cpu_baseline"] = {"value": r, "unit": "updates/s", "cores": cores, "kind": "port",
                                "sample": f"{nvs} seeded random voxels x all {cap.P} pairs "
                                          f"({dt:.1f} s); reference classic_backprojection "
                                          "restated in C with OpenMP"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


OCTREE_SCENES = 6
OCTREE_FP64_SAMPLE = 4096
# (fine tile preset, budgets): 8^3 tiles (the learned octree's, four per CTA) for small
# budgets, the dense pass's 16 x 16 x 8 tiles (a tile then spans 2 x 2 x 1 score blocks)
# for large ones
FRONTIER = ((13, (0.04, 0.05, 0.075, 0.1, 0.2, 0.3, 0.4, 0.5, 0.6)),
            (3, (0.3, 0.4, 0.5, 0.6, 0.7, 0.8)))


def measure_octree(args, dev, frontier: bool = True) -> dict:
    """The learned octree on the octree_256 capture shape (FP16 rows resident), over
    OCTREE_SCENES seeded held-out scenes, against the plain dense FAST pass on FP32 rows
    of the same scenes in the same process.

    Quality per scene, against the dense FP32 volume D: whole-volume rel-L2 and PSNR,
    rel-L2 over the occupied blocks, occupied-voxel recall (occupied: -lap(D) >= tau
    max(-lap(D)), the labels' definition); and against FP64 (bpgb_eval_f64_voxels, the GPU
    restatement of the FP64 oracle, bit-identical to it per tests/test_gpu_eval64.py) on
    OCTREE_FP64_SAMPLE voxels drawn uniformly over the volume, selected and unselected
    blocks alike.  The frontier: budgeted reconstructions (the CNN's blocks first, then
    blocks ranked by the 64^3 pass's detail over the 32^3 one, filled from the 64^3 pass)
    at the FRONTIER budgets (fractions of the blocks) on 8^3 and on 16 x 16 x 8 fine tiles,
    each timed over the same scenes.""" 
    import torch

    from backprojector_gb300 import capi, octree

    if not octree.WEIGHTS.exists():
        raise RuntimeError(f"{octree.WEIGHTS} missing: run python -m backprojector_gb300.octree_train")
    model, state = octree.OccupancyCNN.load(dev)
    p_lo = float(state["p_lo"])
    logit_lo = octree.logit(p_lo)
    geo = octree.OctreeGeometry.of("octree_256")
    rec = octree.Reconstructor(geo, dev)
    s = rec.stream
    P = len(geo.pairs)
    nvox = int(np.prod(geo.fine))
    series = FRONTIER if frontier else ()
    ids = np.sort(np.random.default_rng(args.seed + 7).choice(nvox, OCTREE_FP64_SAMPLE, replace=False))
    d_ids = torch.from_numpy(ids.astype(np.int64)).to(dev)
    d_f64 = torch.empty(len(ids), dtype=torch.float64, device=dev)

    def rel(a, b):
        return float(torch.linalg.vector_norm(a.double() - b.double()) /
                     torch.linalg.vector_norm(b.double()))

    scenes, quality, fp64 = [], [], []
    for k in range(OCTREE_SCENES):
        pts, alb = octree.scene(geo, 2_000_000 + args.seed * 100 + k)
        rec.render(pts, alb)
        rows, amax = rec.rows.clone(), rec.absmax.clone()
        d32 = rec.dense_for_labels().clone()  # plain dense FAST pass, FP32 rows
        occ = rec.occupied_voxels(d32)
        capi.eval_f64_voxels(rec.H, geo.T, rec.d_pairs, P, geo.fine, geo.zero, geo.inc_fine,
                             geo.t0, geo.deltaT, d_ids, d_f64, stream=s)
        s.synchronize()
        f64 = d_f64.clone()
        out = rec.reconstruct(model, logit_lo)
        s.synchronize()
        out = out.double()
        comp = rec.computed_mask()
        quality.append(octree.metrics(out, d32, comp, occ))
        fp64.append({"octree": rel(out.reshape(-1)[d_ids], f64),
                     "dense_fp32": rel(d32.reshape(-1)[d_ids], f64),
                     "sample_selected": float(comp.reshape(-1)[d_ids].float().mean())})
        scenes.append((rows, amax, d32, occ, f64))
        del out
    torch.cuda.synchronize()

    def timed(r, budget, steps, warmup):
        def step(k):
            r.rows, r.absmax = scenes[k % len(scenes)][:2]
            r.reconstruct(model, logit_lo, budget=budget)

        for k in range(warmup):
            step(k)
        r.stream.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0 = capi.launch_count()
        e0.record(r.stream)
        for k in range(steps):
            step(k)
        e1.record(r.stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / steps, capi.launch_count() - l0

    ms, launches = timed(rec, 0.0, args.steps, args.warmup)
    points_raw = []
    for tile, budgets in series:
        r = rec if tile == 13 else octree.Reconstructor(geo, dev, fine_tile=tile, fine_splits=4)
        for b in budgets:
            q = []
            for rows, amax, d32, occ, f64 in scenes:
                r.rows, r.absmax = rows, amax
                ob = r.reconstruct(model, logit_lo, budget=b)
                r.stream.synchronize()
                cb = r.computed_mask()
                q.append({"rel_l2": rel(ob, d32), "computed_fraction": float(cb.float().mean()),
                          "recall": float((cb & occ).sum()) / max(1, int(occ.sum())),
                          "fp64_sample": rel(ob.reshape(-1)[d_ids], f64)})
            t_ms = timed(r, b, max(OCTREE_SCENES, args.steps // 2), 1)[0]
            points_raw.append((tile, b, t_ms, q, tuple(r.tile)))
        if r is not rec:
            r.close()

    # stage breakdown on scene 0
    rec.rows, rec.absmax = scenes[0][:2]
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(6)]
    ev[0].record(s)
    rec.coarse_plan.execute(rec.rows, rec.coarse, s)
    ev[1].record(s)
    model.features(rec.coarse, geo.coarse, 1, rec.X0, s)
    model.forward(rec.X0, geo.coarse, 1, logits=rec.logits, stream=s)
    ev[2].record(s)
    capi.upsample_trilinear(rec.coarse, geo.coarse, rec.fine, geo.fine, s)
    rec.sparse_plan.select_tiles(rec.logits, rec.blocks, octree.BLOCK, logit_lo, rec.tile_list,
                                 rec.tile_count, s)
    ev[3].record(s)
    rec.sparse_plan.execute_tiles(rec.rows, rec.fine, rec.tile_list, rec.tile_count, rec.n_tiles, s)
    ev[4].record(s)
    rec._unscale(rec.fine)
    ev[5].record(s)
    ev[5].synchronize()
    names = ["coarse_pass", "cnn", "fill_select", "sparse_fine_pass", "rescale"]
    stages = {n: ev[i].elapsed_time(ev[i + 1]) for i, n in enumerate(names)}
    n_sel = int(rec.tile_count.item())
    computed_updates = n_sel * int(np.prod(rec.tile)) * P

    # plain dense passes on the same GPU (FP32 and FP16 rows, default FAST plans)
    def time_plan(p, H, out, reps=3):
        p.execute(H, out, s)
        s.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(s)
        for _ in range(reps):
            p.execute(H, out, s)
        b.record(s)
        b.synchronize()
        return a.elapsed_time(b) / reps

    pts, alb = octree.scene(geo, 2_000_000 + args.seed * 100)
    rec.render(pts, alb)
    dense32_ms = time_plan(rec.label_plan, rec.H, rec.fine)
    dense16_ms = time_plan(rec.sparse_plan, rec.rows, rec.fine)

    q = {k: float(np.mean([m[k] for m in quality])) for k in quality[0]}
    q["recall_min"] = float(min(m["recall"] for m in quality))
    q["rel_l2_max"] = float(max(m["rel_l2"] for m in quality))
    q["reference"] = "dense FAST pass on FP32 rows of the same scenes (occupancy from it)"
    f = {"voxels": len(ids), "rel_l2_octree_mean": float(np.mean([x["octree"] for x in fp64])),
         "rel_l2_octree_max": float(max(x["octree"] for x in fp64)),
         "rel_l2_dense_fp32_mean": float(np.mean([x["dense_fp32"] for x in fp64])),
         "selected_fraction_of_sample": float(np.mean([x["sample_selected"] for x in fp64])),
         "how": "bpgb_eval_f64_voxels on the FP32 rows (bit-identical to the FP64 oracle), "
                "seeded voxels uniform over the 256^3 volume"}
    points = []
    for tile, b, t_ms, r, tdim in points_raw:
        points.append({"budget": b, "tile": list(tdim),
                       "computed_fraction": float(np.mean([x["computed_fraction"] for x in r])),
                       "ms_per_recon": t_ms, "speedup_vs_dense_fp32": dense32_ms / t_ms,
                       "rel_l2_whole_mean": float(np.mean([x["rel_l2"] for x in r])),
                       "rel_l2_whole_max": float(max(x["rel_l2"] for x in r)),
                       "rel_l2_fp64_sample_max": float(max(x["fp64_sample"] for x in r)),
                       "recall_min": float(min(x["recall"] for x in r))})
    learned_point = {"budget": 0.0, "tile": list(rec.tile),
                     "computed_fraction": q["computed_fraction"], "ms_per_recon": ms,
                     "speedup_vs_dense_fp32": dense32_ms / ms, "rel_l2_whole_mean": q["rel_l2"],
                     "rel_l2_whole_max": q["rel_l2_max"], "rel_l2_fp64_sample_max": f["rel_l2_octree_max"],
                     "recall_min": q["recall_min"]}
    meeting = [p for p in [learned_point] + points if p["rel_l2_whole_max"] <= 1e-3
               and p["recall_min"] >= 0.99]
    best = max(meeting, key=lambda p: p["speedup_vs_dense_fp32"]) if meeting else None
    fast = [p for p in [learned_point] + points if p["speedup_vs_dense_fp32"] >= 10.0
            and p["recall_min"] >= 0.99]
    best10 = min(fast, key=lambda p: p["rel_l2_whole_max"]) if fast else None
    rec.close()
    return {
        "workload": WORKLOADS["octree_256_learned"],
        "scenes": OCTREE_SCENES, "p_lo": p_lo, "tau": float(state["tau"]),
        "ms_per_recon": {"learned_octree": ms, "dense_fp32": dense32_ms, "dense_fp16": dense16_ms},
        "speedup_vs_dense_fp32": dense32_ms / ms, "speedup_vs_dense_fp16": dense16_ms / ms,
        "effective_updates_per_s": nvox * P / (ms * 1e-3),
        "computed_updates_per_s_sparse_pass": computed_updates / (stages["sparse_fine_pass"] * 1e-3),
        "quality_vs_dense_fp32": q, "fp64_sample": f,
        "target": {"speedup": 10.0, "rel_l2": 1e-3, "recall": 0.99,
                   "speedup_met": dense32_ms / ms >= 10.0, "recall_met": q["recall_min"] >= 0.99,
                   "rel_l2_whole_met": q["rel_l2_max"] <= 1e-3,
                   "rel_l2_fp64_sample_met": f["rel_l2_octree_max"] <= 1e-3},
        "frontier": [learned_point] + points,
        "best_meeting_1e-3": best, "best_at_10x": best10,
        "stages_ms_scene0": stages, "selected_tiles_scene0": n_sel, "tiles": rec.n_tiles,
        "gpu_launches_per_recon": launches / max(1, args.steps),
        "_ms": ms, "_launches": launches, "_sparse_ms": stages["sparse_fine_pass"],
        "_computed_updates": computed_updates, "_n_sel": n_sel, "_tile": rec.tile,
    }


def run_octree(args):
    """octree_256_learned: each step reconstructs one of several seeded test captures
    (FP16 rows resident) through the learned octree (measure_octree); e2e adds the FP16
    rows' upload and the volume's download around each reconstruction."""
    import torch

    from backprojector_gb300 import octree

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    with ClockSampler(local) as clk:
        m = measure_octree(args, dev)
    ms = m["_ms"]
    geo = octree.OctreeGeometry.of("octree_256")
    P = len(geo.pairs)
    nvox = int(np.prod(geo.fine))

    # e2e: FP16 rows and their scale from pinned host memory, volume back, every step
    model, state = octree.OccupancyCNN.load(dev)
    logit_lo = octree.logit(float(state["p_lo"]))
    rec = octree.Reconstructor(geo, dev)
    s = rec.stream
    pts, alb = octree.scene(geo, 2_000_000 + args.seed * 100)
    rec.render(pts, alb)
    hrows = rec.rows.cpu().pin_memory()
    hmax = rec.absmax.cpu().pin_memory()
    hvol = torch.empty(geo.fine, dtype=torch.float32).pin_memory()
    drows = torch.empty_like(rec.rows)
    dmax = torch.empty_like(rec.absmax)

    def e2e_step():
        with torch.cuda.stream(s):
            drows.copy_(hrows, non_blocking=True)
            dmax.copy_(hmax, non_blocking=True)
            rec.rows, rec.absmax = drows, dmax
            out = rec.reconstruct(model, logit_lo)
            hvol.copy_(out, non_blocking=True)
        s.synchronize()

    e2e_step()
    t = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    e2e_s = (time.perf_counter() - t) / args.steps
    rec.close()

    clocks = clk.summary()
    sparse_ms = m["_sparse_ms"]
    roofline = roofline_for(m["_computed_updates"] / (sparse_ms * 1e-3), sparse_ms,
                            hrows.numel() * 2 + m["_n_sel"] * int(np.prod(m["_tile"])) * 4, False,
                            clocks, dev, "bp_fast_kernel (8^3 tiles, tile-list launch)")
    line = {
        "metric": "voxel-pair updates/s (dense-equivalent: 256^3 x 16384 per reconstruction)",
        "value": nvox * P / (ms * 1e-3), "unit": "updates/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f16 storage, f32 accumulate; bf16 CNN",
        "data": "synthetic (seeded octree_256 scenes rendered on the GPU; no dataset available)",
        "config": {"workload": f"octree_256_learned: {WORKLOADS['octree_256_learned']}",
                   "test_scenes": m["scenes"], "p_lo": m["p_lo"], "tau": m["tau"],
                   "l2": "inputs larger than L2 (FP16 rows 134 MB per capture, 6 captures)",
                   "parallelism": "single GPU"},
        "octree": {k: v for k, v in m.items() if not k.startswith("_")},
        "roofline": roofline,
        "e2e": {"value": nvox * P / e2e_s, "unit": "updates/s (dense-equivalent)",
                "h2d_bytes_per_step": int(hrows.numel() * 2 + 4),
                "d2h_bytes_per_step": int(hvol.numel() * 4), "ms_per_step": e2e_s * 1e3,
                "path": "FP16 rows H2D + learned-octree reconstruction + volume D2H"},
        "gpu_launches": int(m["_launches"]),
        "clocks": clocks,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_batch(args):
    """batch_64: every capture of the batch reconstructed per step by one graph replay of
    the persistent batch kernel; e2e adds the packed FP16 rows' upload and the volumes'
    download around it."""
    import torch

    from backprojector_gb300 import capi, synthetic

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    caps = synthetic.make_batch(64, seed=args.seed + rank)
    scales = synthetic.fp16_scales(caps)
    geo = synthetic.batch_geometry(caps, scales)
    opt = dict(h_dtype=capi.DTYPE_F16)
    if args.tile is not None:
        opt["tile"] = args.tile
    layout = capi.Batch(geo, **opt)  # row / voxel layout does not depend on the tile shape
    info = layout.info()
    Hh = synthetic.pack_batch(caps, layout.row_offsets, info["pitch"], np.float16, scales)
    layout.close()
    dH = torch.from_numpy(Hh).to(dev)
    dV = torch.empty(info["total_voxels"], dtype=torch.float32, device=dev)
    tune_rep = None
    if not args.no_tune and args.tile is None:
        t = time.perf_counter()
        tuned, tune_rep = capi.autotune_batch(geo, dH, dV, **opt)
        tune_rep["seconds"] = time.perf_counter() - t
        opt.update(tuned)
    gate = capi.Batch(geo, checked=1, **opt)
    gate.execute(dH, dV)
    if gate.check() != 0:
        raise RuntimeError("window check failed: bins outside the staged windows")
    gate.close()
    batch = capi.Batch(geo, **opt)
    info = batch.info()
    stream = torch.cuda.Stream(device=dev)

    def step():
        batch.graph_launch(dH, dV, stream)

    for _ in range(args.warmup):
        step()
    stream.synchronize()
    batch.check()
    # kernels one batch execute launches (persistent launches + split reductions): the
    # captured graph replays exactly these
    k0 = capi.launch_count()
    batch.execute(dH, dV, stream)
    stream.synchronize()
    per_step = capi.launch_count() - k0
    batch.check()
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    launches0 = capi.launch_count()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        e1.synchronize()
    torch.cuda.synchronize()
    # graph replays launch the captured kernels without passing through the library's
    # counter: per_step kernels each
    launches = max(capi.launch_count() - launches0, 0) + per_step * args.steps
    ms = e0.elapsed_time(e1) / args.steps
    batch.check()
    ms = max_over_ranks(ms, dev)
    updates = int(info["updates"])
    value = updates * ws / (ms * 1e-3)

    # the same captures one plan each, back to back (what a caller without batches does)
    plans = []
    for i, c in enumerate(caps):
        r = batch.row_offsets[i]
        plans.append((capi.Plan(c.pairs, c.T, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT,
                                h_dtype=capi.DTYPE_F16, h_scale=float(scales[i]),
                                h_pitch=info["pitch"]),
                      dH[r:r + c.P], dV[batch.voxel_offsets[i]:batch.voxel_offsets[i] + c.nvox]))
    hp = Hh  # keep numpy alive
    for p, h, v in plans:
        p.execute(h, v, stream)
    stream.synchronize()
    s0 = torch.cuda.Event(enable_timing=True)
    s1 = torch.cuda.Event(enable_timing=True)
    s0.record(stream)
    for p, h, v in plans:
        p.execute(h, v, stream)
    s1.record(stream)
    s1.synchronize()
    per_plan_ms = s0.elapsed_time(s1)
    for p, _, _ in plans:
        p.close()

    # e2e: pinned packed rows up, graph replay, volumes down, every step
    hH = torch.from_numpy(hp).pin_memory()
    hV = torch.empty(info["total_voxels"], dtype=torch.float32).pin_memory()

    def e2e_step():
        with torch.cuda.stream(stream):
            dH.copy_(hH, non_blocking=True)
            batch.graph_launch(dH, dV, stream)
            hV.copy_(dV, non_blocking=True)
        stream.synchronize()

    for _ in range(max(1, args.warmup // 2)):
        e2e_step()
    t = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    e2e_s = (time.perf_counter() - t) / args.steps
    e2e = {"value": updates * ws / e2e_s, "unit": "updates/s",
           "h2d_bytes_per_step": int(hH.numel() * 2), "d2h_bytes_per_step": int(hV.numel() * 4),
           "ms_per_step": e2e_s * 1e3,
           "path": "capi.Batch.graph_launch with the packed rows copied up and the volumes "
                   "copied down inside each step"}
    clocks = clk.summary()
    algo_bytes = int(sum(c.P * c.T * 2 + c.nvox * 4 for c in caps))
    # lasers x SPADs captures (whole 4-SPAD blocks) run the factored body
    fact_updates = sum(c.updates for c in caps
                       if len(np.unique(c.pairs["laser_point"], axis=0)) > 1
                       and (c.P // len(np.unique(c.pairs["laser_point"], axis=0))) % 4 == 0)
    roofline = roofline_for(updates / (ms * 1e-3), ms, algo_bytes, False, clocks, dev,
                            "bp_batch_kernel", fact_updates / updates)
    line = {
        "metric": "voxel-pair updates/s", "value": value, "unit": "updates/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f16 storage, f32 accumulate",
        "data": "synthetic (seeded scenes rendered per pair; no dataset available)",
        "config": {"workload": f"batch_64: {WORKLOADS['batch_64']}", "captures": len(caps),
                   "updates_per_step": updates, "batch": info, "autotune": tune_rep,
                   "l2": f"inputs larger than L2 (packed H = {Hh.nbytes / 1e6:.0f} MB > 129 MB)",
                   "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU"},
        "roofline": roofline,
        "per_capture_plans": {"ms_per_step": per_plan_ms,
                              "value": updates / (per_plan_ms * 1e-3), "unit": "updates/s",
                              "note": "the same 64 captures as 64 plan launches on one stream"},
        "e2e": e2e,
        "gpu_launches": int(launches),
        "clocks": clocks,
    }
    if rank == 0 and not args.no_cpu_baseline:
        probe = max(1, args.cpu_sample // 64)
        r, dt, nvs, cores = cpu_baseline_batch(caps, probe)
        per = cpu_sample_for(r, sum(c.P for c in caps), args.cpu_seconds, probe,
                             min(c.nvox for c in caps))
        if per > nvs:
            r, dt, nvs, cores = cpu_baseline_batch(caps, per)
        line["cpu_baseline"] = {"value": r, "unit": "updates/s", "cores": cores, "kind": "port",
                                "sample": f"{nvs} seeded random voxels of each of the 64 "
                                          f"captures x all their pairs ({dt:.1f} s); reference "
                                          "classic_backprojection restated in C with OpenMP"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    batch.close()
    if ws > 1:
        torch.distributed.destroy_process_group()


def cpu_baseline_batch(caps, per_capture: int, seed: int = 0):
    """cpu_baseline over every capture of a batch: `per_capture` voxels of each."""
    upd, secs, cores = 0, 0.0, None
    for i, c in enumerate(caps):
        r, dt, n, cores = cpu_baseline(c, per_capture, seed=seed * 1000 + i)
        upd += n * c.P
        secs += dt
    return upd / secs, secs, per_capture, cores


def roofline_for(achieved, ms, algo_bytes, phasor, clocks, dev, kernel, factored=0.0):
    """Roofline of the FAST kernels: per-update pipe work against the pipe rates measured
    on this GPU, at the median SM clock of the timed region.  factored: the fraction of the
    updates that run the factored lasers x SPADs body (1.0 for a factored plan); the peak
    blends the two bodies' peaks by their updates."""
    import torch

    from backprojector_gb300 import capi

    peaks = measured_peaks()
    sm_mhz = clocks.get("sm_mhz") or peaks.get("sm_max_mhz", 2070.0)
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    # Pipe work of one FAST update: FP32 lanes (dz, q, x, +row constant, +1.5*2^23,
    # accumulate; complex accumulates two lanes), one rsqrt, one shared gather (two bank
    # slots for complex).  Pipe rates are measured on this GPU (bpgb_diag_pipe_rates).
    try:
        rates = capi.pipe_rates()
        rate_src = "measured on this GPU by bpgb_diag_pipe_rates"
    except Exception:
        rates = {"rsqrt_per_sm_clk": float(MUFU_PER_SM_PER_CLK), "fp32_lanes_per_sm_clk": 128.0,
                 "lds_per_sm_clk": 32.0}
        rate_src = "nominal (probe unavailable)"
    work = {"fp32": 7.0 if phasor else 6.0, "sfu": 1.0, "smem": 2.0 if phasor else 1.0}
    # lasers x SPADs with factored legs: A + B, the rounding add and the accumulate per
    # update, plus the laser leg of each voxel (3 lanes and one rsqrt) shared by the 4 SPADs
    # of a block
    fwork = {"fp32": 3.0 + 3.4 / 4, "sfu": 1.0 / 4, "smem": 1.0}

    def body_peak(w):
        per_clk = {"fp32": rates["fp32_lanes_per_sm_clk"] / w["fp32"],
                   "sfu": rates["rsqrt_per_sm_clk"] / w["sfu"],
                   "smem": rates["lds_per_sm_clk"] / w["smem"]}
        b = min(per_clk, key=per_clk.get)
        return b, sms * per_clk[b] * sm_mhz * 1e6

    bound, peak_updates = body_peak(work)
    fbound, fpeak = body_peak(fwork)
    if factored >= 1.0:
        bound, peak_updates, work = fbound, fpeak, fwork
    elif factored > 0.0:
        peak_updates = 1.0 / ((1.0 - factored) / peak_updates + factored / fpeak)
        bound = f"{bound} ({1 - factored:.0%} of updates) / {fbound} ({factored:.0%}, factored)"
    return {
        "bound": bound, "kernel": kernel,
        "achieved": achieved, "peak": peak_updates, "unit": "voxel-pair updates/s",
        "frac": achieved / peak_updates,
        "factored_fraction": factored,
        "peak_basis": f"{sms} SMs x {sm_mhz:.0f} MHz (median SM clock in the timed region) x "
                      f"min over pipes of rate / work per update: fp32 "
                      f"{rates['fp32_lanes_per_sm_clk']:.1f} lanes/clk / {work['fp32']:g}, sfu "
                      f"{rates['rsqrt_per_sm_clk']:.1f} rsqrt/clk / {work['sfu']:g}, smem "
                      f"{rates['lds_per_sm_clk']:.1f} loads/clk / {work['smem']:g}; rates "
                      f"{rate_src}",
        "pipe_rates_per_sm_clk": rates,
        "traffic": None,
        "algorithmic_bytes": algo_bytes,
        "hbm_achieved_gbs": algo_bytes / (ms * 1e-3) / 1e9,
        "hbm_peak_gbs": peaks.get("hbm_gbs"),
        "hbm_frac": algo_bytes / (ms * 1e-3) / 1e9 / peaks.get("hbm_gbs", 6800.0),
    }


PROFILE_CASES = ("dense256", "batch64", "octree", "cnn_train", "phasor128", "exhaustive32",
                 "pulse128")


def _timed(torch, stream, fn, reps):
    ms = None
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
    return ms


def run_profile_case(args):
    """--profile-case NAME: a fixed launch sequence for profiling one kernel (ncu -k
    <kernel> -s <n> -c 1), repeated --reps times (one to warm, one to capture); prints the
    CUDA-event time of the last repetition.  Launch order per repetition (for ncu -s):
      dense256: bp_fast_kernel x1;  batch64: bp_batch_kernel launches (+ split reductions);
      phasor128: bp_fast_kernel, reduce_splits_kernel (pair splits > 1);
      pulse128: phasor_pulse_kernel x1 (the 128^3 phasor capture's 16,384 rows);
      exhaustive32: bp_fact_kernel (bp_fast_kernel with --unfactored), reduce_splits_kernel;
      octree: bp_fast_kernel (coarse), conv_fwd_kernel x4, upsample, select_tiles,
              bp_fast_kernel (tile list), scale;
      cnn_train: conv_fwd x4, bce, conv_wgrad + reduce x4 interleaved with conv_fwd
              (backward data) x3, adam x4, pack x4."""
    from backprojector_gb300 import capi, octree, synthetic

    args.tile = -1 if args.tile is None else args.tile
    import torch

    dev = torch.device("cuda:0")
    s = torch.cuda.Stream()
    out = {"case": args.profile_case}
    if args.profile_case == "pulse128":
        cap = synthetic.make_capture("phasor_128", seed=0)
        dH = torch.from_numpy(cap.H).to(dev)
        Hc = torch.empty(cap.H.shape, dtype=torch.complex64, device=dev)
        out["ms"] = _timed(torch, s, lambda: capi.phasor_pulse_device(
            dH, cap.P, cap.T, cap.T, cap.wavelength, cap.deltaT, Hc, cap.T, stream=s), args.reps)
        out["taps"] = int(capi.phasor_taps(cap.wavelength, cap.deltaT).shape[1])
        out["outputs"] = cap.P * cap.T
    elif args.profile_case in ("dense256", "octree"):
        geo = octree.OctreeGeometry.of("octree_256")
        rec = octree.Reconstructor(geo, dev)
        rec.render(*octree.scene(geo, 2_000_000))
        if args.profile_case == "dense256":
            f16 = args.dtype == "f16"
            p = capi.Plan(geo.pairs, geo.T, geo.fine, geo.zero, geo.inc_fine, geo.t0, geo.deltaT,
                          algo=capi.ALGO_FAST, tile=args.tile,
                          h_dtype=capi.DTYPE_F16 if f16 else capi.DTYPE_F32)
            rows = rec.rows if f16 else rec.H
            out["ms"] = _timed(torch, s, lambda: p.execute(rows, rec.fine, s), args.reps)
            out["plan"] = p.info()
            out["updates"] = out["plan"]["updates"]
            p.close()
        else:
            model, state = octree.OccupancyCNN.load(dev)
            lo = octree.logit(float(state["p_lo"]))
            out["ms"] = _timed(torch, rec.stream, lambda: rec.reconstruct(model, lo), args.reps)
            out["selected_tiles"] = int(rec.tile_count.item())
            out["tile"] = list(rec.tile)
            out["updates_sparse"] = out["selected_tiles"] * int(np.prod(rec.tile)) * len(geo.pairs)
        rec.close()
    elif args.profile_case == "phasor128":
        cap = synthetic.make_capture("phasor_128", seed=0)
        Hc = torch.empty(cap.H.shape, dtype=torch.complex64, device=dev)
        capi.phasor_pulse_device(torch.from_numpy(cap.H).to(dev), cap.P, cap.T, cap.T,
                                 cap.wavelength, cap.deltaT, Hc, cap.T)
        opt = dict(algo=capi.ALGO_FAST, tile=args.tile, chunk=args.chunk, stages=args.stages,
                   pair_splits=args.splits, h_dtype=capi.DTYPE_C64)
        rows = Hc
        if args.dtype == "f16":
            flat = torch.view_as_real(Hc)
            scale = float(flat.abs().max()) / 16384.0 or 1.0
            rows = (flat / scale).half().contiguous()
            opt.update(h_dtype=capi.DTYPE_C32, h_scale=scale)
        N = tuple(int(v) for v in cap.voxels_per_side)
        dV = torch.empty(N, dtype=torch.complex64, device=dev)
        torch.cuda.synchronize()
        p = capi.Plan(cap.pairs, cap.T, N, cap.zero, cap.inc, cap.t0, cap.deltaT, **opt)
        out["ms"] = _timed(torch, s, lambda: p.execute(rows, dV, s), args.reps)
        out["plan"] = p.info()
        p.close()
    elif args.profile_case == "exhaustive32":
        cap = synthetic.make_capture("dense_exhaustive_16", seed=0)
        N = tuple(int(v) for v in cap.voxels_per_side)
        dH = torch.from_numpy(cap.H).to(dev)
        dV = torch.empty(N, dtype=torch.float32, device=dev)
        p = capi.Plan(cap.pairs, cap.T, N, cap.zero, cap.inc, cap.t0, cap.deltaT,
                      algo=capi.ALGO_FAST, tile=args.tile, chunk=args.chunk, stages=args.stages,
                      pair_splits=args.splits, unfactored=int(args.unfactored))
        torch.cuda.synchronize()
        out["ms"] = _timed(torch, s, lambda: p.execute(dH, dV, s), args.reps)
        out["plan"] = p.info()
        p.close()
    elif args.profile_case == "batch64":
        caps = synthetic.make_batch(64, seed=0)
        scales = synthetic.fp16_scales(caps)
        b = capi.Batch(synthetic.batch_geometry(caps, scales), h_dtype=capi.DTYPE_F16,
                       unfactored=int(args.unfactored))
        info = b.info()
        H = synthetic.pack_batch(caps, b.row_offsets, info["pitch"], np.float16, scales)
        dH = torch.from_numpy(H).to(dev)
        dV = torch.empty(info["total_voxels"], device=dev)
        out["ms"] = _timed(torch, s, lambda: b.execute(dH, dV, s), args.reps)
        out["batch"] = info
        b.close()
    else:
        geo = octree.OctreeGeometry.of("octree_256")
        rec = octree.Reconstructor(geo, dev)
        n = 16
        coarse = torch.empty((n, int(np.prod(geo.coarse))), device=dev)
        bnorm = torch.empty_like(coarse)
        for i in range(n):
            rec.render(*octree.scene(geo, 1_000_000 + i))
            coarse[i] = rec.coarse_pass().reshape(-1)
            bnorm[i] = rec.labels_from_dense(rec.dense_for_labels()).reshape(-1)
        rec.close()
        model = octree.OccupancyCNN(dev, seed=0)
        X = model.features(coarse, geo.coarse, n)
        y = (bnorm >= octree.TAU).to(torch.uint8).reshape(-1).contiguous()
        torch.cuda.synchronize()
        out["ms"] = _timed(torch, torch.cuda.current_stream(),
                           lambda: model.train_step(X, y, geo.coarse, n, 1e-3, 50.0), args.reps)
        out["voxels"] = n * int(np.prod(geo.coarse))
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="octree_256")
    ap.add_argument("--algo", choices=["fast", "exact"], default="fast")
    ap.add_argument("--dtype", choices=["f32", "f16"], default="f32")
    ap.add_argument("--kahan", action="store_true")
    ap.add_argument("--tile", type=int, default=None,
                    help="fixed tile preset (skips the autotuner)")
    ap.add_argument("--no-tune", action="store_true", help="untuned default configuration")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--voxels", type=int, default=None,
                    help="override the volume resolution (reduced profiling cases)")
    ap.add_argument("--cpu-sample", type=int, default=1024,
                    help="voxels of the calibration run of the CPU baseline")
    ap.add_argument("--cpu-seconds", type=float, default=10.0,
                    help="CPU work the cpu_baseline sample is sized to")
    ap.add_argument("--ref-sample", type=int, default=256,
                    help="smallest per-step voxel sample of --impl reference")
    ap.add_argument("--ref-seconds", type=float, default=1.0,
                    help="CPU work per step --impl reference sizes its sample to")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-octree", action="store_true",
                    help="octree_256: skip the learned-octree object of the line")
    ap.add_argument("--no-ref-gpu", action="store_true", help="accepted for compatibility")
    ap.add_argument("--profile-case", choices=PROFILE_CASES, default=None,
                    help="run a fixed launch sequence for ncu instead of the bench")
    ap.add_argument("--reps", type=int, default=2, help="--profile-case repetitions")
    ap.add_argument("--chunk", type=int, default=0, help="--profile-case: rows per stage")
    ap.add_argument("--stages", type=int, default=0, help="--profile-case: pipeline depth")
    ap.add_argument("--splits", type=int, default=0, help="--profile-case: pair splits")
    ap.add_argument("--unfactored", action="store_true", help="--profile-case: per-pair legs")
    args = ap.parse_args()
    if args.profile_case:
        run_profile_case(args)
    elif args.impl == "reference":
        run_reference_arm(args)
    elif args.workload == "batch_64":
        run_batch(args)
    elif args.workload == "octree_256_learned":
        run_octree(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
