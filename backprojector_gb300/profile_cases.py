"""Fixed launch sequences for profiling single kernels (ncu -k <kernel> -s <n> -c 1).

    python -m backprojector_gb300.profile_cases dense256 [--dtype f32|f16] [--tile N]
    python -m backprojector_gb300.profile_cases batch64 [--unfactored]
    python -m backprojector_gb300.profile_cases octree          # 2 learned-octree recons
    python -m backprojector_gb300.profile_cases cnn_train       # 2 CNN training steps
    python -m backprojector_gb300.profile_cases phasor128 [--dtype f32|f16] [--tile N]
        [--chunk C --stages S --splits K]                        # complex rows, 128^3
    python -m backprojector_gb300.profile_cases exhaustive32 [--unfactored] [--tile N]
        [--chunk C --stages S --splits K]       # 16x16 lasers x 16x16 SPADs, 32^3, FP32

Each case renders its seeded input on the GPU, runs the workload `--reps` times (default 2:
one to warm, one to capture) and prints the CUDA-event time of the last repetition.
Launch order per repetition (for `ncu -s`):
  dense256: bp_fast_kernel x1;  batch64: bp_batch_kernel x1;
  phasor128: bp_fast_kernel, reduce_splits_kernel (pair splits > 1);
  exhaustive32: bp_fact_kernel (bp_fast_kernel with --unfactored), reduce_splits_kernel;
  octree: bp_fast_kernel (coarse), conv_fwd_kernel x4, upsample, select_tiles,
          bp_fast_kernel (tile list), scale;
  cnn_train: conv_fwd x4, bce, conv_wgrad + reduce x4 interleaved with conv_fwd
          (backward data) x3, adam x4, pack x4.
"""
from __future__ import annotations

import argparse
import json

import numpy as np

from . import capi, octree, synthetic


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


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["dense256", "batch64", "octree", "cnn_train", "phasor128",
                                         "exhaustive32"])
    ap.add_argument("--dtype", choices=["f32", "f16"], default="f32")
    ap.add_argument("--tile", type=int, default=-1)
    ap.add_argument("--reps", type=int, default=2)
    ap.add_argument("--chunk", type=int, default=0)
    ap.add_argument("--stages", type=int, default=0)
    ap.add_argument("--splits", type=int, default=0)
    ap.add_argument("--unfactored", action="store_true")
    args = ap.parse_args(argv)

    import torch

    dev = torch.device("cuda:0")
    s = torch.cuda.Stream()
    out = {"case": args.case}
    if args.case in ("dense256", "octree"):
        geo = octree.OctreeGeometry.of("octree_256")
        rec = octree.Reconstructor(geo, dev)
        rec.render(*octree.scene(geo, 2_000_000))
        if args.case == "dense256":
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
    elif args.case == "phasor128":
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
    elif args.case == "exhaustive32":
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
    elif args.case == "batch64":
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


if __name__ == "__main__":
    main()
