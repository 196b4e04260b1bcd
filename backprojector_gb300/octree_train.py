"""Trains the occupancy CNN of the learned octree on seeded synthetic scenes.

    python -m backprojector_gb300.octree_train [--scenes 2000] [--epochs 60] [--out PATH]

Data: scene i (seed seed0 + i, octree_256 configuration: one laser, 128 x 128 SPADs,
T = 4096, 1-5 spheres / boxes / tori of 10,000 surface points) is rendered on the GPU
(bpgb_synth_render_device); its input is the 32^3 coarse FAST pass, its labels the
8^3-block occupancy of the 256^3 dense FAST pass after the 7-point Laplacian filter
(octree module docstring).  The last 10% of the scenes are held out: the block
threshold p_lo is the largest that keeps >= --recall of their occupied blocks.  The
weights, p_lo and the validation figures are written to --out (numpy .npz).
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import octree


def main(argv=None) -> dict:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--scenes", type=int, default=2000)
    ap.add_argument("--seed0", type=int, default=1_000_000)
    ap.add_argument("--epochs", type=int, default=60)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--tau", type=float, default=octree.TAU)
    ap.add_argument("--recall", type=float, default=0.995)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", default=str(octree.WEIGHTS))
    args = ap.parse_args(argv)

    import torch

    dev = torch.device("cuda:0")
    geo = octree.OctreeGeometry.of("octree_256")
    rec = octree.Reconstructor(geo, dev)
    t = time.perf_counter()
    coarse, bnorm = octree.make_training_set(rec, args.scenes, args.seed0)
    t_data = time.perf_counter() - t
    rec.close()
    ntrain = int(round(0.9 * args.scenes))
    model = octree.OccupancyCNN(dev, seed=args.seed)
    t = time.perf_counter()
    hist = octree.train(model, coarse[:ntrain], bnorm[:ntrain], geo.coarse, epochs=args.epochs,
                        batch=args.batch, lr=args.lr, tau=args.tau, seed=args.seed)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t
    scores = octree.block_scores(model, coarse[ntrain:], geo.coarse)
    occ = bnorm[ntrain:] >= args.tau
    p_lo = octree.calibrate(scores, bnorm[ntrain:], args.tau, args.recall)
    sel = scores >= p_lo
    summary = {
        "scenes": args.scenes, "train": ntrain, "val": args.scenes - ntrain,
        "seed0": args.seed0, "epochs": args.epochs, "tau": args.tau, "p_lo": p_lo,
        "val_block_recall": float((sel & occ).sum() / max(1, int(occ.sum()))),
        "val_selected_fraction": float(sel.float().mean()),
        "val_occupied_fraction": float(occ.float().mean()),
        "final_loss": hist[-1], "first_loss": hist[0],
        "data_seconds": t_data, "train_seconds": t_train,
    }
    model.save(args.out, tau=args.tau, p_lo=p_lo, loss=np.asarray(hist, np.float32),
               summary=json.dumps(summary))
    print(json.dumps(summary), flush=True)
    return summary


if __name__ == "__main__":
    main()
