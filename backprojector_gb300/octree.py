"""Learned octree: replaces the reference's threshold octree (octree_volume.hpp:18-198,
backproject.hpp:264-335, backproject_cuda.cu:183-367) with a learned block proposal.

Pipeline for one capture (all on the GPU, no host synchronisation inside):
  1. coarse dense pass: the FAST kernel at 32^3 over the target box;
  2. occupancy CNN (4 conv3d 3x3x3 layers, 1-16-16-16-1 channels, ReLU, BF16 weights
     and activations, FP32 accumulation on the tensor cores) on the coarse volume
     divided by its maximum: one logit per coarse voxel = per 8^3 block of the 256^3
     target (the 32^3 grid and the 8^3 blocks tile the same box);
  3. every fine voxel gets the trilinear upsampling of the coarse pass;
  4. blocks scoring p >= p_lo are backprojected at full resolution (FAST kernel,
     block-sparse tile-list launch): p >= p_hi confident, p_lo <= p < p_hi the
     low-confidence band for which the dense pass is the fallback; p < p_lo keep step 3.

Budgeted form (Reconstructor.reconstruct(budget=b)): a second coarse pass at 64^3 fills
the skipped blocks instead, and the fine pass computes round(b x blocks) blocks: the
CNN's blocks first, then the blocks where the 64^3 pass adds the most detail over the
32^3 one (bpgb_block_detail, the predictor of the fill's error), selected on the device
(bpgb_plan_select_tiles_topk).  Sweeping b gives the measured trade of speed against
whole-volume error.

Occupancy (labels and recall): voxel v of the dense reconstruction D is occupied when
its negated 7-point Laplacian response F = -lap(D) (bpgb_laplacian7) reaches
tau * max(F), tau = 0.2: the sharpened surfaces of the unfiltered backprojection, whose
raw values are a broad low-frequency bump (on these scenes D >= 0.5 max(D) marks 13% of
the voxels and 16% of the 8^3 blocks; F >= 0.2 max(F) marks 6.7% of the blocks).  A
block is occupied when it holds an occupied voxel.  The CNN is trained only on dense reconstructions the plain FAST method makes
from seeded synthetic scenes (synthetic.make_scene, octree_256 configuration).
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import capi, synthetic

COARSE = 32
BLOCK = 8
TAU = 0.2
IN_CHANNELS = 2  # coarse / max, and its negated 7-point Laplacian / max magnitude


def layers(in_channels: int = IN_CHANNELS):
    """(cin, cout, relu) of the four conv3d layers."""
    return ((in_channels, 16, True), (16, 16, True), (16, 16, True), (16, 1, False))


LAYERS = layers()
WEIGHTS = Path(__file__).resolve().parent / "weights" / "octree_cnn.npz"


def _np(cout: int) -> int:
    return 8 if cout <= 8 else 16


class OccupancyCNN:
    """The 4-layer occupancy CNN on the bpgb_cnn_* kernels (torch tensors hold memory)."""

    def __init__(self, device, seed: int = 0, state: dict | None = None,
                 in_channels: int = IN_CHANNELS):
        import torch

        self.torch = torch
        self.device = device
        if state is not None and "in_channels" in state:
            in_channels = int(state["in_channels"])
        self.in_channels = in_channels
        self.layers = layers(in_channels)
        rng = np.random.default_rng(seed)
        ws = []
        for li, (cin, cout, _) in enumerate(self.layers):
            kp = capi.cnn_kp(cin)
            if state is not None:
                w = np.asarray(state[f"w{li}"], np.float32)
                assert w.shape == (kp, cout), (w.shape, kp, cout)
            else:
                w = np.zeros((kp, cout), np.float32)
                fan_in = 27 * cin
                w[:27 * cin] = rng.normal(0.0, math.sqrt(2.0 / fan_in), (27 * cin, cout))
            ws.append(w)
        # masters, Adam moments and gradients: one flat buffer each (one Adam launch), the
        # layers as views [KP][COUT] into it
        self.shapes = [w.shape for w in ws]
        self.flat_W = torch.from_numpy(np.concatenate([w.reshape(-1) for w in ws])).to(device)
        self.flat_M = torch.zeros_like(self.flat_W)
        self.flat_V = torch.zeros_like(self.flat_W)
        self.flat_G = torch.zeros_like(self.flat_W)
        self.W, self.M, self.V, self.G = (self._views(f) for f in (
            self.flat_W, self.flat_M, self.flat_V, self.flat_G))
        self.step = int(state["step"]) if state is not None and "step" in state else 0
        self.Wt, self.Wb = [], []
        for li, (cin, cout, _) in enumerate(self.layers):
            self.Wt.append(torch.zeros((_np(cout), capi.cnn_kp(cin)), dtype=torch.bfloat16,
                                       device=device))
            self.Wb.append(torch.zeros((16, capi.cnn_kp(cout)), dtype=torch.bfloat16,
                                       device=device) if li > 0 else None)
        # tensor-core (tcgen05) weight images of the training step: forward, backward-data
        self.Wtc, self.Wtc_b = [], []
        for li, (cin, cout, _) in enumerate(self.layers):
            self.Wtc.append(torch.zeros(capi.cnn_tc_weight_bytes(cin) // 2, dtype=torch.bfloat16,
                                        device=device))
            self.Wtc_b.append(torch.zeros(capi.cnn_tc_weight_bytes(cout) // 2,
                                          dtype=torch.bfloat16, device=device)
                              if li > 0 else None)
        self._bufs = {}
        self._mma_stale = False
        self.pack()

    def _views(self, flat):
        out, off = [], 0
        for kp, cout in self.shapes:
            out.append(flat[off:off + kp * cout].view(kp, cout))
            off += kp * cout
        return out

    # ---- weights
    def pack(self, stream=None):
        self.pack_mma(stream)
        self.pack_tc(stream)

    def pack_mma(self, stream=None):
        """BF16 images of the inference kernels (bpgb_cnn_conv3d)."""
        for li, (cin, cout, _) in enumerate(self.layers):
            capi.cnn_pack_weights(self.W[li], cin, cout, _np(cout), self.Wt[li],
                                  16 if li > 0 else 0, self.Wb[li], stream)
        self._mma_stale = False

    def pack_tc(self, stream=None):
        """BF16 images of the tensor-core training kernels (bpgb_cnn_tc_conv3d), one launch."""
        capi.cnn_tc_pack_layers(self.W, [l[0] for l in self.layers], [l[1] for l in self.layers],
                                self.Wtc, self.Wtc_b, stream)

    def bias(self, li: int):
        """FP32 bias row of layer li (a view into the master weights)."""
        return self.W[li][27 * self.layers[li][0]]

    def state(self) -> dict:
        d = {f"w{li}": self.W[li].cpu().numpy() for li in range(len(self.layers))}
        d["step"] = np.int64(self.step)
        d["in_channels"] = np.int64(self.in_channels)
        return d

    def save(self, path, **meta) -> None:
        path = Path(path)
        path.parent.mkdir(parents=True, exist_ok=True)
        np.savez(path, **self.state(), **{k: np.asarray(v) for k, v in meta.items()})

    @classmethod
    def load(cls, device, path=WEIGHTS) -> tuple["OccupancyCNN", dict]:
        z = np.load(path)
        state = {k: z[k] for k in z.files}
        return cls(device, state=state), state

    # ---- buffers
    def _buf(self, name, shape, dtype):
        t = self._bufs.get(name)
        if t is None or t.shape != shape or t.dtype != dtype:
            t = self.torch.empty(shape, dtype=dtype, device=self.device)
            self._bufs[name] = t
        return t

    # ---- passes
    def features(self, coarse, dims, batch: int, X=None, stream=None):
        """BF16 input [batch * prod(dims) * in_channels] of FP32 coarse volumes."""
        n = batch * int(np.prod(dims)) * self.in_channels
        if X is None:
            X = self.torch.empty(n, dtype=self.torch.bfloat16, device=self.device)
        if self.in_channels == 1:
            capi.cnn_normalize(coarse, dims, batch, X, stream)
        else:
            scr = self._buf(f"feat{batch}", (2 * batch,), self.torch.float32)
            capi.cnn_features(coarse, dims, batch, X, scr, stream)
        return X

    def forward(self, X0, dims, batch: int, logits=None, stream=None, tc: bool | None = None):
        """logits (FP32 [batch * prod(dims)]) of input features X0 (features()): on the
        tcgen05 kernels when the volume allows it (tc=None), else on the mma.sync kernels."""
        if tc is None:
            tc = self.tc_supported(dims)
        if tc:
            if logits is None:
                logits = self._buf("Z", (batch * int(np.prod(dims)),), self.torch.float32)
            self._forward_tc(X0, dims, batch, logits, stream)
            return logits
        return self._forward_mma(X0, dims, batch, logits, stream)

    def _forward_tc(self, X0, dims, batch, logits, stream):
        """Forward pass on line-planes tensors; returns (layer inputs, activations)."""
        ci = self.in_channels
        X0l = self._lp(f"X0l_{batch}", ci, 0, dims, batch)
        Yl = [self._lp(f"Y{i}l_{batch}", 16, 0, dims, batch) for i in (1, 2, 3)]
        capi.cnn_lp_pack(X0, ci, ci, dims, batch, 0, X0l, stream)
        ins = [X0l] + Yl
        for li, (cin, cout, relu) in enumerate(self.layers):
            if li < 3:
                capi.cnn_tc_conv3d(ins[li], cin, 0, dims, batch, self.Wtc[li], self.bias(li), cout,
                                   relu, d_Y=Yl[li], stream=stream)
            else:
                capi.cnn_tc_conv3d(ins[li], cin, 0, dims, batch, self.Wtc[li], self.bias(li), cout,
                                   False, d_Yf=logits, stream=stream)
        return ins, Yl

    def _forward_mma(self, X0, dims, batch, logits, stream):
        torch = self.torch
        if self._mma_stale:
            self.pack_mma(stream)
        V = batch * int(np.prod(dims))
        Y1 = self._buf("Y1", (V, 16), torch.bfloat16)
        Y2 = self._buf("Y2", (V, 16), torch.bfloat16)
        Y3 = self._buf("Y3", (V, 16), torch.bfloat16)
        if logits is None:
            logits = self._buf("Z", (V,), torch.float32)
        ci = self.in_channels
        capi.cnn_conv3d(X0, ci, ci, dims, batch, self.Wt[0], 16, True, d_Y=Y1, stream=stream)
        capi.cnn_conv3d(Y1, 16, 16, dims, batch, self.Wt[1], 16, True, d_Y=Y2, stream=stream)
        capi.cnn_conv3d(Y2, 16, 16, dims, batch, self.Wt[2], 16, True, d_Y=Y3, stream=stream)
        capi.cnn_conv3d(Y3, 16, 16, dims, batch, self.Wt[3], 8, False, d_Yf=logits, stream=stream)
        return logits

    def _lp(self, name, channels, zpad, dims, batch):
        """A line-planes tensor, cleared once when (re)allocated: its padding rows stay 0."""
        n = capi.cnn_lp_bytes(channels, zpad, dims, batch) // 2
        t = self._bufs.get(name)
        if t is None or t.numel() != n:
            t = self.torch.zeros(n, dtype=self.torch.bfloat16, device=self.device)
            self._bufs[name] = t
        return t

    def tc_supported(self, dims) -> bool:
        """The tensor-core kernels take z-lines of 32 voxels and n1 % 8 == 0."""
        return int(dims[2]) == 32 and int(dims[1]) % 8 == 0

    def train_step(self, X0, labels, dims, batch: int, lr: float, pos_weight: float,
                   stream=None, tc: bool | None = None):
        """One Adam step on BCE-with-logits; returns the loss tensor (per voxel).

        Runs on the tcgen05 kernels (bpgb_cnn_tc_*) when the volume allows it (tc=None),
        else, or with tc=False, on the mma.sync kernels (bpgb_cnn_conv3d*)."""
        if tc is None:
            tc = self.tc_supported(dims)
        if tc:
            return self._train_step_tc(X0, labels, dims, batch, lr, pos_weight, stream)
        return self._train_step_mma(X0, labels, dims, batch, lr, pos_weight, stream)

    def _train_step_tc(self, X0, labels, dims, batch, lr, pos_weight, stream):
        torch = self.torch
        V = batch * int(np.prod(dims))
        ci = self.in_channels
        dZl = self._lp("dZl", 1, 1, dims, batch)
        dYl = [self._lp(f"dY{i}l", 16, 1, dims, batch) for i in (1, 2, 3)]
        logits = self._buf("Z", (V,), torch.float32)
        loss = self._buf("loss", (V,), torch.float32)
        G = self.G
        nscr = max(capi.cnn_tc_wgrad_scratch_bytes(16, dims, batch),
                   capi.cnn_tc_wgrad_scratch_bytes(ci, dims, batch))
        scr = self._buf("tc_scratch", (nscr // 4,), torch.float32)
        conv, wgrad = capi.cnn_tc_conv3d, capi.cnn_tc_conv3d_wgrad
        ins, Yl = self._forward_tc(X0, dims, batch, logits, stream)
        capi.cnn_tc_bce_grad(logits, labels, dims, batch, pos_weight, 1.0 / V, dZl, loss, stream)
        # backward: weight gradient of layer li, then the input gradient (masked by the
        # ReLU of the layer below)
        grads = [dYl[0], dYl[1], dYl[2], dZl]
        for li in (3, 2, 1, 0):
            cin, cout, _ = self.layers[li]
            wgrad(ins[li], cin, grads[li], cout, dims, batch, scr, nscr, G[li], stream)
            if li > 0:
                conv(grads[li], cout, 1, dims, batch, self.Wtc_b[li], None, cin, False,
                     d_mask=Yl[li - 1], d_Y=dYl[li - 1], out_zpad=1, stream=stream)
        self._adam(lr, stream)
        self.pack_tc(stream)
        self._mma_stale = True
        return loss

    def _adam(self, lr, stream):
        """One Adam step of every layer (the flat buffers) on the gradients in self.G."""
        self.step += 1
        capi.cnn_adam(self.flat_W, self.flat_G, self.flat_M, self.flat_V, self.flat_W.numel(), lr,
                      0.9, 0.999, 1e-8, self.step, stream)

    def _train_step_mma(self, X0, labels, dims, batch, lr, pos_weight, stream):
        torch = self.torch
        V = batch * int(np.prod(dims))
        logits = self.forward(X0, dims, batch, stream=stream, tc=False)
        Y1, Y2, Y3 = self._bufs["Y1"], self._bufs["Y2"], self._bufs["Y3"]
        dZ = self._buf("dZ", (V, 8), torch.bfloat16)
        loss = self._buf("loss", (V,), torch.float32)
        capi.cnn_bce_grad(logits, labels, V, pos_weight, 1.0 / V, dZ, loss, stream)
        dY3 = self._buf("dY3", (V, 16), torch.bfloat16)
        dY2 = self._buf("dY2", (V, 16), torch.bfloat16)
        dY1 = self._buf("dY1", (V, 16), torch.bfloat16)
        G = self.G
        ci = self.in_channels
        nscr = max(capi.cnn_wgrad_scratch_bytes(16, 16, dims, batch),
                   capi.cnn_wgrad_scratch_bytes(ci, 16, dims, batch))
        scr = self._buf("scratch", (nscr // 4,), torch.float32)
        capi.cnn_conv3d_wgrad(Y3, 16, 16, dims, batch, dZ, 8, 1, scr, nscr, G[3], stream)
        capi.cnn_conv3d(dZ, 1, 8, dims, batch, self.Wb[3], 16, False, d_Y=dY3, d_mask=Y3,
                        mask_stride=16, stream=stream)
        capi.cnn_conv3d_wgrad(Y2, 16, 16, dims, batch, dY3, 16, 16, scr, nscr, G[2], stream)
        capi.cnn_conv3d(dY3, 16, 16, dims, batch, self.Wb[2], 16, False, d_Y=dY2, d_mask=Y2,
                        mask_stride=16, stream=stream)
        capi.cnn_conv3d_wgrad(Y1, 16, 16, dims, batch, dY2, 16, 16, scr, nscr, G[1], stream)
        capi.cnn_conv3d(dY2, 16, 16, dims, batch, self.Wb[1], 16, False, d_Y=dY1, d_mask=Y1,
                        mask_stride=16, stream=stream)
        capi.cnn_conv3d_wgrad(X0, ci, ci, dims, batch, dY1, 16, 16, scr, nscr, G[0], stream)
        self._adam(lr, stream)
        self.pack(stream)
        return loss


# ---------------------------------------------------------------- capture geometry

@dataclass
class OctreeGeometry:
    """The octree_256 capture geometry at the fine and coarse resolutions."""
    pairs: np.ndarray
    T: int
    t0: float
    deltaT: float
    fine: tuple
    coarse: tuple
    zero: np.ndarray
    inc_fine: np.ndarray
    inc_coarse: np.ndarray
    volume_position: np.ndarray
    volume_size: np.ndarray
    spec: synthetic.CaptureSpec = field(repr=False)

    @classmethod
    def of(cls, name: str = "octree_256", small: bool = False, **overrides) -> "OctreeGeometry":
        c = synthetic.make_capture(name, seed=0, small=small, render=False, **overrides)
        n = int(c.voxels_per_side[0])
        coarse = n // BLOCK
        # the coarse grid spans the same box: each step x (n - 1) / (coarse - 1), formed in
        # FP64 from the fine steps (as bpgb_octree_create does)
        ic = (np.asarray(c.inc, np.float64).reshape(3, 3) * (n - 1) / (coarse - 1))
        ic = ic.astype(np.float32).reshape(-1)
        return cls(c.pairs, c.T, c.t0, c.deltaT, (n, n, n), (coarse, coarse, coarse), c.zero,
                   c.inc, ic, c.volume_position, c.volume_size, c.spec)


def scene(geo: OctreeGeometry, seed: int):
    """Seeded scene points/albedo of the octree configuration (seed drives the scene)."""
    rng = np.random.default_rng(seed)
    lo = geo.volume_position.astype(np.float64) - geo.spec.volume_edge / 2
    hi = geo.volume_position.astype(np.float64) + geo.spec.volume_edge / 2
    return synthetic.make_scene(geo.spec, rng, lo, hi)


H_TARGET = 16384.0  # FP16 rows: the capture's largest |H| maps to this value


class Reconstructor:
    """Device state for rendering and reconstructing captures of one geometry.

    Rows are stored as `h_dtype` (FP16 by default: each capture divided by
    max|H| / H_TARGET, computed and applied on the device; the volumes are multiplied
    back at the end of each pass)."""

    def __init__(self, geo: OctreeGeometry, device, fine_tile: int | None = 13,
                 h_dtype: int = capi.DTYPE_F16, fine_splits: int = 8, fill: int | None = None,
                 **fine_opt):
        import torch

        self.torch = torch
        self.geo = geo
        self.device = device
        self.h_dtype = h_dtype
        self.stream = torch.cuda.Stream(device=device)
        P = len(geo.pairs)
        self.d_pairs = torch.from_numpy(geo.pairs.view(np.uint8).copy()).to(device)
        self.H = torch.empty((P, geo.T), dtype=torch.float32, device=device)
        self.absmax = torch.ones(1, dtype=torch.float32, device=device)
        if h_dtype == capi.DTYPE_F16:
            self.rows = torch.empty((P, geo.T), dtype=torch.float16, device=device)
        else:
            self.rows = self.H
        self.coarse = torch.empty(geo.coarse, dtype=torch.float32, device=device)
        self.fine = torch.empty(geo.fine, dtype=torch.float32, device=device)
        self.coarse_plan = capi.Plan(geo.pairs, geo.T, geo.coarse, geo.zero, geo.inc_coarse,
                                     geo.t0, geo.deltaT, algo=capi.ALGO_FAST, h_dtype=h_dtype)
        # The fine plan serves both the dense reference (execute) and the block-sparse
        # pass (execute_tiles): FAST arithmetic is tile-relative, so one plan gives
        # bit-identical voxels in both.
        # pair splits: a few hundred to a few thousand selected tiles fill 1-3 waves of
        # CTAs; splitting each tile's pairs over 8 CTAs keeps the last wave short.  Tile
        # preset 13: 8^3 tiles (the CNN's blocks), four per CTA with one producer and
        # stage ring, so an SM holds 24 consumer warps (preset 10, one 8^3 tile per
        # 3-warp CTA: 12).  Measured on the octree_256 scenes: fine pass 2.78 against
        # 2.90 ms, bit-identical voxels.
        opt = dict(algo=capi.ALGO_FAST, pair_splits=fine_splits, h_dtype=h_dtype)
        if fine_tile is not None:
            opt["tile"] = fine_tile
        opt.update(fine_opt)
        self.sparse_plan = capi.Plan(geo.pairs, geo.T, geo.fine, geo.zero, geo.inc_fine, geo.t0,
                                     geo.deltaT, **opt)
        # labels only: the fastest dense configuration (its own tiles)
        self.label_plan = capi.Plan(geo.pairs, geo.T, geo.fine, geo.zero, geo.inc_fine, geo.t0,
                                    geo.deltaT, algo=capi.ALGO_FAST)
        info = self.sparse_plan.info()
        self.tile = tuple(info["tile"])
        self.n_tiles = int(np.prod([-(-f // t) for f, t in zip(geo.fine, self.tile)]))
        self.tile_list = torch.empty(self.n_tiles, dtype=torch.int32, device=device)
        self.tile_count = torch.zeros(1, dtype=torch.int32, device=device)
        self.blocks = geo.coarse
        self.block_max = torch.empty(self.blocks, dtype=torch.float32, device=device)
        # budgeted reconstructions: a second coarse pass at `fill`^3 fills the blocks the
        # fine pass skips, and its detail over the 32^3 pass ranks the blocks
        fill = 2 * geo.coarse[0] if fill is None else int(fill)
        self.fill_dims = (fill, fill, fill)
        n = geo.fine[0]
        inc_fill = (np.asarray(geo.inc_fine, np.float64).reshape(3, 3) * (n - 1) / (fill - 1))
        self.fill_plan = capi.Plan(geo.pairs, geo.T, self.fill_dims, geo.zero,
                                   inc_fill.astype(np.float32).reshape(-1), geo.t0, geo.deltaT,
                                   algo=capi.ALGO_FAST, h_dtype=h_dtype)
        self.fill_vol = torch.empty(self.fill_dims, dtype=torch.float32, device=device)
        self.score = torch.empty(self.blocks, dtype=torch.float32, device=device)
        self.X0 = torch.empty(int(np.prod(geo.coarse)) * 2, dtype=torch.bfloat16, device=device)
        self.logits = torch.empty(int(np.prod(geo.coarse)), dtype=torch.float32, device=device)

    def render(self, points: np.ndarray, albedo: np.ndarray) -> None:
        torch = self.torch
        dp = torch.from_numpy(np.ascontiguousarray(points, np.float32)).to(self.device)
        da = torch.from_numpy(np.ascontiguousarray(albedo, np.float32)).to(self.device)
        capi.synth_render_device(self.d_pairs, len(self.geo.pairs), self.geo.T, self.geo.t0,
                                 self.geo.deltaT, dp, da, len(points), self.H,
                                 stream=self.stream)
        self.ingest()

    def ingest(self) -> None:
        """Stores self.H (FP32) as the plans' row type (synchronous)."""
        if self.h_dtype == capi.DTYPE_F16:
            P, T = self.H.shape
            capi.rows_absmax(self.H, P, T, T, self.absmax, self.stream)
            capi.rows_to_half(self.H, P, T, T, capi.DTYPE_F16, self.rows, T,
                              d_absmax=self.absmax, target=H_TARGET, stream=self.stream)
        self.stream.synchronize()

    def _unscale(self, vol) -> None:
        if self.h_dtype == capi.DTYPE_F16:
            capi.volume_scale(vol, vol.numel(), d_absmax=self.absmax, target=H_TARGET,
                              stream=self.stream)

    def dense(self, out=None):
        """Dense fine pass (synchronous: the result is ready on return)."""
        out = self.fine if out is None else out
        self.sparse_plan.execute(self.rows, out, self.stream)
        self._unscale(out)
        self.stream.synchronize()
        return out

    def computed_mask(self):
        """Bool [fine] mask of the voxels the last reconstruct() backprojected."""
        torch = self.torch
        self.stream.synchronize()
        n = int(self.tile_count.item())
        ids = self.tile_list[:n].long()
        nt = [-(-f // t) for f, t in zip(self.geo.fine, self.tile)]
        tz = ids % nt[2]
        tx = (ids // nt[2]) % nt[0]
        ty = ids // (nt[2] * nt[0])
        tmask = torch.zeros(nt, dtype=torch.bool, device=self.device)
        tmask[tx, ty, tz] = True
        m = tmask.repeat_interleave(self.tile[0], 0).repeat_interleave(self.tile[1], 1)
        m = m.repeat_interleave(self.tile[2], 2)
        return m[:self.geo.fine[0], :self.geo.fine[1], :self.geo.fine[2]]

    def coarse_pass(self):
        """Coarse pass (synchronous)."""
        self.coarse_plan.execute(self.rows, self.coarse, self.stream)
        self.stream.synchronize()
        return self.coarse  # in stored-row units (the CNN input is scale-free)

    def labels_from_dense(self, dense) -> "torch.Tensor":
        """Block maxima of the filtered dense volume F = -lap(D) divided by max(F)
        ([32^3] FP32); a block is occupied where this reaches tau."""
        filt = self._filtered(dense)
        capi.block_max(filt, self.geo.fine, BLOCK, self.block_max, self.stream)
        self.stream.synchronize()
        return self.block_max / filt.max()

    def _filtered(self, dense):
        if getattr(self, "filt", None) is None:
            self.filt = self.torch.empty(self.geo.fine, dtype=self.torch.float32,
                                         device=self.device)
        capi.laplacian7(dense, self.geo.fine, self.filt, self.stream)
        self.stream.synchronize()
        return self.filt

    def occupied_voxels(self, dense, tau: float = TAU):
        """Bool [fine] mask: F = -lap(dense) >= tau max(F)."""
        f = self._filtered(dense)
        return f >= tau * f.max()

    def reconstruct(self, model: OccupancyCNN, logit_lo: float, out=None,
                    budget: float = 0.0):
        """Steps 1-4 of the module docstring on self.H, queued on self.stream (the
        caller synchronises); returns the fine volume.

        budget > 0: a budgeted reconstruction.  The fill comes from the second coarse pass
        (`fill`^3), and the fine pass computes the round(budget x blocks) blocks ranked
        first -- the CNN's blocks (p >= p_lo) ahead of all others, then by the detail the
        finer coarse pass adds over the 32^3 one (bpgb_block_detail), the predictor of
        the fill's error; the k-th score is found on the device."""
        out = self.fine if out is None else out
        s = self.stream
        self.coarse_plan.execute(self.rows, self.coarse, s)
        model.features(self.coarse, self.geo.coarse, 1, self.X0, s)
        model.forward(self.X0, self.geo.coarse, 1, logits=self.logits, stream=s)
        if budget > 0.0:
            self.fill_plan.execute(self.rows, self.fill_vol, s)
            capi.upsample_trilinear(self.fill_vol, self.fill_dims, out, self.geo.fine, s)
            capi.block_detail(self.coarse, self.geo.coarse, self.fill_vol, self.fill_dims,
                              self.geo.fine, BLOCK, self.score, d_logits=self.logits,
                              logit_lo=logit_lo, stream=s)
            k = int(round(min(budget, 1.0) * int(np.prod(self.blocks))))
            self.sparse_plan.select_tiles_topk(self.score, self.blocks, BLOCK, k, self.tile_list,
                                               self.tile_count, s)
        else:
            capi.upsample_trilinear(self.coarse, self.geo.coarse, out, self.geo.fine, s)
            self.sparse_plan.select_tiles(self.logits, self.blocks, BLOCK, logit_lo,
                                          self.tile_list, self.tile_count, s)
        self.sparse_plan.execute_tiles(self.rows, out, self.tile_list, self.tile_count,
                                       self.n_tiles, s)
        self._unscale(out)
        return out

    def dense_for_labels(self, out=None):
        """Dense fine pass with the label plan (synchronous)."""
        out = self.fine if out is None else out
        self.label_plan.execute(self.H, out, self.stream)
        self.stream.synchronize()
        return out

    def close(self):
        for p in (self.coarse_plan, self.sparse_plan, self.label_plan, self.fill_plan):
            p.close()


def logit(p: float) -> float:
    return math.log(p / (1.0 - p))


# ---------------------------------------------------------------- training data

def make_training_set(rec: Reconstructor, n: int, seed0: int, log=print):
    """Renders n seeded scenes, returns (coarse [n, 32^3] FP32, block_norm [n, 32^3] FP32):
    the coarse pass and the dense pass's block maxima over its maximum."""
    torch = rec.torch
    nc = int(np.prod(rec.geo.coarse))
    coarse = torch.empty((n, nc), dtype=torch.float32, device=rec.device)
    bnorm = torch.empty((n, nc), dtype=torch.float32, device=rec.device)
    t = time.perf_counter()
    for i in range(n):
        pts, alb = scene(rec.geo, seed0 + i)
        rec.render(pts, alb)
        coarse[i] = rec.coarse_pass().reshape(-1)
        bnorm[i] = rec.labels_from_dense(rec.dense_for_labels()).reshape(-1)
        if log and (i + 1) % 200 == 0:
            log(f"  scenes {i + 1}/{n} ({time.perf_counter() - t:.1f} s)")
    rec.stream.synchronize()
    return coarse, bnorm


def train(model: OccupancyCNN, coarse, bnorm, dims, epochs: int = 30, batch: int = 16,
          lr: float = 2e-3, tau: float = TAU, seed: int = 0, max_pos_weight: float = 50.0,
          log=print) -> list[float]:
    torch = model.torch
    n = coarse.shape[0]
    nc = coarse.shape[1]
    labels = (bnorm >= tau).to(torch.uint8)
    pos = float(labels.float().mean().item())
    pos_weight = min(max_pos_weight, (1.0 - pos) / max(pos, 1e-6))
    X = model.features(coarse, dims, n).reshape(n, -1)
    rng = np.random.default_rng(seed)
    hist = []
    for ep in range(epochs):
        order = rng.permutation(n)
        rate = lr * 0.5 * (1.0 + math.cos(math.pi * ep / epochs))
        tot = 0.0
        for b0 in range(0, n - batch + 1, batch):
            idx = torch.from_numpy(order[b0:b0 + batch]).to(model.device)
            xb = X.index_select(0, idx).reshape(-1).contiguous()
            yb = labels.index_select(0, idx).reshape(-1).contiguous()
            loss = model.train_step(xb, yb, dims, batch, rate, pos_weight)
            tot += float(loss.sum().item())
        steps = max(1, n // batch)
        hist.append(tot / steps)
        if log:
            log(f"  epoch {ep + 1}/{epochs} loss {hist[-1]:.4f} (pos {pos:.4f}, w {pos_weight:.1f})")
    return hist


def block_scores(model: OccupancyCNN, coarse, dims):
    """Sigmoid scores [n, 32^3] of the model over a set of coarse volumes."""
    torch = model.torch
    n, nc = coarse.shape
    X = model.features(coarse, dims, n).reshape(n, -1)
    out = torch.empty((n, nc), dtype=torch.float32, device=model.device)
    for i in range(n):
        model.forward(X[i], dims, 1, logits=out[i])
    torch.cuda.synchronize()
    return torch.sigmoid(out)


def calibrate(scores, bnorm, tau: float = TAU, recall: float = 0.995) -> float:
    """Largest p_lo whose block recall of occupied blocks on (scores, bnorm) >= recall."""
    occ = bnorm >= tau
    s = scores[occ]
    if s.numel() == 0:
        return 0.5
    q = float(np.quantile(s.float().cpu().numpy(), 1.0 - recall))
    return max(min(q, 0.5), 1e-6)


def metrics(out, dense, computed, occ_vox, block: int = BLOCK) -> dict:
    """Octree volume vs a dense reference (same grid): occupied-voxel recall (occupied
    voxels, `occ_vox`, that the octree backprojected at full resolution, `computed`),
    rel-L2 over all voxels and over occupied blocks, PSNR, computed fraction."""
    import torch as T

    d = dense.double()
    o = out.double()
    mx = float(d.max())
    exact = computed
    n = d.shape[0] // block
    bl = occ_vox.reshape(n, block, n, block, n, block).any(dim=5).any(dim=3).any(dim=1)
    occ_blocks = bl.repeat_interleave(block, 0).repeat_interleave(block, 1).repeat_interleave(block, 2)
    diff = o - d
    res = {
        "occupied_voxels": int(occ_vox.sum()),
        "recall": float((exact & occ_vox).sum()) / max(1, int(occ_vox.sum())),
        "rel_l2": float(T.linalg.vector_norm(diff) / T.linalg.vector_norm(d)),
        "rel_l2_occupied_blocks": float(T.linalg.vector_norm(diff[occ_blocks]) /
                                        max(1e-300, float(T.linalg.vector_norm(d[occ_blocks])))),
        "psnr_db": float(10.0 * math.log10(mx * mx / max(1e-300, float((diff * diff).mean())))),
        "computed_fraction": float(computed.float().mean()),
    }
    return res


# ---------------------------------------------------------------- phasor fields

class PhasorOctree:
    """Block-sparse phasor-field reconstruction: the reference's phasor path with octree
    access (backproject.hpp:1012-1018, CPU only there, refining a threshold octree and
    passing the uncropped t0 with cropped rows).  Here: the complex FAST pass on the 8x
    coarser grid over the same box, block scores |coarse| (one coarse voxel per 8^3 fine
    block), a full-resolution complex pass over the blocks scoring >= rho * max, zeros
    elsewhere.  Phasor-field volumes are sharp (no low-frequency bump), so the coarse
    magnitude marks the objects without a learned proposal.  t0 is the caller's (pass the
    chunk t0 of cropped rows)."""

    def __init__(self, pairs, T: int, voxels_per_side, zero, inc, t0: float, deltaT: float,
                 device, rho: float = 0.1, fine_tile: int = 10, fine_splits: int = 4,
                 h_pitch: int = 0):
        import torch

        self.torch = torch
        self.device = device
        self.rho = float(rho)
        self.fine = tuple(int(v) for v in voxels_per_side)
        assert all(v % BLOCK == 0 and v >= 2 * BLOCK for v in self.fine), self.fine
        self.coarse = tuple(v // BLOCK for v in self.fine)
        n = np.asarray(self.fine, np.float64)
        ic = (np.asarray(inc, np.float64).reshape(3, 3) * ((n - 1) / (n // BLOCK - 1))[:, None])
        ic = ic.astype(np.float32).reshape(-1)
        common = dict(algo=capi.ALGO_FAST, h_dtype=capi.DTYPE_C64, h_pitch=h_pitch)
        self.coarse_plan = capi.Plan(pairs, T, self.coarse, zero, ic, t0, deltaT, **common)
        self.fine_plan = capi.Plan(pairs, T, self.fine, zero, inc, t0, deltaT, tile=fine_tile,
                                   pair_splits=fine_splits, **common)
        info = self.fine_plan.info()
        self.tile = tuple(info["tile"])
        self.n_tiles = int(np.prod([-(-f // t) for f, t in zip(self.fine, self.tile)]))
        nc = int(np.prod(self.coarse))
        self.coarse_vol = torch.empty(nc, dtype=torch.complex64, device=device)
        self.mag = torch.empty(nc, dtype=torch.float32, device=device)
        self.mx = torch.empty(1, dtype=torch.float32, device=device)
        self.tile_list = torch.empty(self.n_tiles, dtype=torch.int32, device=device)
        self.tile_count = torch.zeros(1, dtype=torch.int32, device=device)

    def dense(self, d_Hc, out, stream=None) -> None:
        """The full-resolution complex pass of the same plan (the reference result)."""
        self.fine_plan.execute(d_Hc, out, stream)

    def reconstruct(self, d_Hc, out, stream=None) -> int:
        """Complex volume of the selected blocks (zeros elsewhere) into `out`; returns the
        number of fine tiles computed (one host read of the coarse maximum)."""
        nc = self.mag.numel()
        self.coarse_plan.execute(d_Hc, self.coarse_vol, stream)
        capi.complex_abs(self.coarse_vol, nc, self.mag, stream)
        capi.rows_absmax(self.mag, 1, nc, nc, self.mx, stream)
        s = self.torch.cuda.current_stream() if stream is None else stream
        s.synchronize()
        threshold = self.rho * float(self.mx.item())
        with self.torch.cuda.stream(s):
            out.zero_()
        self.fine_plan.select_tiles(self.mag, self.coarse, BLOCK, threshold, self.tile_list,
                                    self.tile_count, stream)
        self.fine_plan.execute_tiles(d_Hc, out, self.tile_list, self.tile_count, self.n_tiles,
                                     stream)
        s.synchronize()
        return int(self.tile_count.item())

    def close(self) -> None:
        self.coarse_plan.close()
        self.fine_plan.close()
