"""Learned-octree kernels against plain PyTorch FP32 references of the same ops, and the
block-sparse reconstruction against the dense FAST pass.

Tolerances: BF16 outputs (conv3d forward / backward-data) within 1e-2 relative of the
FP32 reference on BF16-exact inputs (one BF16 rounding of an FP32 sum); FP32 outputs
(weight gradients) within 1e-3; the block-sparse fine pass equals the dense pass
bit for bit on every tile it computes (same kernel arithmetic per tile)."""
from __future__ import annotations

import math

import numpy as np
import pytest

from backprojector_gb300 import capi, octree, synthetic
from oracle import oracle

pytestmark = pytest.mark.gpu

CONV_CASES = [(1, 16, True, 16), (2, 16, True, 16), (16, 16, True, 16), (16, 1, False, 8)]


def bf16_exact(t):
    return t.bfloat16().float()


def torch_weight(Wm, cin, cout):
    import torch

    w = Wm[:27 * cin].reshape(3, 3, 3, cin, cout).permute(4, 3, 0, 1, 2).contiguous()
    b = Wm[27 * cin].clone()
    return w, b


def random_master(cin, cout, seed, device):
    import torch

    g = torch.Generator().manual_seed(seed)
    kp = capi.cnn_kp(cin)
    W = torch.zeros((kp, cout))
    W[:27 * cin + 1] = torch.randn((27 * cin + 1, cout), generator=g) * 0.3
    return bf16_exact(W).to(device)


@pytest.mark.parametrize("cin,cout,relu,np_", CONV_CASES)
def test_conv3d_forward_vs_torch(cuda, cin, cout, relu, np_):
    import torch
    import torch.nn.functional as F

    dims, batch = (6, 5, 7), 2
    g = torch.Generator().manual_seed(cin * 100 + cout)
    X = bf16_exact(torch.randn((batch, *dims, cin), generator=g))
    W = random_master(cin, cout, 7, cuda)
    Wt = torch.empty((np_, capi.cnn_kp(cin)), dtype=torch.bfloat16, device=cuda)
    capi.cnn_pack_weights(W, cin, cout, np_, Wt)
    dX = X.reshape(-1, cin).to(cuda).bfloat16().contiguous()
    V = batch * int(np.prod(dims))
    Y = torch.zeros((V, np_), dtype=torch.bfloat16, device=cuda)
    Yf = torch.zeros(V, device=cuda)
    capi.cnn_conv3d(dX, cin, cin, dims, batch, Wt, np_, relu, d_Y=Y, d_Yf=Yf)
    torch.cuda.synchronize()
    w, b = torch_weight(W.cpu(), cin, cout)
    ref = F.conv3d(X.permute(0, 4, 1, 2, 3), w, b, padding=1)
    if relu:
        ref = ref.clamp_min(0)
    ref = ref.permute(0, 2, 3, 4, 1).reshape(V, cout)
    got = Y.float().cpu()[:, :cout]
    assert torch.allclose(got, ref, rtol=1e-2, atol=1e-2 * float(ref.abs().max())), \
        float((got - ref).abs().max())
    assert torch.allclose(Yf.cpu(), ref[:, 0], rtol=1e-5, atol=1e-4 * float(ref.abs().max()))
    if np_ > cout:
        assert torch.all(Y.float().cpu()[:, cout:] == (0 if not relu else 0))


@pytest.mark.parametrize("cin,cout,relu,np_", CONV_CASES)
def test_conv3d_weight_and_input_gradients_vs_torch(cuda, cin, cout, relu, np_):
    import torch
    import torch.nn.functional as F

    dims, batch = (5, 6, 4), 3
    V = batch * int(np.prod(dims))
    g = torch.Generator().manual_seed(5 + cin + cout)
    X = bf16_exact(torch.randn((batch, *dims, cin), generator=g))
    dY = bf16_exact(torch.randn((batch, *dims, cout), generator=g))
    W = random_master(cin, cout, 11, cuda)
    # weight gradient (bias row included)
    dX = X.reshape(V, cin).to(cuda).bfloat16().contiguous()
    dYp = torch.zeros((V, np_), dtype=torch.bfloat16, device=cuda)
    dYp[:, :cout] = dY.reshape(V, cout).to(cuda).bfloat16()
    nscr = capi.cnn_wgrad_scratch_bytes(cin, np_, dims, batch)
    scr = torch.empty(nscr // 4, device=cuda)
    dW = torch.full(tuple(W.shape), float("nan"), device=cuda)
    capi.cnn_conv3d_wgrad(dX, cin, cin, dims, batch, dYp, np_, cout, scr, nscr, dW)
    torch.cuda.synchronize()
    w, b = torch_weight(W.cpu(), cin, cout)
    xt = X.permute(0, 4, 1, 2, 3).clone().requires_grad_(True)
    wt = w.clone().requires_grad_(True)
    bt = b.clone().requires_grad_(True)
    out = F.conv3d(xt, wt, bt, padding=1)
    out.backward(dY.permute(0, 4, 1, 2, 3))
    ref_w = wt.grad.permute(2, 3, 4, 1, 0).reshape(27 * cin, cout)
    got = dW.cpu()
    scale = float(ref_w.abs().max())
    assert torch.allclose(got[:27 * cin], ref_w, rtol=1e-3, atol=1e-4 * scale)
    assert torch.allclose(got[27 * cin], bt.grad, rtol=1e-3, atol=1e-4 * float(bt.grad.abs().max()))
    assert torch.all(got[27 * cin + 1:] == 0)
    # input gradient: the forward kernel on dY with the backward weights and a ReLU mask
    if cin == 16:
        Wt = torch.empty((np_, capi.cnn_kp(cin)), dtype=torch.bfloat16, device=cuda)
        Wb = torch.empty((16, capi.cnn_kp(cout)), dtype=torch.bfloat16, device=cuda)
        capi.cnn_pack_weights(W, cin, cout, np_, Wt, 16, Wb)
        mask = bf16_exact(torch.randn((V, 16), generator=g)).to(cuda).bfloat16()
        gX = torch.zeros((V, 16), dtype=torch.bfloat16, device=cuda)
        capi.cnn_conv3d(dYp, cout, np_, dims, batch, Wb, 16, False, d_Y=gX, d_mask=mask,
                        mask_stride=16)
        torch.cuda.synchronize()
        ref_x = xt.grad.permute(0, 2, 3, 4, 1).reshape(V, cin) * (mask.float().cpu() > 0)
        gotx = gX.float().cpu()
        assert torch.allclose(gotx, ref_x, rtol=1e-2, atol=1e-2 * float(ref_x.abs().max()))


def test_bce_and_adam_vs_torch(cuda):
    import torch

    n = 1000
    g = torch.Generator().manual_seed(3)
    z = (torch.randn(n, generator=g) * 3).to(cuda)
    y = (torch.rand(n, generator=g) < 0.2).to(torch.uint8).to(cuda)
    dZ = torch.empty((n, 8), dtype=torch.bfloat16, device=cuda)
    loss = torch.empty(n, device=cuda)
    capi.cnn_bce_grad(z, y, n, 4.0, 1.0 / n, dZ, loss)
    torch.cuda.synchronize()
    zr = z.cpu().clone().requires_grad_(True)
    w = torch.where(y.cpu() > 0, 4.0, 1.0)
    lr_ = (w * torch.nn.functional.binary_cross_entropy_with_logits(
        zr, y.cpu().float(), reduction="none")) / n
    lr_.sum().backward()
    assert torch.allclose(loss.cpu(), lr_.detach(), rtol=1e-5, atol=1e-9)
    assert torch.allclose(dZ[:, 0].float().cpu(), zr.grad, rtol=1e-2, atol=1e-6)
    assert torch.all(dZ[:, 1:].float() == 0)
    # Adam, three steps against torch.optim.Adam
    p0 = torch.randn(300, generator=g)
    p = p0.clone().to(cuda)
    m = torch.zeros_like(p)
    v = torch.zeros_like(p)
    ref = p0.clone().requires_grad_(True)
    opt = torch.optim.Adam([ref], lr=1e-2, betas=(0.9, 0.999), eps=1e-8)
    for step in range(1, 4):
        grad = torch.randn(300, generator=g)
        capi.cnn_adam(p, grad.to(cuda), m, v, 300, 1e-2, 0.9, 0.999, 1e-8, step)
        ref.grad = grad.clone()
        opt.step()
    torch.cuda.synchronize()
    assert torch.allclose(p.cpu(), ref.detach(), rtol=1e-5, atol=1e-6)


def test_device_renderer_matches_host_renderer(cuda):
    import torch

    c = synthetic.make_capture("octree_256", seed=3, small=True)
    H = torch.empty((c.P, c.T + 64), device=cuda)
    dp = torch.from_numpy(c.pairs.view(np.uint8).copy()).to(cuda)
    capi.synth_render_device(dp, c.P, c.T, c.t0, c.deltaT, torch.from_numpy(c.points).to(cuda),
                             torch.from_numpy(c.albedo).to(cuda), len(c.points), H, c.T + 64)
    torch.cuda.synchronize()
    got = H.cpu().numpy()
    assert np.all(got[:, c.T:] == 0)
    got = got[:, :c.T]
    # same hits up to FP32 path rounding: totals per pair agree; a hit moves to the next
    # bin when its FP32 path lies within rounding of a bin edge (~1e-4 of 30,000 hits per
    # pair here, each changing two of the pair's 1,024 bins)
    assert np.allclose(got.sum(1), c.H.sum(1), rtol=1e-5)
    changed = np.abs(got - c.H) > 1e-5 * np.abs(c.H).max()
    assert changed.mean() < 1e-2
    assert oracle.rel_l2(got, c.H) < 5e-2
    # deterministic
    H2 = torch.empty_like(H)
    capi.synth_render_device(dp, c.P, c.T, c.t0, c.deltaT, torch.from_numpy(c.points).to(cuda),
                             torch.from_numpy(c.albedo).to(cuda), len(c.points), H2, c.T + 64)
    torch.cuda.synchronize()
    assert torch.equal(H, H2)


@pytest.mark.parametrize("grid_wide", [False, True])
def test_cnn_features_vs_torch(cuda, grid_wide):
    import torch
    import torch.nn.functional as F

    g = torch.Generator().manual_seed(9)
    dims, batch = (6, 7, 5) if not grid_wide else (32, 32, 32), 2
    coarse = torch.rand((batch, *dims), generator=g)
    X = torch.empty((batch * int(np.prod(dims)) * 2,), dtype=torch.bfloat16, device=cuda)
    scr = torch.full((2 * batch,), 7.0, device=cuda) if grid_wide else None
    capi.cnn_features(coarse.to(cuda), dims, batch, X, scr)
    torch.cuda.synchronize()
    got = X.float().cpu().reshape(batch, *dims, 2)
    k = torch.zeros((1, 1, 3, 3, 3))
    for d in ((0, 1, 1), (2, 1, 1), (1, 0, 1), (1, 2, 1), (1, 1, 0), (1, 1, 2)):
        k[0, 0][d] = 1.0
    cnt = F.conv3d(torch.ones((1, 1, *dims)), k, padding=1)[0, 0]
    for b in range(batch):
        c = coarse[b]
        lap = cnt * c - F.conv3d(c[None, None], k, padding=1)[0, 0]
        assert torch.allclose(got[b, ..., 0], (c / c.max()).bfloat16().float())
        ref1 = (lap / lap.abs().max()).bfloat16().float()
        assert torch.allclose(got[b, ..., 1], ref1, atol=1e-2)


def test_laplacian7_vs_torch(cuda):
    import torch
    import torch.nn.functional as F

    g = torch.Generator().manual_seed(4)
    vol = torch.randn((9, 7, 11), generator=g)
    out = torch.empty_like(vol).to(cuda)
    capi.laplacian7(vol.to(cuda), (9, 7, 11), out)
    torch.cuda.synchronize()
    # sum over in-volume neighbours of (c - n): 6-neighbour count x c minus neighbour sum
    ones = torch.ones((1, 1, 9, 7, 11))
    k = torch.zeros((1, 1, 3, 3, 3))
    for d in ((0, 1, 1), (2, 1, 1), (1, 0, 1), (1, 2, 1), (1, 1, 0), (1, 1, 2)):
        k[0, 0][d] = 1.0
    nsum = F.conv3d(vol[None, None], k, padding=1)[0, 0]
    cnt = F.conv3d(ones, k, padding=1)[0, 0]
    ref = cnt * vol - nsum
    assert torch.allclose(out.cpu(), ref, rtol=1e-5, atol=1e-5)


@pytest.mark.parametrize("dtype", ["f16", "bf16"])
def test_rows_to_half_with_device_scale(cuda, dtype):
    import torch

    g = torch.Generator().manual_seed(2)
    H = (torch.rand((37, 100), generator=g) * 1e5).to(cuda)
    H[3, 7] = -2.5e5
    mx = torch.empty(1, device=cuda)
    capi.rows_absmax(H, 37, 90, 100, mx)
    out = torch.full((37, 96), 7.0, dtype=torch.float16 if dtype == "f16" else torch.bfloat16,
                     device=cuda)
    code = capi.DTYPE_F16 if dtype == "f16" else capi.DTYPE_BF16
    capi.rows_to_half(H, 37, 90, 100, code, out, 96, d_absmax=mx, target=16384.0)
    vol = H[:, :90].clone()
    capi.volume_scale(vol, vol.numel(), d_absmax=mx, target=16384.0)
    torch.cuda.synchronize()
    assert float(mx) == 2.5e5
    inv = 1.0 / torch.tensor(2.5e5 / 16384.0, dtype=torch.float32)
    ref = (H[:, :90].cpu() * inv).to(out.dtype)
    assert torch.equal(out[:, :90].cpu(), ref)
    assert torch.all(out[:, 90:] == 0)
    assert torch.allclose(vol, H[:, :90] * (2.5e5 / 16384.0), rtol=1e-6)


def test_block_max_and_upsample(cuda):
    import torch
    import torch.nn.functional as F

    g = torch.Generator().manual_seed(1)
    vol = torch.randn((20, 16, 12), generator=g)
    out = torch.empty((3, 2, 2), device=cuda)
    capi.block_max(vol.to(cuda), (20, 16, 12), 8, out)
    torch.cuda.synchronize()
    ref = F.max_pool3d(F.pad(vol[None, None], (0, 4, 0, 0, 0, 4), value=-1e30), 8)[0, 0]
    assert torch.equal(out.cpu(), ref)
    coarse = torch.randn((4, 5, 3), generator=g)
    fine = torch.empty((10, 13, 7), device=cuda)
    capi.upsample_trilinear(coarse.to(cuda), (4, 5, 3), fine, (10, 13, 7))
    torch.cuda.synchronize()
    ref = F.interpolate(coarse[None, None], size=(10, 13, 7), mode="trilinear",
                        align_corners=True)[0, 0]
    assert torch.allclose(fine.cpu(), ref, rtol=1e-5, atol=1e-5)


@pytest.mark.parametrize("tile", [10, 11, 12, 13])
def test_small_tile_presets_vs_oracle(cuda, tile):
    import torch

    c = synthetic.make_capture("octree_256", seed=5, small=True)
    ref = oracle.bp_gpu_f64(c.H, c.pairs, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT)
    dH = torch.from_numpy(c.H).to(cuda)
    dV = torch.empty(tuple(int(v) for v in c.voxels_per_side), device=cuda)
    with capi.Plan(c.pairs, c.T, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT,
                   algo=capi.ALGO_FAST, tile=tile, checked=1) as p:
        p.execute(dH, dV)
        assert p.check() == 0
        assert p.info()["threads"] in (96, 160, 288)
    assert oracle.rel_l2(dV.cpu().numpy(), ref) < 5e-3


@pytest.mark.parametrize("tile,splits", [(0, 1), (10, 1), (10, 2), (11, 3), (0, 4), (13, 1),
                                         (13, 3)])
def test_tile_list_execution_matches_dense(cuda, tile, splits):
    import torch

    c = synthetic.make_capture("octree_256", seed=6, small=True)
    dH = torch.from_numpy(c.H).to(cuda)
    N = tuple(int(v) for v in c.voxels_per_side)
    dense = torch.empty(N, device=cuda)
    with capi.Plan(c.pairs, c.T, N, c.zero, c.inc, c.t0, c.deltaT, algo=capi.ALGO_FAST,
                   tile=tile, pair_splits=splits) as p:
        p.execute(dH, dense)
        info = p.info()
        assert info["pair_splits"] == splits
        td = info["tile"]
        nt = [-(-n // t) for n, t in zip(N, td)]
        ntiles = int(np.prod(nt))
        # score blocks: every other 8^3 block
        nb = [n // 8 for n in N]
        score = torch.zeros(nb, device=cuda)
        score.view(-1)[::2] = 1.0
        lst = torch.empty(ntiles, dtype=torch.int32, device=cuda)
        cnt = torch.zeros(1, dtype=torch.int32, device=cuda)
        p.select_tiles(score, nb, 8, 0.5, lst, cnt)
        out = torch.full(N, float("nan"), device=cuda)
        p.execute_tiles(dH, out, lst, cnt, ntiles)
        p.check()
    n_sel = int(cnt.item())
    assert 0 < n_sel <= ntiles
    sel = sorted(lst[:n_sel].cpu().tolist())
    assert len(set(sel)) == n_sel
    o, d = out.cpu().numpy(), dense.cpu().numpy()
    computed = ~np.isnan(o)
    # computed voxels = exactly the selected tiles, bit-identical to the dense pass
    mask = np.zeros(N, bool)
    for t in sel:
        tz = t % nt[2]
        tx = (t // nt[2]) % nt[0]
        ty = t // (nt[2] * nt[0])
        mask[tx * td[0]:(tx + 1) * td[0], ty * td[1]:(ty + 1) * td[1], tz * td[2]:(tz + 1) * td[2]] = True
    assert np.array_equal(computed, mask)
    assert np.array_equal(o[mask], d[mask])
    # every selected tile overlaps a scored block, every scored block is covered
    sc = score.cpu().numpy().repeat(8, 0).repeat(8, 1).repeat(8, 2) > 0.5
    assert np.all(mask[sc])


@pytest.mark.parametrize("fine_tile", [10, 13])
def test_octree_pipeline_limits(cuda, fine_tile):
    """Untrained model: p_lo = 0 computes every block (equals dense); p_lo -> 1 computes
    none (the trilinear fill of the coarse pass).  One 8^3 tile per CTA (preset 10) and
    four (preset 13)."""
    import torch

    geo = octree.OctreeGeometry.of("octree_256", small=True)
    rec = octree.Reconstructor(geo, cuda, fine_tile=fine_tile)
    model = octree.OccupancyCNN(cuda, seed=1)
    pts, alb = octree.scene(geo, 7)
    rec.render(pts, alb)
    dense = rec.dense().clone()
    out = rec.reconstruct(model, -1e30)
    rec.stream.synchronize()
    out = out.clone()
    assert torch.equal(out, dense)
    m = octree.metrics(out, dense, rec.computed_mask(), rec.occupied_voxels(dense))
    assert m["recall"] == 1.0 and m["rel_l2"] == 0.0 and m["computed_fraction"] == 1.0
    out2 = rec.reconstruct(model, 1e30)
    rec.stream.synchronize()
    out2 = out2.clone()
    assert not rec.computed_mask().any()
    fill = torch.empty_like(dense)
    capi.upsample_trilinear(rec.coarse, geo.coarse, fill, geo.fine, rec.stream)
    rec._unscale(fill)
    rec.stream.synchronize()
    assert torch.equal(out2, fill)
    rec.close()


def test_cnn_training_reduces_loss(cuda):
    import torch

    model = octree.OccupancyCNN(cuda, seed=0)
    dims, n = (8, 8, 8), 8
    g = torch.Generator().manual_seed(0)
    coarse = torch.rand((n, 512), generator=g).to(cuda)
    bnorm = coarse.clone()  # the label is a threshold of the input itself
    hist = octree.train(model, coarse, bnorm, dims, epochs=40, batch=4, lr=5e-3, tau=0.7,
                        log=None)
    assert hist[-1] < 0.5 * hist[0], hist


def test_trained_model_full_size_recall(cuda):
    """The committed CNN on two held-out full-size octree_256 scenes: >= 99% of the
    occupied voxels are backprojected at full resolution, from < 15% of the blocks, and
    those voxels equal the dense pass."""
    import torch

    model, state = octree.OccupancyCNN.load(cuda)
    geo = octree.OctreeGeometry.of("octree_256")
    rec = octree.Reconstructor(geo, cuda)
    lo = octree.logit(float(state["p_lo"]))
    for seed in (3_000_001, 3_000_002):
        rec.render(*octree.scene(geo, seed))
        dense = rec.dense().clone()
        out = rec.reconstruct(model, lo)
        rec.stream.synchronize()
        out = out.clone()
        comp = rec.computed_mask()
        m = octree.metrics(out, dense, comp, rec.occupied_voxels(dense))
        assert m["recall"] >= 0.99, m
        assert m["computed_fraction"] < 0.15, m
        assert torch.equal(out[comp], dense[comp])
        # occupied voxels of the octree volume against the FP64 oracle (256-voxel sample)
        occ = (rec.occupied_voxels(dense) & comp).reshape(-1)
        ids_all = torch.nonzero(occ).reshape(-1).cpu().numpy()
        ids = np.sort(np.random.default_rng(seed).choice(ids_all, size=min(256, len(ids_all)),
                                                         replace=False))
        ref = oracle.bp_gpu_f64(rec.H.cpu().numpy(), geo.pairs, geo.fine, geo.zero, geo.inc_fine,
                                geo.t0, geo.deltaT, voxels=ids)
        got = out.reshape(-1)[torch.from_numpy(ids).to(cuda)].double().cpu().numpy()
        err = float(np.linalg.norm(got - ref) / np.linalg.norm(ref))
        print(f"\n[octree_256 seed {seed}] recall {m['recall']:.5f} computed "
              f"{m['computed_fraction']:.4f} occupied-voxel rel-L2 vs FP64 oracle {err:.2e}")
        assert err <= 1e-3
    rec.close()


def test_native_octree_matches_python_pipeline(cuda):
    """bpgb_octree_* (one native object) against the Python Reconstructor on a full-size
    held-out scene.  Both stage FP16 rows the same way, derive the 32^3 grid the same way
    and run the same plans and CNN kernels, so the volumes are identical; backprojected
    occupied voxels equal the dense pass."""
    import torch

    model, state = octree.OccupancyCNN.load(cuda)
    geo = octree.OctreeGeometry.of("octree_256")
    rec = octree.Reconstructor(geo, cuda)
    rec.render(*octree.scene(geo, 3_000_003))
    dense = rec.dense().clone()
    py = rec.reconstruct(model, octree.logit(float(state["p_lo"])))
    rec.stream.synchronize()
    py = py.clone()
    with capi.NativeOctree(geo.pairs, geo.T, geo.fine, geo.zero, geo.inc_fine, geo.t0,
                           geo.deltaT, octree.WEIGHTS, h_dtype=capi.DTYPE_F16) as nat:
        info = nat.info()
        assert info["coarse"] == list(geo.coarse) and info["tile"] == [8, 8, 8]
        out = torch.empty_like(dense)
        nat.reconstruct(rec.H, out)
        n_sel = nat.selected()
        host = nat.reconstruct_host(rec.H.cpu().numpy())
    assert np.array_equal(host, out.cpu().numpy())
    assert torch.equal(out, py)
    occ = rec.occupied_voxels(dense)
    recall = ((out == dense) & occ).sum().item() / occ.sum().item()
    assert recall >= 0.99
    assert 0 < n_sel < 0.15 * info["tiles"]
    rec.close()


@pytest.mark.parametrize("splits,h_dtype", [(1, capi.DTYPE_F32), (2, capi.DTYPE_F16),
                                             (3, capi.DTYPE_BF16)])
def test_grouped_tile_list_ragged(cuda, splits, h_dtype):
    """Four 8^3 tiles per CTA (preset 13) over a list whose length is no multiple of four:
    a count above max_tiles is clamped to it, an entry outside the volume is skipped, the
    entries past max_tiles stay untouched, and every listed tile equals the dense pass of
    the same plan bit for bit (FP32, FP16 and BF16 rows)."""
    import torch

    c = synthetic.make_capture("octree_256", seed=7, small=True)
    H = torch.from_numpy(c.H).to(cuda)
    opt = dict(algo=capi.ALGO_FAST, tile=13, pair_splits=splits, h_dtype=h_dtype)
    if h_dtype == capi.DTYPE_F16:
        H = H.half()
    elif h_dtype == capi.DTYPE_BF16:
        H = H.bfloat16()
    N = tuple(int(v) for v in c.voxels_per_side)
    dense = torch.empty(N, device=cuda)
    with capi.Plan(c.pairs, c.T, N, c.zero, c.inc, c.t0, c.deltaT, **opt) as p:
        info = p.info()
        assert info["threads"] == 288 and list(info["tile"]) == [8, 8, 8]
        p.execute(H, dense)
        nt = [-(-n // 8) for n in N]
        ntiles = int(np.prod(nt))
        ids = [5, ntiles + 3, 17, 2, ntiles - 1, 40, 41, 9, 11, 30]
        lst = torch.tensor(ids, dtype=torch.int32, device=cuda)
        cnt = torch.tensor([12], dtype=torch.int32, device=cuda)
        out = torch.full(N, float("nan"), device=cuda)
        p.execute_tiles(H, out, lst, cnt, 9)
        assert p.check() == 0
    o, d = out.cpu().numpy(), dense.cpu().numpy()
    mask = np.zeros(N, bool)
    for t in ids[:9]:
        if t >= ntiles:
            continue
        tz, tx, ty = t % nt[2], (t // nt[2]) % nt[0], t // (nt[2] * nt[0])
        mask[tx * 8:(tx + 1) * 8, ty * 8:(ty + 1) * 8, tz * 8:(tz + 1) * 8] = True
    assert np.array_equal(~np.isnan(o), mask)
    assert np.array_equal(o[mask], d[mask])


@pytest.mark.parametrize("h_dtype", [capi.DTYPE_C64, capi.DTYPE_C32])
def test_complex_tile_list_with_splits_matches_dense(cuda, h_dtype):
    """Complex rows (complex64 and FP16 pairs) through tile-list launches with pair splits:
    the tile-local complex partial sums and their reduction give the dense pass's values
    bit for bit on every selected tile."""
    import torch

    c = synthetic.make_capture("phasor_128", seed=4, small=True)
    Hc = oracle.phasor_pulse(c.H, c.wavelength, c.deltaT).astype(np.complex64)
    opt = dict(algo=capi.ALGO_FAST, tile=10, pair_splits=3, h_dtype=h_dtype)
    if h_dtype == capi.DTYPE_C32:
        flat = Hc.view(np.float32)
        scale = float(np.abs(flat).max()) / 16384.0
        dH = torch.from_numpy(flat / np.float32(scale)).to(cuda).half()
        opt["h_scale"] = scale
    else:
        dH = torch.from_numpy(Hc).to(cuda)
    N = tuple(int(v) for v in c.voxels_per_side)
    dense = torch.empty(N, dtype=torch.complex64, device=cuda)
    with capi.Plan(c.pairs, c.T, N, c.zero, c.inc, c.t0, c.deltaT, **opt) as p:
        p.execute(dH, dense)
        td = p.info()["tile"]
        nt = [-(-n // t) for n, t in zip(N, td)]
        ntiles = int(np.prod(nt))
        lst = torch.arange(0, ntiles, 2, dtype=torch.int32, device=cuda)
        cnt = torch.tensor([lst.numel()], dtype=torch.int32, device=cuda)
        out = torch.full(N, complex(float("nan"), float("nan")), dtype=torch.complex64,
                         device=cuda)
        p.execute_tiles(dH, out, lst, cnt, ntiles)
        p.check()
    o, d = out.cpu().numpy(), dense.cpu().numpy()
    mask = np.zeros(N, bool)
    for t in range(0, ntiles, 2):
        tz = t % nt[2]
        tx = (t // nt[2]) % nt[0]
        ty = t // (nt[2] * nt[0])
        mask[tx * td[0]:(tx + 1) * td[0], ty * td[1]:(ty + 1) * td[1], tz * td[2]:(tz + 1) * td[2]] = True
    assert np.array_equal(~np.isnan(o.real), mask)
    assert np.array_equal(o[mask], d[mask])


def test_phasor_octree_full_size(cuda):
    """Block-sparse phasor fields on the full phasor capture (128^3, 16,384 pairs, T =
    4096 complex rows): the blocks whose coarse magnitude reaches 0.1 of its maximum are
    backprojected at full resolution and equal the dense complex pass; >= 99% of the voxels
    with |V| >= 0.5 max|V| are among them."""
    import torch

    c = synthetic.make_capture("phasor_128", seed=8)
    dH = torch.from_numpy(c.H).to(cuda)
    Hc = torch.empty((c.P, c.T), dtype=torch.complex64, device=cuda)
    capi.phasor_pulse_device(dH, c.P, c.T, c.T, c.wavelength, c.deltaT, Hc, c.T)
    po = octree.PhasorOctree(c.pairs, c.T, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT,
                             cuda)
    N = tuple(int(v) for v in c.voxels_per_side)
    dense = torch.empty(N, dtype=torch.complex64, device=cuda)
    out = torch.empty_like(dense)
    po.dense(Hc, dense)
    po.reconstruct(Hc, out)
    torch.cuda.synchronize()
    e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    e[0].record()
    po.dense(Hc, dense)
    e[1].record()
    n_sel = po.reconstruct(Hc, out)
    e[2].record()
    e[2].synchronize()
    ms_dense, ms_oct = e[0].elapsed_time(e[1]), e[1].elapsed_time(e[2])
    mag = dense.abs()
    occ = mag >= 0.5 * mag.max()
    recall = ((out == dense) & occ).sum().item() / occ.sum().item()
    rel = (torch.linalg.vector_norm(out - dense) / torch.linalg.vector_norm(dense)).item()
    print(f"\n[phasor_128] dense {ms_dense:.2f} ms, block-sparse {ms_oct:.2f} ms "
          f"({ms_dense / ms_oct:.1f}x), tiles {n_sel}/{po.n_tiles}, recall {recall:.4f}, "
          f"rel-L2 {rel:.3e}")
    assert recall >= 0.99
    assert 0 < n_sel < 0.5 * po.n_tiles
    po.close()


def test_topk_tile_selection_vs_numpy(cuda):
    """bpgb_plan_select_tiles_topk lists exactly the tiles of the k highest-scoring
    blocks (8^3 tiles on 8^3 blocks: one block per tile), ties and +inf included."""
    import torch

    c = synthetic.make_capture("precision_64", seed=2, small=True, render=False, voxels=64)
    with capi.Plan(c.pairs, c.T, c.voxels_per_side, c.zero, c.inc, c.t0, c.deltaT,
                   algo=capi.ALGO_FAST, tile=10) as plan:
        nb = (8, 8, 8)
        rng = np.random.default_rng(4)
        score = rng.random(512).astype(np.float32)
        score[rng.choice(512, 20, replace=False)] = np.inf
        score[:5] = score[100]  # a tie
        score[300:310] = 0.0
        d_score = torch.from_numpy(score).to(cuda)
        lst = torch.empty(512, dtype=torch.int32, device=cuda)
        cnt = torch.zeros(1, dtype=torch.int32, device=cuda)
        for k in (0, 1, 7, 20, 37, 200, 511, 512, 900):
            plan.select_tiles_topk(d_score, nb, 8, k, lst, cnt)
            torch.cuda.synchronize()
            n = int(cnt.item())
            got = set(int(t) for t in lst[:n].cpu().numpy())
            if k == 0:
                assert n == 0
                continue
            kth = np.sort(score)[::-1][min(k, 512) - 1]
            # tile id t = (ty * tiles_x + tx) * tiles_z + tz; block id b = (bx * 8 + by) * 8 + bz
            want = set()
            for b in np.flatnonzero(score >= kth):
                bx, by, bz = b // 64, (b // 8) % 8, b % 8
                want.add(int((by * 8 + bx) * 8 + bz))
            assert got == want, (k, len(got), len(want))


def test_block_detail_vs_torch(cuda):
    import torch
    import torch.nn.functional as F

    g = torch.Generator().manual_seed(3)
    lo = torch.randn((4, 4, 4), generator=g)
    hi = torch.randn((8, 8, 8), generator=g)
    fine = (32, 32, 32)
    out = torch.empty((4, 4, 4), device=cuda)
    logits = torch.zeros(64)
    logits[5] = 3.0
    capi.block_detail(lo.to(cuda), (4, 4, 4), hi.to(cuda), (8, 8, 8), fine, 8, out, samples=4,
                      d_logits=logits.to(cuda), logit_lo=1.0)
    torch.cuda.synchronize()
    fl = F.interpolate(lo[None, None], size=fine, mode="trilinear", align_corners=True)[0, 0]
    fh = F.interpolate(hi[None, None], size=fine, mode="trilinear", align_corners=True)[0, 0]
    pts = torch.tensor([1, 3, 5, 7])  # 4 samples per axis in an 8-voxel block
    ref = torch.empty((4, 4, 4))
    for bx in range(4):
        for by in range(4):
            for bz in range(4):
                d = (fh - fl)[bx * 8 + pts][:, by * 8 + pts][:, :, bz * 8 + pts]
                ref[bx, by, bz] = (d * d).mean()
    got = out.cpu()
    assert torch.isinf(got.reshape(-1)[5])
    mask = torch.ones(64, dtype=torch.bool)
    mask[5] = False
    assert torch.allclose(got.reshape(-1)[mask], ref.reshape(-1)[mask], rtol=1e-4, atol=1e-6)


@pytest.mark.parametrize("fine_tile", [10, 13])
def test_budgeted_reconstruction_limits(cuda, fine_tile):
    """budget = 1 computes every block (equal to the dense pass bit for bit); a small
    budget computes at least the CNN's blocks and fills the rest from the 64^3-style
    second pass."""
    import torch

    geo = octree.OctreeGeometry.of("octree_256", small=True)
    rec = octree.Reconstructor(geo, cuda, fine_tile=fine_tile)
    model = octree.OccupancyCNN(cuda, seed=1)
    rec.render(*octree.scene(geo, 9))
    dense = rec.dense().clone()
    out = rec.reconstruct(model, 1e30, budget=1.0)
    rec.stream.synchronize()
    assert torch.equal(out.clone(), dense)
    assert rec.computed_mask().all()
    out = rec.reconstruct(model, -1e30, budget=0.01)  # every block is a CNN block
    rec.stream.synchronize()
    assert rec.computed_mask().all()
    out = rec.reconstruct(model, 1e30, budget=0.25)
    rec.stream.synchronize()  # the copy below runs on torch's stream, not the reconstructor's
    out = out.clone()
    comp = rec.computed_mask()
    nb = int(np.prod(rec.blocks))
    assert int(rec.tile_count.item()) >= round(0.25 * nb)
    assert torch.equal(out[comp], dense[comp])
    rec.close()


def test_trained_model_recall_vs_fp64_occupancy(cuda):
    """Occupancy taken from FP64 values, not from an FP32 pass: the negated Laplacian of
    the FP64 volume (bpgb_eval_f64_voxels, bit-identical to the FP64 oracle) on every voxel
    whose FP32 response reaches 0.1 max and their face neighbours; the FP64-occupied voxels
    (>= 0.2 of the FP64 maximum) are a subset of those candidates, since the FP32 and FP64
    responses differ far less than 0.1 max.  The committed CNN backprojects >= 99% of them
    at full resolution."""
    import torch

    model, state = octree.OccupancyCNN.load(cuda)
    geo = octree.OctreeGeometry.of("octree_256")
    rec = octree.Reconstructor(geo, cuda)
    lo = octree.logit(float(state["p_lo"]))
    n = geo.fine[0]
    P = len(geo.pairs)
    for seed in (3_000_004, 3_000_005):
        rec.render(*octree.scene(geo, seed))
        d32 = rec.dense_for_labels().clone()
        f32 = torch.empty_like(d32)
        capi.laplacian7(d32, geo.fine, f32)
        cand = f32 >= 0.1 * f32.max()
        near = cand.clone()
        for ax in range(3):
            near |= torch.roll(cand, 1, ax) | torch.roll(cand, -1, ax)
        ids = torch.nonzero(near.reshape(-1)).reshape(-1)
        d64 = torch.empty(len(ids), dtype=torch.float64, device=cuda)
        capi.eval_f64_voxels(rec.H, geo.T, rec.d_pairs, P, geo.fine, geo.zero, geo.inc_fine,
                             geo.t0, geo.deltaT, ids, d64)
        vol64 = torch.zeros(n ** 3, dtype=torch.float64, device=cuda)
        vol64[ids] = d64
        vol64 = vol64.reshape(geo.fine)
        lap = torch.zeros_like(vol64)
        for ax in range(3):
            for sh in (1, -1):
                nb = torch.roll(vol64, sh, ax)
                valid = torch.ones_like(vol64, dtype=torch.bool)
                idx = [slice(None)] * 3
                idx[ax] = 0 if sh == 1 else n - 1
                valid[tuple(idx)] = False
                lap += torch.where(valid, vol64 - nb, torch.zeros_like(vol64))
        lap = torch.where(cand, lap, torch.full_like(lap, -np.inf))
        occ64 = lap >= 0.2 * lap.max()
        assert (f32[occ64] >= 0.15 * f32.max()).all()  # well inside the candidates
        rec.reconstruct(model, lo)
        rec.stream.synchronize()
        comp = rec.computed_mask()
        recall = float((comp & occ64).sum()) / max(1, int(occ64.sum()))
        print(f"\n[octree_256 seed {seed}] recall of FP64-occupied voxels {recall:.5f} "
              f"({int(occ64.sum())} voxels, {len(ids)} evaluated in FP64)")
        assert recall >= 0.99
    rec.close()
