"""The occupancy CNN's tensor-core (tcgen05) kernels against plain PyTorch FP32
references of the same ops, on line-planes tensors (bpgb_cnn_lp_*).

Tolerances as for the mma.sync kernels: BF16 outputs (forward, backward-data) within
1e-2 relative of the FP32 reference on BF16-exact inputs (one BF16 rounding of an FP32
sum); FP32 weight gradients within 1e-3.  Every test also checks that no bounded wait of
the kernels gave up (bpgb_cnn_tc_status)."""
from __future__ import annotations

import numpy as np
import pytest

from backprojector_gb300 import capi

pytestmark = pytest.mark.gpu

DIMS, BATCH = (3, 8, 32), 2
CASES = [(2, 16, True), (16, 16, True), (16, 1, False), (1, 16, False), (16, 8, True)]


def bf16_exact(t):
    return t.bfloat16().float()


def torch_weight(Wm, cin, cout):
    w = Wm[:27 * cin].reshape(3, 3, 3, cin, cout).permute(4, 3, 0, 1, 2).contiguous()
    return w, Wm[27 * cin].clone()


def random_master(cin, cout, seed, device):
    import torch

    g = torch.Generator().manual_seed(seed)
    W = torch.zeros((capi.cnn_kp(cin), cout))
    W[:27 * cin + 1] = torch.randn((27 * cin + 1, cout), generator=g) * 0.3
    return bf16_exact(W).to(device)


def lp_empty(ch, zpad, cuda, dims=DIMS, batch=BATCH):
    import torch

    n = capi.cnn_lp_bytes(ch, zpad, dims, batch)
    assert n > 0
    return torch.zeros(n // 2, dtype=torch.bfloat16, device=cuda)


def to_lp(X, zpad, cuda, dims=DIMS, batch=BATCH):
    """X: [batch, n0, n1, 32, C] (BF16-exact floats) -> line-planes tensor."""
    C = X.shape[-1]
    buf = lp_empty(C, zpad, cuda, dims, batch)
    src = X.reshape(-1, C).to(cuda).bfloat16().contiguous()
    capi.cnn_lp_pack(src, C, C, dims, batch, zpad, buf)
    return buf


def from_lp(buf, C, zpad, cuda, dims=DIMS, batch=BATCH):
    import torch

    V = batch * int(np.prod(dims))
    out = torch.empty((V, C), dtype=torch.bfloat16, device=cuda)
    capi.cnn_lp_unpack(buf, C, zpad, dims, batch, out)
    torch.cuda.synchronize()
    return out.float().cpu()


@pytest.mark.parametrize("C,zpad", [(2, 0), (16, 0), (1, 1), (16, 1)])
def test_lp_roundtrip_and_zero_padding(cuda, C, zpad):
    import torch

    g = torch.Generator().manual_seed(C + 10 * zpad)
    X = bf16_exact(torch.randn((BATCH, *DIMS, C), generator=g))
    buf = to_lp(X, zpad, cuda)
    back = from_lp(buf, C, zpad, cuda)
    assert torch.equal(back, X.reshape(-1, C))
    # exactly the voxels' channels are non-zero: the padding rows and unused channels stay 0
    nz = int((buf != 0).sum())
    assert nz == int((X != 0).sum())


def test_umma_status_clean_before(cuda):
    capi.cnn_tc_status(reset=True)


@pytest.mark.parametrize("in_zpad", [0, 1])
@pytest.mark.parametrize("cin,cout,relu", CASES)
def test_tc_conv3d_forward_vs_torch(cuda, cin, cout, relu, in_zpad):
    import torch
    import torch.nn.functional as F

    g = torch.Generator().manual_seed(cin * 100 + cout + in_zpad)
    X = bf16_exact(torch.randn((BATCH, *DIMS, cin), generator=g))
    W = random_master(cin, cout, 7, cuda)
    Wf = torch.zeros(capi.cnn_tc_weight_bytes(cin) // 2, dtype=torch.bfloat16, device=cuda)
    capi.cnn_tc_pack_weights(W, cin, cout, Wf)
    bias = W[27 * cin].contiguous()
    xl = to_lp(X, in_zpad, cuda)
    V = BATCH * int(np.prod(DIMS))
    for out_zpad in (0, 1):
        Y = lp_empty(cout, out_zpad, cuda)
        Yf = torch.full((V,), float("nan"), device=cuda)
        capi.cnn_tc_conv3d(xl, cin, in_zpad, DIMS, BATCH, Wf, bias, cout, relu, d_Y=Y,
                           out_zpad=out_zpad, d_Yf=Yf)
        assert capi.cnn_tc_status() == 0
        w, b = torch_weight(W.cpu(), cin, cout)
        ref = F.conv3d(X.permute(0, 4, 1, 2, 3), w, b, padding=1)
        ref = ref.permute(0, 2, 3, 4, 1).reshape(V, cout)
        got = from_lp(Y, cout, out_zpad, cuda)
        refr = ref.clamp_min(0) if relu else ref
        tol = 1e-2 * float(refr.abs().max())
        assert torch.allclose(got, refr, rtol=1e-2, atol=tol), float((got - refr).abs().max())
        # the FP32 channel-0 output is the unrounded sum (before ReLU)
        assert torch.allclose(Yf.cpu(), ref[:, 0], rtol=1e-5, atol=1e-4 * float(ref.abs().max()))
        # nothing outside the interior rows was written
        assert int((Y != 0).sum()) == int((got != 0).sum())


@pytest.mark.parametrize("cin,cout,relu", CASES)
def test_tc_weight_gradient_vs_torch(cuda, cin, cout, relu):
    import torch
    import torch.nn.functional as F

    g = torch.Generator().manual_seed(5 + cin + cout)
    X = bf16_exact(torch.randn((BATCH, *DIMS, cin), generator=g))
    dY = bf16_exact(torch.randn((BATCH, *DIMS, cout), generator=g))
    W = random_master(cin, cout, 11, cuda)
    xl, dyl = to_lp(X, 0, cuda), to_lp(dY, 1, cuda)
    nscr = capi.cnn_tc_wgrad_scratch_bytes(cin, DIMS, BATCH)
    scr = torch.empty(nscr // 4, device=cuda)
    dW = torch.full(tuple(W.shape), float("nan"), device=cuda)
    capi.cnn_tc_conv3d_wgrad(xl, cin, dyl, cout, DIMS, BATCH, scr, nscr, dW)
    assert capi.cnn_tc_status() == 0
    w, b = torch_weight(W.cpu(), cin, cout)
    xt = X.permute(0, 4, 1, 2, 3).clone().requires_grad_(True)
    wt = w.clone().requires_grad_(True)
    bt = b.clone().requires_grad_(True)
    F.conv3d(xt, wt, bt, padding=1).backward(dY.permute(0, 4, 1, 2, 3))
    ref_w = wt.grad.permute(2, 3, 4, 1, 0).reshape(27 * cin, cout)
    got = dW.cpu()
    assert torch.allclose(got[:27 * cin], ref_w, rtol=1e-3, atol=1e-4 * float(ref_w.abs().max()))
    assert torch.allclose(got[27 * cin], bt.grad, rtol=1e-3,
                          atol=1e-4 * float(bt.grad.abs().max()))
    assert torch.all(got[27 * cin + 1:] == 0)


@pytest.mark.parametrize("cin,cout,relu", CASES)
def test_tc_backward_data_vs_torch(cuda, cin, cout, relu):
    import torch
    import torch.nn.functional as F

    g = torch.Generator().manual_seed(17 + cin + cout)
    X = bf16_exact(torch.randn((BATCH, *DIMS, cin), generator=g))
    dY = bf16_exact(torch.randn((BATCH, *DIMS, cout), generator=g))
    mask = bf16_exact(torch.randn((BATCH, *DIMS, cin), generator=g))
    W = random_master(cin, cout, 13, cuda)
    Wf = torch.zeros(capi.cnn_tc_weight_bytes(cin) // 2, dtype=torch.bfloat16, device=cuda)
    Wb = torch.zeros(capi.cnn_tc_weight_bytes(cout) // 2, dtype=torch.bfloat16, device=cuda)
    capi.cnn_tc_pack_weights(W, cin, cout, Wf, Wb)
    dyl, ml = to_lp(dY, 1, cuda), to_lp(mask, 0, cuda)
    gX = lp_empty(cin, 1, cuda)
    capi.cnn_tc_conv3d(dyl, cout, 1, DIMS, BATCH, Wb, None, cin, False, d_mask=ml, d_Y=gX,
                       out_zpad=1)
    assert capi.cnn_tc_status() == 0
    w, b = torch_weight(W.cpu(), cin, cout)
    xt = X.permute(0, 4, 1, 2, 3).clone().requires_grad_(True)
    F.conv3d(xt, w, b, padding=1).backward(dY.permute(0, 4, 1, 2, 3))
    V = BATCH * int(np.prod(DIMS))
    ref = xt.grad.permute(0, 2, 3, 4, 1).reshape(V, cin) * (mask.reshape(V, cin) > 0)
    got = from_lp(gX, cin, 1, cuda)
    assert torch.allclose(got, ref, rtol=1e-2, atol=1e-2 * float(ref.abs().max()))


def test_tc_bce_matches_channels_last(cuda):
    import torch

    V = BATCH * int(np.prod(DIMS))
    g = torch.Generator().manual_seed(3)
    z = (torch.randn(V, generator=g) * 3).to(cuda)
    y = (torch.rand(V, generator=g) < 0.2).to(torch.uint8).to(cuda)
    dZ = torch.zeros((V, 8), dtype=torch.bfloat16, device=cuda)
    loss = torch.zeros(V, device=cuda)
    capi.cnn_bce_grad(z, y, V, 4.0, 1.0 / V, dZ, loss)
    dzl = lp_empty(1, 1, cuda)
    loss2 = torch.zeros(V, device=cuda)
    capi.cnn_tc_bce_grad(z, y, DIMS, BATCH, 4.0, 1.0 / V, dzl, loss2)
    got = from_lp(dzl, 1, 1, cuda)
    assert torch.equal(got[:, 0], dZ[:, 0].float().cpu())
    assert torch.equal(loss2.cpu(), loss.cpu())


def test_tc_train_step_matches_mma_step(cuda):
    """One training step of the 4-layer CNN on the tensor-core kernels against the same
    step on the mma.sync kernels, from the same weights and inputs (batch 4 of 32^3):
    per-voxel losses and every layer's weight gradient agree to BF16 rounding of the
    activations (summation orders differ)."""
    import torch

    from backprojector_gb300 import octree

    dims, batch = (32, 32, 32), 4
    g = torch.Generator().manual_seed(0)
    coarse = torch.rand((batch, 32 ** 3), generator=g).to(cuda)
    y = (torch.rand(batch * 32 ** 3, generator=g) < 0.1).to(torch.uint8).to(cuda)
    ma, mb = octree.OccupancyCNN(cuda, seed=0), octree.OccupancyCNN(cuda, seed=0)
    X = ma.features(coarse, dims, batch)
    la = ma.train_step(X, y, dims, batch, 1e-3, 10.0, tc=True)
    lb = mb.train_step(X, y, dims, batch, 1e-3, 10.0, tc=False)
    torch.cuda.synchronize()
    assert capi.cnn_tc_status() == 0
    la, lb = la.double().cpu(), lb.double().cpu()
    assert float((la - lb).norm() / lb.norm()) < 1e-2
    for li in range(4):
        ga, gb = ma.G[li].double().cpu(), mb.G[li].double().cpu()
        rel = float((ga - gb).norm() / gb.norm())
        print(f"\nlayer {li}: weight-gradient rel-L2 tc vs mma.sync {rel:.2e}")
        assert rel < 2e-2, (li, rel)


def test_tc_pack_layers_matches_per_layer_packing(cuda):
    import torch

    specs = [(2, 16), (16, 16), (16, 16), (16, 1)]
    Ws = [random_master(ci, co, 30 + i, cuda) for i, (ci, co) in enumerate(specs)]
    one_f = [torch.zeros(capi.cnn_tc_weight_bytes(ci) // 2, dtype=torch.bfloat16, device=cuda)
             for ci, _ in specs]
    one_b = [torch.zeros(capi.cnn_tc_weight_bytes(co) // 2, dtype=torch.bfloat16, device=cuda)
             for _, co in specs]
    for (ci, co), W, f, b in zip(specs, Ws, one_f, one_b):
        capi.cnn_tc_pack_weights(W, ci, co, f, b)
    all_f = [torch.full_like(f, float("nan")) for f in one_f]
    all_b = [None] + [torch.full_like(b, float("nan")) for b in one_b[1:]]
    capi.cnn_tc_pack_layers(Ws, [s[0] for s in specs], [s[1] for s in specs], all_f, all_b)
    torch.cuda.synchronize()
    for i in range(4):
        assert torch.equal(all_f[i], one_f[i])
        if all_b[i] is not None:
            assert torch.equal(all_b[i], one_b[i])
