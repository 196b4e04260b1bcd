"""Known-answer tests of the tensor-core (tcgen05.mma kind::f16) descriptor and
accumulator layouts that the CNN kernels are built on (bpgb_diag_umma_probe).

Operands are small integers, exact in BF16, so every product and sum is exact in FP32
and the accumulator must equal numpy's product bit for bit.  Each case lays A and B out
in the no-swizzle canonical form (core matrices of 8 rows x 16 B), K-major or MN-major,
and checks which assignment of the two descriptor strides (the K-direction and the
M/N-direction core-matrix offsets) the tensor core follows, and where the rows of D land
in tensor memory for M = 128 and M = 64."""
from __future__ import annotations

import numpy as np
import pytest

from backprojector_gb300 import capi

pytestmark = pytest.mark.gpu

IMG_BYTES = 48 * 1024


def idesc(M, N, a_mn=False, b_mn=False):
    return ((1 << 4) | (1 << 7) | (1 << 10) | (int(a_mn) << 15) | (int(b_mn) << 16)
            | ((N >> 3) << 17) | ((M >> 4) << 24))


def bf16(x):
    return (np.asarray(x, np.float32).view(np.uint32) >> 16).astype(np.uint16)


def place(img, off, X, s_rows, s_k, mn_major):
    """X[r][k] (r = M or N index) at core matrix (r // 8, k // 8): offset r//8 * s_rows +
    k//8 * s_k; inside it row (k % 8 if MN-major else r % 8) of 16 bytes."""
    R, K = X.shape
    b = bf16(X)
    for r in range(R):
        for k in range(K):
            if mn_major:
                a = off + (r // 8) * s_rows + (k // 8) * s_k + (k % 8) * 16 + (r % 8) * 2
            else:
                a = off + (r // 8) * s_rows + (k // 8) * s_k + (r % 8) * 16 + (k % 8) * 2
            assert a % 2 == 0 and a + 2 <= IMG_BYTES
            img[a // 2] = b[r, k]


def operands(M, N, K, seed):
    rng = np.random.default_rng(seed)
    A = rng.integers(-4, 5, (M, K)).astype(np.float32)
    B = rng.integers(-4, 5, (N, K)).astype(np.float32)
    return A, B, A @ B.T


def run(M, N, K, a_mn, b_mn, a_lay, b_lay, swap_a, swap_b, seed=0):
    """a_lay / b_lay = (offset, stride between row groups, stride between K groups)."""
    A, B, D = operands(M, N, K, seed)
    img = np.zeros(IMG_BYTES // 2, np.uint16)
    place(img, a_lay[0], A, a_lay[1], a_lay[2], a_mn)
    place(img, b_lay[0], B, b_lay[1], b_lay[2], b_mn)
    nk = K // 16

    def fields(lay, swap):
        rows, k = lay[1], lay[2]
        return (rows, k) if swap else (k, rows)  # (lbo, sbo)

    al, as_ = fields(a_lay, swap_a)
    bl, bs = fields(b_lay, swap_b)
    prm = (a_lay[0], al, as_, 2 * a_lay[2], b_lay[0], bl, bs, 2 * b_lay[2],
           idesc(M, N, a_mn, b_mn), nk)
    out, st = capi.umma_probe(img, prm, max(16, (N + 15) // 16 * 16))
    assert st == 0, st
    return out[:, :N], D


def lanes_of(out, D):
    """Lane holding each row of D (-1 when absent)."""
    lanes = []
    for m in range(D.shape[0]):
        hit = np.nonzero(np.all(out == D[m], axis=1))[0]
        lanes.append(int(hit[0]) if len(hit) == 1 else -1)
    return lanes


CASES = {
    # name: M, N, K, a_mn, b_mn, A (offset, row-group stride, K-group stride), B (...)
    "kmajor_m128_n16": (128, 16, 16, False, False, (0, 128, 2048), (32768, 128, 256)),
    "kmajor_m128_n16_k32": (128, 16, 32, False, False, (0, 128, 2048), (32768, 128, 256)),
    "kmajor_m64_n32": (64, 32, 16, False, False, (0, 128, 1024), (32768, 128, 512)),
    "mnmajor_a_m64_n16": (64, 16, 32, True, True, (0, 512, 128), (32768, 512, 128)),
    "mnmajor_a_m128_n16": (128, 16, 16, True, False, (0, 256, 128), (32768, 128, 256)),
}


@pytest.mark.parametrize("name", list(CASES))
def test_umma_layouts(cuda, name):
    M, N, K, a_mn, b_mn, a_lay, b_lay = CASES[name]
    found = []
    for swap_a in (False, True):
        for swap_b in (False, True):
            out, D = run(M, N, K, a_mn, b_mn, a_lay, b_lay, swap_a, swap_b)
            lanes = lanes_of(out, D)
            ok = all(l >= 0 for l in lanes)
            print(f"\n[{name}] swap_a={swap_a} swap_b={swap_b}: rows found "
                  f"{sum(l >= 0 for l in lanes)}/{M}; lanes {lanes[:4]}..{lanes[-4:]}")
            if ok:
                found.append((swap_a, swap_b, lanes))
    assert found, f"{name}: no stride assignment reproduces A @ B^T"
    for swap_a, swap_b, lanes in found:
        print(f"[{name}] MATCH swap_a={swap_a} swap_b={swap_b} lanes={lanes}")


def test_umma_issue_rates(cuda):
    """The MMA issue floor: a small MMA costs a fixed number of cycles, a full-width one
    (M128 N256) runs at the dense BF16 rate (M N K / 4096 MACs per clock = 128 cycles)."""
    r = capi.umma_issue_rates()
    print("\ncycles per tcgen05.mma:", {k: round(v, 1) for k, v in r.items()})
    assert all(v > 0 for v in r.values())
    assert r["m128_n256_k"] >= r["m128_n48_k"]
