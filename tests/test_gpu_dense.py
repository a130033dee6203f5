"""The dense product XW = H W of the graph-convolution layer
(accspmm_dense_matmul, tcgen05 tensor cores), checked against FP64 products
within the TF32 (1e-3) and 3xTF32 (1e-6) relative Frobenius tolerances, over
shapes that exercise partial row tiles, k_in not a multiple of 32 or of 4
(H repacked), k_out past one 256-column tile, a misaligned H and n = 0."""
import numpy as np
import pytest

from accspmm_gb300 import api, capi
from tests.helpers import TOL_3XTF32_VS_F64, TOL_TF32_VS_F64, max_row_rel, rel_fro, torch_dev

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

SHAPES = [(1000, 48, 64), (4096, 128, 128), (300, 5, 8), (130, 33, 260), (20000, 256, 256),
          (128, 512, 16), (777, 64, 32), (1, 32, 4), (70001, 96, 48)]


def run(n, k_in, k_out, prec, seed, h_offset=0):
    rng = np.random.default_rng(seed)
    H = rng.standard_normal((n, k_in)).astype(np.float32)
    W = (rng.standard_normal((k_in, k_out)) / np.sqrt(k_in)).astype(np.float32)
    if h_offset:
        # H starting 4 bytes into a buffer: not 16-byte aligned
        buf = torch.empty(n * k_in + h_offset, dtype=torch.float32, device="cuda")
        Hd = buf[h_offset:].view(n, k_in)
        Hd.copy_(torch.from_numpy(H))
    else:
        Hd = torch_dev(H)
    XW = torch.full((max(n, 1), k_out), float("nan"), dtype=torch.float32, device="cuda")
    api.dense_matmul(Hd, n, k_in, torch_dev(W), k_out, XW, prec)
    torch.cuda.synchronize()
    capi.call("accspmm_device_status", None)
    return XW.cpu().numpy()[:n], H.astype(np.float64) @ W.astype(np.float64)


@pytest.mark.parametrize("n,k_in,k_out", SHAPES)
@pytest.mark.parametrize("prec,tol", [(capi.PREC_TF32, TOL_TF32_VS_F64), (capi.PREC_3XTF32, TOL_3XTF32_VS_F64)])
def test_dense_matmul_against_fp64(n, k_in, k_out, prec, tol):
    got, want = run(n, k_in, k_out, prec, seed=n + k_in + k_out)
    assert np.isfinite(got).all()
    assert rel_fro(got, want) < tol
    # every row, not only the norm: a wrong tile would show in its rows
    assert max_row_rel(got, want) < 20 * tol


def test_dense_matmul_misaligned_h():
    got, want = run(513, 36, 40, capi.PREC_TF32, seed=3, h_offset=1)
    assert rel_fro(got, want) < TOL_TF32_VS_F64


def test_dense_matmul_repeatable_and_empty():
    a, _ = run(2048, 64, 128, capi.PREC_TF32, seed=5)
    b, _ = run(2048, 64, 128, capi.PREC_TF32, seed=5)
    assert np.array_equal(a, b)
    got, want = run(0, 16, 16, capi.PREC_TF32, seed=1)
    assert got.shape == (0, 16)


def test_dense_matmul_argument_errors():
    H = torch.zeros((8, 8), device="cuda")
    W = torch.zeros((8, 8), device="cuda")
    XW = torch.zeros((8, 8), device="cuda")
    with pytest.raises(capi.AccSpmmError) as e:
        api.dense_matmul(H, 8, 8, W, 6, XW)  # k_out not a multiple of 4
    assert e.value.status == capi.ERROR_INVALID_VALUE
    with pytest.raises(capi.AccSpmmError):
        api.dense_matmul(H, 8, 8, W, 8, XW, precision=9)
    flat = torch.zeros(65, device="cuda")
    with pytest.raises(capi.AccSpmmError):
        api.dense_matmul(H, 8, 8, W, 4, flat[1:])  # XW not 16-byte aligned
