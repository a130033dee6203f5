"""Fused SpMM epilogue (bias + ReLU applied as C is stored) and the GCN layer
out = act(A (H W) + bias).  The fused epilogue must give the same bits as the
plain SpMM followed by a separate FP32 bias add and ReLU; the layer is checked
against an FP64 evaluation within the TF32 / 3xTF32 tolerances."""
import numpy as np
import pytest

from accspmm_gb300 import api, capi
from oracle import oracle
from tests.helpers import TOL_3XTF32_VS_F64, TOL_TF32_VS_F64, empty_dev, gold, rel_fro, torch_dev

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def device_matrix(name):
    g = gold(name)
    csr = dict(rows=int(g["dims"][0]), cols=int(g["dims"][1]), nnz=int(g["dims"][2]),
               row_ptr=g["csr_row_ptr"], col_idx=g["csr_col_idx"], data=g["csr_data"])
    m = api.DeviceMETCF.from_csr(api.DeviceCSR.upload(csr))
    torch.cuda.synchronize()
    return m, csr


@pytest.mark.parametrize("name", ["plsym1000", "longwin"])
@pytest.mark.parametrize("K", [32, 100, 128])
@pytest.mark.parametrize("act", [capi.ACT_NONE, capi.ACT_RELU])
def test_fused_epilogue_equals_separate_bias_and_relu(name, K, act):
    m, csr = device_matrix(name)
    rng = np.random.default_rng(K + act)
    B = torch_dev(rng.uniform(-1, 1, (csr["cols"], K)).astype(np.float32))
    bias = torch_dev(rng.uniform(-1, 1, K).astype(np.float32))
    plain = empty_dev(m.c_rows, K)
    m.spmm(B, plain, K)
    want = plain + bias
    if act == capi.ACT_RELU:
        want = torch.clamp_min(want, 0.0)
    got = empty_dev(m.c_rows, K)
    m.spmm_bias_act(B, got, K, bias, act)
    torch.cuda.synchronize()
    assert torch.equal(got, want)
    # no bias, ReLU only
    got2 = empty_dev(m.c_rows, K)
    m.spmm_bias_act(B, got2, K, None, capi.ACT_RELU)
    torch.cuda.synchronize()
    assert torch.equal(got2, torch.clamp_min(plain, 0.0))


@pytest.mark.parametrize("K", [64, 128, 200])
def test_fused_epilogue_over_packed_b_equals_separate_bias_and_relu(K):
    """A B of 4 MiB or more is packed for the fused epilogue too (128-column
    slices for K > 64, 64-column ones for K = 64): still bit for bit the plain
    SpMM followed by a separate FP32 bias add and ReLU."""
    from accspmm_gb300 import synth
    n = 20000
    rp, ci, vals = synth.powerlaw_local(n=n, seed=11)
    csr = dict(rows=n, cols=n, nnz=len(ci), row_ptr=rp, col_idx=ci, data=vals)
    m = api.DeviceMETCF.from_csr(api.DeviceCSR.upload(csr))
    rng = np.random.default_rng(K)
    B = torch_dev(rng.uniform(-1, 1, (n, K)).astype(np.float32))
    assert B.numel() * 4 >= 4 << 20
    bias = torch_dev(rng.uniform(-1, 1, K).astype(np.float32))
    plain = empty_dev(m.c_rows, K)
    m.spmm(B, plain, K)
    got = empty_dev(m.c_rows, K)
    m.spmm_bias_act(B, got, K, bias, capi.ACT_RELU)
    torch.cuda.synchronize()
    assert torch.equal(got, torch.clamp_min(plain + bias, 0.0))


@pytest.mark.parametrize("prec,tol", [(capi.PREC_TF32, TOL_TF32_VS_F64),
                                      (capi.PREC_3XTF32, TOL_3XTF32_VS_F64)])
def test_gcn_layer_against_fp64(prec, tol):
    m, csr = device_matrix("plsym1000")
    h = m.to_numpy()
    rng = np.random.default_rng(7)
    k_in, k_out = 48, 64
    H = rng.standard_normal((csr["cols"], k_in)).astype(np.float32)
    W = (rng.standard_normal((k_in, k_out)) / np.sqrt(k_in)).astype(np.float32)
    b = rng.uniform(-0.5, 0.5, k_out).astype(np.float32)
    out = empty_dev(m.c_rows, k_out)
    m.gcn_layer(torch_dev(H), k_in, torch_dev(W), k_out, out, torch_dev(b), capi.ACT_RELU, prec)
    torch.cuda.synchronize()
    xw = H.astype(np.float64) @ W.astype(np.float64)
    ref = np.maximum(oracle.spmm_metcf_f64(h, csr["cols"], xw) + b, 0.0)
    got = out.cpu().numpy()[:csr["rows"]]
    assert rel_fro(got, ref[:csr["rows"]]) < tol


def test_epilogue_argument_errors():
    m, csr = device_matrix("kat10")
    B = empty_dev(csr["cols"], 8, 0.0)
    C = empty_dev(m.c_rows, 8)
    bias = torch.zeros(9, device="cuda")
    with pytest.raises(capi.AccSpmmError) as e:
        m.spmm_bias_act(B, C, 8, bias[1:], capi.ACT_NONE)  # 4-byte aligned only
    assert e.value.status == capi.ERROR_INVALID_VALUE
    with pytest.raises(capi.AccSpmmError):
        m.spmm_bias_act(B, C, 8, None, 7)


@pytest.mark.parametrize("hops", [1, 2, 3, 4])
def test_chain_equals_repeated_spmm(hops):
    m, csr = device_matrix("plsym1000")
    K = 64
    B = torch_dev(np.random.default_rng(hops).uniform(-1, 1, (csr["cols"], K)).astype(np.float32))
    want = B
    for _ in range(hops):
        nxt = empty_dev(m.c_rows, K)
        m.spmm(want, nxt, K)
        want = nxt
    got = empty_dev(m.c_rows, K)
    m.spmm_chain(B, got, K, hops)
    torch.cuda.synchronize()
    assert torch.equal(got, want)


def test_chain_needs_a_square_matrix():
    m, csr = device_matrix("longwin")  # 64 x 600
    B = empty_dev(csr["cols"], 8, 0.0)
    with pytest.raises(capi.AccSpmmError):
        m.spmm_chain(B, empty_dev(m.c_rows, 8), 8, 2)
