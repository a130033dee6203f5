"""SpMM values pinned to the reference's own GPU kernels (plain and adaptive).

tests/golden/ref_spmm/<case>_k<K>.npz hold what the reference's
tf32_mma_kernel (include/mma_tf32.cuh:13-228, built from the reference
sources into a cubin and run once on a GB300 by tests/golden/make_ref_spmm.py)
wrote for three golden matrices and B with identical rows v -- the inputs on
which that kernel computes A*B (see the generator for why).  The oracle's TF32
emulation and our kernels must reproduce those outputs within the TF32
emulation tolerance (they differ from the reference only in the FP32
accumulation order inside and across MMAs), and the reference's output must be
within the TF32 tolerance of the FP64 product."""
import numpy as np
import pytest

from oracle import oracle
from tests.helpers import GOLD, TOL_TF32_VS_EMU, TOL_TF32_VS_F64, empty_dev, gold, rel_fro

CASES = [(c, k) for c in ("rand203", "longwin", "plsym1000") for k in (64, 128)]


def metcf_of(case):
    """The reference's METCF arrays of a golden case."""
    g = gold(case)
    return dict(rows=int(g["dims"][0]), cols=int(g["dims"][1]), nnz=int(g["dims"][2]), rwo=g["m_rwo"],
                tc_offset=g["m_tc_offset"], bits=g["m_bits"], a2b=g["m_a2b"], data=g["m_data"])


def load(case, K):
    m = metcf_of(case)
    z = np.load(f"{GOLD}/ref_spmm/{case}_k{K}.npz")
    B = np.tile(z["v"], (m["cols"], 1)).astype(np.float32)
    return m, B, z["C"]


@pytest.mark.parametrize("case,K", CASES)
def test_oracle_reproduces_the_reference_kernel(case, K):
    m, B, ref = load(case, K)
    assert ref.shape == (8 * (len(m["rwo"]) - 1), K) and np.isfinite(ref).all()
    emu = oracle.spmm_metcf_tf32(m, m["cols"], B)
    assert rel_fro(emu, ref) < TOL_TF32_VS_EMU
    assert rel_fro(ref, oracle.spmm_metcf_f64(m, m["cols"], B)) < TOL_TF32_VS_F64


@pytest.mark.gpu
@pytest.mark.parametrize("case,K", CASES)
def test_our_kernels_reproduce_the_reference_kernel(case, K):
    torch = pytest.importorskip("torch")
    from accspmm_gb300 import api
    from tests.helpers import torch_dev
    m, B, ref = load(case, K)
    dm = api.DeviceMETCF.upload(m)
    C = empty_dev(dm.c_rows, K)
    dm.spmm(torch_dev(B), C, K)
    a = dm.adpbme()
    cr = a.c_rows()
    Ca = empty_dev(cr, K)
    a.spmm(torch_dev(B), Ca, cr, K)
    torch.cuda.synchronize()
    got = C.cpu().numpy()
    assert rel_fro(got, ref) < TOL_TF32_VS_EMU
    assert np.array_equal(Ca.cpu().numpy()[:dm.c_rows], got)


# The adaptive path: tests/golden/ref_spmm/<case>_adp_k<K>.npz hold what the
# reference's tf32_mma_balance_kernel (include/mma_tf32.cuh:552-792) wrote,
# launched once on a zeroed C of max(8G, rowIndices.back() + 8) rows with the
# reference's own AdpBME arrays, for B whose columns repeat with period 16
# (B = tile(B0, K / 16)) -- the inputs on which that kernel computes A*B.
ADP_CASES = [(c, k) for c in ("rand203", "longwin", "plsym1000", "ragged_unsorted") for k in (64, 128)]


def load_adp(case, K):
    m = metcf_of(case)
    z = np.load(f"{GOLD}/ref_spmm/{case}_adp_k{K}.npz")
    B = np.ascontiguousarray(np.tile(z["B0"], (1, K // 16))).astype(np.float32)
    return m, B, z["C"]


def same_rows(a, b):
    """The common rows of two C layouts, after checking that the rows only
    one of them has are zero."""
    n = min(len(a), len(b))
    assert not a[n:].any() and not b[n:].any()
    return a[:n], b[:n]


@pytest.mark.parametrize("case,K", ADP_CASES)
def test_oracle_reproduces_the_reference_adaptive_kernel(case, K):
    m, B, ref = load_adp(case, K)
    g = gold(case)
    go, ri = g["a_group_offset"], g["a_row_indices"]
    assert ref.shape == (max(8 * (len(go) - 1), int(ri[-1]) + 8), K) and np.isfinite(ref).all()
    emu, r = same_rows(oracle.spmm_metcf_tf32(m, m["cols"], B), ref)
    assert rel_fro(emu, r) < TOL_TF32_VS_EMU
    f64, r = same_rows(oracle.spmm_metcf_f64(m, m["cols"], B), ref)
    assert rel_fro(r, f64) < TOL_TF32_VS_F64


@pytest.mark.gpu
@pytest.mark.parametrize("case,K", ADP_CASES)
def test_our_adaptive_path_reproduces_the_reference_adaptive_kernel(case, K):
    torch = pytest.importorskip("torch")
    from accspmm_gb300 import api
    from tests.helpers import torch_dev
    m, B, ref = load_adp(case, K)
    dm = api.DeviceMETCF.upload(m)
    a = dm.adpbme()
    cr = a.c_rows()
    assert cr == ref.shape[0]  # the same C layout as the reference's driver
    Ca = empty_dev(cr, K)
    a.spmm(torch_dev(B), Ca, cr, K)
    torch.cuda.synchronize()
    got = Ca.cpu().numpy()
    assert not got[8 * len(m["rwo"][1:]):].any()
    assert rel_fro(got, ref) < TOL_TF32_VS_EMU
