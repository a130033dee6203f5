"""Reverse Cuthill-McKee reordering and the symmetric permutation P A P^T.

On a 2D grid graph whose vertex numbers were shuffled, RCM must recover a
banded numbering (bandwidth near the grid width) and METCF of the reordered
matrix needs fewer tiles; P A P^T must equal A[perm][:, perm]; and the
reordered product, mapped back, must equal the original product (GPU)."""
import numpy as np
import pytest
import scipy.sparse as sp

from accspmm_gb300 import api, capi
from tests.helpers import TOL_TF32_VS_F64, empty_dev, rel_fro, torch_dev


def shuffled_grid(side=120, seed=0):
    n = side * side
    idx = np.arange(n).reshape(side, side)
    r = np.concatenate([idx[:, :-1].ravel(), idx[:-1, :].ravel()])
    c = np.concatenate([idx[:, 1:].ravel(), idx[1:, :].ravel()])
    rows = np.concatenate([r, c, np.arange(n)])
    cols = np.concatenate([c, r, np.arange(n)])
    vals = np.random.default_rng(seed).uniform(0.1, 1.0, rows.size).astype(np.float32)
    lab = np.random.default_rng(seed + 1).permutation(n)
    A = sp.csr_matrix((vals, (lab[rows], lab[cols])), shape=(n, n))
    A.sort_indices()
    return dict(rows=n, cols=n, nnz=A.nnz, row_ptr=A.indptr.astype(np.uint32),
                col_idx=A.indices.astype(np.uint32), data=A.data.astype(np.float32)), A


def test_rcm_recovers_a_banded_numbering():
    csr, A = shuffled_grid()
    perm, bw0, bw1 = api.reorder_rcm(csr)
    n = csr["rows"]
    assert sorted(perm.tolist()) == list(range(n))
    assert bw0 > n // 2
    assert bw1 <= 2 * 120 + 2
    again, _, _ = api.reorder_rcm(csr)
    assert np.array_equal(perm, again)  # deterministic


def test_csr_permute_is_p_a_pt():
    csr, A = shuffled_grid(side=40, seed=3)
    perm, _, _ = api.reorder_rcm(csr)
    out = api.csr_permute(csr, perm)
    want = A[perm][:, perm].tocsr()
    want.sort_indices()
    np.testing.assert_array_equal(out["row_ptr"], want.indptr)
    np.testing.assert_array_equal(out["col_idx"], want.indices)
    np.testing.assert_array_equal(out["data"], want.data)


def test_reordering_cuts_metcf_tiles():
    # a 5-point grid stencil: 8 shuffled rows touch ~40 distinct columns (5
    # tiles), 8 consecutive rows of the RCM order share neighbours (~4 tiles)
    csr, _ = shuffled_grid()
    perm, _, _ = api.reorder_rcm(csr)
    t0 = len(api.metcf_from_csr(csr)["bits"])
    t1 = len(api.metcf_from_csr(api.csr_permute(csr, perm))["bits"])
    assert t1 < 0.85 * t0


def test_bad_inputs_are_refused():
    csr, _ = shuffled_grid(side=10)
    rect = dict(csr, cols=csr["cols"] + 1)
    with pytest.raises(capi.AccSpmmError):
        api.reorder_rcm(rect)
    bad = np.zeros(csr["rows"], np.uint32)  # not a permutation
    with pytest.raises(capi.AccSpmmError):
        api.csr_permute(csr, bad)


@pytest.mark.parametrize("case", ["row_ptr_decreases", "last_offset_not_nnz", "first_offset_not_zero",
                                  "column_past_cols"])
def test_malformed_host_csr_is_refused_before_it_is_read(case):
    """The host entry points that walk a CSR (RCM, P A P^T, the host METCF
    builder) check its offsets and columns first and return
    ACCSPMM_ERROR_INVALID_VALUE instead of reading past its arrays."""
    csr, _ = shuffled_grid(side=10)
    rp, ci = csr["row_ptr"].copy(), csr["col_idx"].copy()
    if case == "row_ptr_decreases":
        rp[5] = rp[7] + 1
    elif case == "last_offset_not_nnz":
        rp[-1] = csr["nnz"] + 8
    elif case == "first_offset_not_zero":
        rp[0] = 2
    else:
        ci[3] = csr["cols"] + 4
    bad = dict(csr, row_ptr=rp, col_idx=ci)
    perm = np.arange(csr["rows"], dtype=np.uint32)
    for call in (lambda: api.reorder_rcm(bad), lambda: api.csr_permute(bad, perm),
                 lambda: api.metcf_from_csr(bad)):
        with pytest.raises(capi.AccSpmmError) as e:
            call()
        assert e.value.status == capi.ERROR_INVALID_VALUE


@pytest.mark.gpu
def test_reordered_product_maps_back_to_the_original():
    torch = pytest.importorskip("torch")
    csr, A = shuffled_grid()
    n, K = csr["rows"], 64
    perm, _, _ = api.reorder_rcm(csr)
    m = api.DeviceMETCF.from_csr(api.DeviceCSR.upload(api.csr_permute(csr, perm)))
    B = np.random.default_rng(5).uniform(-1, 1, (n, K)).astype(np.float32)
    dB, dP = torch_dev(B), torch_dev(perm.view(np.int32))
    PB = torch.empty_like(dB)
    api.permute_rows(dB, PB, dP, n, K)  # PB[i] = B[perm[i]]
    Cp = empty_dev(m.c_rows, K)
    m.spmm(PB, Cp, K)
    Cout = torch.full((n, K), float("nan"), device="cuda")
    api.permute_rows(Cp, Cout, dP, n, K, scatter=True)  # C[perm[i]] = C'[i]
    torch.cuda.synchronize()
    ref = A.astype(np.float64) @ B.astype(np.float64)
    assert rel_fro(Cout.cpu().numpy(), ref) < TOL_TF32_VS_F64


@pytest.mark.gpu
@pytest.mark.parametrize("n,K", [(1003, 12), (517, 260), (4, 128), (1, 4)])
def test_row_permutation_is_exact(n, K):
    """Gather and scatter move rows bit for bit, for row counts that are not
    a multiple of the rows a warp moves and rows shorter and longer than one
    warp's float4s."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(n + K)
    perm = rng.permutation(n).astype(np.uint32)
    B = rng.standard_normal((n, K)).astype(np.float32)
    dB, dP = torch_dev(B), torch_dev(perm.view(np.int32))
    G = torch.full((n, K), float("nan"), device="cuda")
    S = torch.full((n, K), float("nan"), device="cuda")
    api.permute_rows(dB, G, dP, n, K)
    api.permute_rows(dB, S, dP, n, K, scatter=True)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(G.cpu().numpy(), B[perm])
    want = np.empty_like(B)
    want[perm] = B
    np.testing.assert_array_equal(S.cpu().numpy(), want)
