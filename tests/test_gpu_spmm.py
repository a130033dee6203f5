"""GPU parity: device builders bit-exact with the reference layout, SpMM within
the stated tolerances of the oracle, all through the C ABI."""
import ctypes
import glob
import os

import numpy as np
import pytest

from accspmm_gb300 import api, capi, synth
from oracle import oracle
from tests.helpers import (GOLD, TOL_3XTF32_VS_F64, TOL_TF32_VS_EMU, TOL_TF32_VS_F64, empty_dev,
                           gold, max_row_rel, rel_fro, torch_dev)

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

OK_CASES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLD, "*.npz"))
                  if int(np.load(p)["status"][0]) == 0)


def csr_of_gold(g):
    return dict(rows=int(g["dims"][0]), cols=int(g["dims"][1]), nnz=int(g["dims"][2]),
                row_ptr=g["csr_row_ptr"], col_idx=g["csr_col_idx"], data=g["csr_data"])


def device_metcf(csr):
    d = api.DeviceCSR.upload(csr)
    m = api.DeviceMETCF.from_csr(d)
    torch.cuda.synchronize()
    return m


@pytest.mark.parametrize("name", OK_CASES)
def test_device_builders_match_reference(name):
    g = gold(name)
    m = device_metcf(csr_of_gold(g))
    h = m.to_numpy()
    for k, gk in [("rwo", "m_rwo"), ("tc_offset", "m_tc_offset"), ("bits", "m_bits"),
                  ("a2b", "m_a2b"), ("data", "m_data")]:
        np.testing.assert_array_equal(h[k], g[gk], err_msg=k)
    assert m.balance_strategy() == int(g["balance"][0])
    if "a_group_offset" in g:
        a = m.adpbme().to_numpy()
        for k, gk in [("group_offset", "a_group_offset"), ("tc_offset", "a_tc_offset"),
                      ("row_indices", "a_row_indices"), ("bits", "a_bits"), ("a2b", "a_a2b"),
                      ("data", "a_data")]:
            np.testing.assert_array_equal(a[k], g[gk], err_msg=k)
        b = m.adpbme(2, 3, 5, 4).to_numpy()
        np.testing.assert_array_equal(b["group_offset"], g["b_group_offset"])


@pytest.mark.parametrize("params", [(3, 1, 2, 16), (2, 3, 5, 4), (1, 0, 0, 1), (10, 5, 7, 60),
                                    (7, 7, 7, 100)])
def test_device_adpbme_groups_match_the_oracle(params):
    """The GPU group packing (chunk tables composed level by level, then
    replayed per chunk) equals the oracle's sequential greedy walk on a
    131,072-row matrix (about 2,000 chunks): the reference's parameters, a
    one-tile target, a state space of 909 states (several shared-memory
    pieces per walk) and one past the tabulated limit (the sequential
    kernel)."""
    n = 1 << 17
    rp, ci, vals = synth.powerlaw_local(n=n, seed=3)
    m = device_metcf(dict(rows=n, cols=n, nnz=len(ci), row_ptr=rp, col_idx=ci, data=vals))
    rwo = m.to_numpy()["rwo"]
    got = m.adpbme(*params).to_numpy()["group_offset"]
    np.testing.assert_array_equal(got, oracle.adpbme_groups(rwo, *params))


def test_device_csr_from_coo_matches_host():
    g = gold("ragged_unsorted")
    rows, cols = int(g["dims"][0]), int(g["dims"][1])
    import ctypes as C
    coo = api.coo_struct(rows, cols, g["coo_row"], g["coo_col"], g["coo_data"])
    dcoo = capi.COO()
    capi.call("accspmm_coo_copy", C.byref(coo.struct), capi.DEVICE, C.byref(dcoo), None)
    dcsr = capi.CSR()
    capi.call("accspmm_csr_from_coo", C.byref(dcoo), C.byref(dcsr), None)
    hcsr = capi.CSR()
    capi.call("accspmm_csr_copy", C.byref(dcsr), capi.HOST, C.byref(hcsr), None)
    got = api.csr_to_numpy(hcsr)
    np.testing.assert_array_equal(got["row_ptr"], g["csr_row_ptr"])
    np.testing.assert_array_equal(got["col_idx"], g["csr_col_idx"])
    np.testing.assert_array_equal(got["data"], g["csr_data"])
    lib = capi.load()
    for s, f in ((dcoo, lib.accspmm_coo_destroy), (dcsr, lib.accspmm_csr_destroy),
                 (hcsr, lib.accspmm_csr_destroy)):
        f(C.byref(s))


@pytest.mark.parametrize("seed", [0, 3])
def test_device_metcf_config1_and_unsorted(seed):
    r, c, v = synth.powerlaw_symmetric(n=16384, seed=seed)
    r, c, v = synth.expand_symmetric(r, c, v)
    csr = api.csr_from_coo(16384, 16384, r, c, v)
    o = oracle.metcf(16384, csr["row_ptr"], csr["col_idx"], csr["data"])
    h = device_metcf(csr).to_numpy()
    for k in ("rwo", "tc_offset", "bits", "a2b", "data"):
        np.testing.assert_array_equal(h[k], o[k], err_msg=k)
    # unsorted rows with duplicates
    rng = np.random.default_rng(seed)
    rows, cols, nnz = 2000, 3000, 40000
    rr = np.sort(rng.integers(0, rows, nnz)).astype(np.uint32)
    cc = rng.integers(0, cols, nnz).astype(np.uint32)
    vv = rng.random(nnz, dtype=np.float32)
    csr = api.csr_from_coo(rows, cols, rr, cc, vv)
    o = oracle.metcf(rows, csr["row_ptr"], csr["col_idx"], csr["data"])
    h = device_metcf(csr).to_numpy()
    for k in ("rwo", "tc_offset", "bits", "a2b", "data"):
        np.testing.assert_array_equal(h[k], o[k], err_msg=k)


@pytest.mark.parametrize("cols", [20000, 3_000_000])
def test_device_metcf_windows_of_every_sort_class(cols):
    """The device builder orders each window's entries in shared memory when
    the window holds up to 256 or up to 2,048 entries, and gathers larger
    windows for a radix sort: windows of 1, 200, 1,500, 2,048, 2,049 and
    about 9,000 entries (rows in random column order with duplicates, one row
    alone holding 6,000 entries), next to empty windows, give the oracle's
    arrays; with 32-bit sort keys (20,000 columns) and 64-bit ones (3,000,000
    columns, past the 2^21 a 32-bit key holds beside an 11-bit position)."""
    rng = np.random.default_rng(11)
    rows = 3001
    per_window = {0: 1, 1: 200, 2: 1500, 3: 2048, 4: 2049, 6: 9000, 9: 0, 10: 37}
    rr, cc = [], []
    for w, n in per_window.items():
        if w == 6:
            counts = [6000, 500, 500, 500, 500, 400, 400, 200]
        else:
            counts = np.bincount(rng.integers(0, 8, n), minlength=8)
        for r, k in enumerate(counts):
            rr.append(np.full(k, 8 * w + r, np.uint32))
            cc.append(rng.integers(0, cols, k).astype(np.uint32))  # duplicates included
    rr.append(rng.integers(100, rows, 5000).astype(np.uint32))
    cc.append(rng.integers(0, cols, 5000).astype(np.uint32))
    rr, cc = np.concatenate(rr), np.concatenate(cc)
    perm = rng.permutation(len(rr))
    rr, cc = rr[perm], cc[perm]
    vv = rng.random(len(rr), dtype=np.float32)
    csr = api.csr_from_coo(rows, cols, rr, cc, vv)
    o = oracle.metcf(rows, csr["row_ptr"], csr["col_idx"], csr["data"])
    h = device_metcf(csr).to_numpy()
    for k in ("rwo", "tc_offset", "bits", "a2b", "data"):
        np.testing.assert_array_equal(h[k], o[k], err_msg=k)


@pytest.mark.parametrize("case", ["column_past_cols", "window_start_after_its_end", "first_offset_not_zero",
                                  "last_offset_short", "last_offset_past_nnz"])
def test_device_metcf_refuses_a_malformed_csr(case):
    """A device CSR whose column indices or row offsets are inconsistent is
    refused with ACCSPMM_ERROR_INVALID_VALUE (every kernel of the build keeps
    its reads and writes inside the arrays; the host checks the flags they
    raise before any kernel indexes by the sorted entries)."""
    n = 4096
    rp, ci, v = synth.powerlaw_local(n=n, seed=2)
    rp, ci = rp.astype(np.uint32).copy(), ci.astype(np.uint32).copy()
    nnz = len(ci)
    if case == "column_past_cols":
        ci[100] = n + 5
    elif case == "window_start_after_its_end":
        rp[8] = rp[16] + 1  # window 1 (rows 8..15) would start after it ends
    elif case == "first_offset_not_zero":
        rp[0] = 1
    elif case == "last_offset_short":
        rp[-1] = nnz - 3
    else:
        rp[-1] = nnz + 3
    d = api.DeviceCSR.upload(dict(rows=n, cols=n, nnz=nnz, row_ptr=rp, col_idx=ci, data=v))
    with pytest.raises(capi.AccSpmmError) as e:
        api.DeviceMETCF.from_csr(d)
    assert e.value.status == capi.ERROR_INVALID_VALUE


def spmm_plain(m, B, K, prec=capi.PREC_TF32):
    dB = torch_dev(B)
    dC = empty_dev(m.c_rows, K)
    m.spmm(dB, dC, K, prec)
    torch.cuda.synchronize()
    return dC.cpu().numpy()[:m.c_rows]


@pytest.mark.parametrize("name", OK_CASES)
@pytest.mark.parametrize("K", [4, 32, 36, 64, 128, 200, 256, 516])
def test_spmm_tf32_matches_oracle(name, K):
    g = gold(name)
    csr = csr_of_gold(g)
    m = device_metcf(csr)
    h = m.to_numpy()
    B = np.random.default_rng(K).uniform(-1, 1, (csr["cols"], K)).astype(np.float32)
    got = spmm_plain(m, B, K)
    c64 = oracle.spmm_metcf_f64(h, csr["cols"], B)
    emu = oracle.spmm_metcf_tf32(h, csr["cols"], B)
    assert got.shape == c64.shape
    assert np.isfinite(got).all()
    assert rel_fro(got, emu) < TOL_TF32_VS_EMU
    assert rel_fro(got, c64) < TOL_TF32_VS_F64
    # rows past the last matrix row (window padding) are written as zeros
    assert not got[csr["rows"]:].any()


@pytest.mark.parametrize("K", [32, 64, 128, 256])
def test_spmm_3xtf32_matches_fp64(K):
    g = gold("plsym1000")
    csr = csr_of_gold(g)
    m = device_metcf(csr)
    h = m.to_numpy()
    B = synth.dense_scaled_normal(csr["cols"], K, seed=K)
    got = spmm_plain(m, B, K, capi.PREC_3XTF32)
    c64 = oracle.spmm_metcf_f64(h, csr["cols"], B)
    assert rel_fro(got, c64) < TOL_3XTF32_VS_F64
    assert max_row_rel(got, c64) < 1e-5
    tf = spmm_plain(m, B, K, capi.PREC_TF32)
    assert rel_fro(tf, c64) > 10 * rel_fro(got, c64)


def test_spmm_config1_against_csr_fp64():
    r, c, v = synth.powerlaw_symmetric(n=16384, seed=0)
    r, c, v = synth.expand_symmetric(r, c, v)
    csr = api.csr_from_coo(16384, 16384, r, c, v)
    m = device_metcf(csr)
    B = synth.dense_uniform(16384, 128, seed=0)
    got = spmm_plain(m, B, 128)
    ref = oracle.spmm_csr_f64(csr["row_ptr"], csr["col_idx"], csr["data"], B)
    assert rel_fro(got[:16384], ref) < TOL_TF32_VS_F64
    got3 = spmm_plain(m, B, 128, capi.PREC_3XTF32)
    assert rel_fro(got3[:16384], ref) < TOL_3XTF32_VS_F64


@pytest.mark.parametrize("name", ["longwin", "plsym1000", "rand203", "ragged_unsorted"])
@pytest.mark.parametrize("prec", [capi.PREC_TF32, capi.PREC_3XTF32])
@pytest.mark.parametrize("K", [32, 36, 64, 128, 200, 256, 516])
def test_adaptive_equals_plain(name, prec, K):
    """The adaptive entry point gives bit-identical rows to the plain one and
    zeros in the extra rows of its larger C, on both sides of the reference's
    K = 128 switch between tf32_mma_balance_kernel and _g128_kernel
    (include/tf32_comp.hpp:101-111) and at widths that are not multiples of
    32 or of the 128-column slice."""
    g = gold(name)
    csr = csr_of_gold(g)
    m = device_metcf(csr)
    a = m.adpbme()
    c_rows = a.c_rows()
    ah = a.to_numpy()
    assert c_rows == max(8 * (len(ah["group_offset"]) - 1), int(ah["row_indices"][-1]) + 8)
    B = np.random.default_rng(1).uniform(-1, 1, (csr["cols"], K)).astype(np.float32)
    dB = torch_dev(B)
    dC = empty_dev(c_rows, K)
    a.spmm(dB, dC, c_rows, K, prec)
    torch.cuda.synchronize()
    ad = dC.cpu().numpy()[:c_rows]
    pl = spmm_plain(m, B, K, prec)
    n = min(c_rows, pl.shape[0])
    np.testing.assert_array_equal(ad[:n], pl[:n])
    assert not ad[n:].any()


@pytest.mark.parametrize("name", ["plsym1000", "powerlaw40k"])
@pytest.mark.parametrize("K", [256, 512])
def test_adaptive_matches_oracle_above_k128(name, K):
    """The adaptive path in the regime the reference serves with
    tf32_mma_balance_g128_kernel (K > 128, include/mma_tf32.cuh:794-1042):
    against the oracle's TF32 emulation (1e-5) and FP64 (1e-3), every row,
    with zeros past the matrix's rows."""
    if name == "powerlaw40k":
        rp, ci, v = synth.powerlaw_local(n=40000, mean=16.0, d_max=1024, seed=5)
        csr = dict(rows=40000, cols=40000, nnz=len(ci), row_ptr=rp, col_idx=ci, data=v)
    else:
        csr = csr_of_gold(gold(name))
    m = device_metcf(csr)
    h = m.to_numpy()
    a = m.adpbme()
    cr = a.c_rows()
    B = np.random.default_rng(K + 1).uniform(-1, 1, (csr["cols"], K)).astype(np.float32)
    dC = empty_dev(cr, K)
    a.spmm(torch_dev(B), dC, cr, K)
    torch.cuda.synchronize()
    got = dC.cpu().numpy()
    rows = 8 * m.struct.num_windows
    emu = oracle.spmm_metcf_tf32(h, csr["cols"], B)
    c64 = oracle.spmm_metcf_f64(h, csr["cols"], B)
    assert np.isfinite(got).all()
    assert rel_fro(got[:rows], emu) < TOL_TF32_VS_EMU
    assert rel_fro(got[:rows], c64) < TOL_TF32_VS_F64
    assert max_row_rel(got[:rows], c64) < 10 * TOL_TF32_VS_F64
    assert not got[rows:].any()


def test_spmm_deterministic():
    g = gold("longwin")
    csr = csr_of_gold(g)
    m = device_metcf(csr)
    B = np.random.default_rng(2).uniform(-1, 1, (csr["cols"], 128)).astype(np.float32)
    a = spmm_plain(m, B, 128)
    b = spmm_plain(m, B, 128)
    np.testing.assert_array_equal(a, b)


def test_spmm_empty_matrix_writes_zeros():
    csr = dict(rows=20, cols=20, nnz=0, row_ptr=np.zeros(21, np.uint32),
               col_idx=np.zeros(0, np.uint32), data=np.zeros(0, np.float32))
    m = device_metcf(csr)
    assert m.struct.num_tiles == 0
    got = spmm_plain(m, np.ones((20, 32), np.float32), 32)
    assert got.shape == (24, 32) and not got.any()


def test_spmm_rejects_bad_arguments():
    g = gold("kat10")
    m = device_metcf(csr_of_gold(g))
    dB = torch_dev(np.ones((10, 32), np.float32))
    dC = empty_dev(16, 32)
    with pytest.raises(capi.AccSpmmError) as e:
        m.spmm(dB, dC, 30)
    assert e.value.status == capi.ERROR_INVALID_VALUE
    with pytest.raises(capi.AccSpmmError):
        m.spmm(dB.data_ptr() + 4, dC, 32)
    with pytest.raises(capi.AccSpmmError):
        m.spmm(dB, dC, 32, precision=7)


def test_row_identical_b_regime():
    """With every B row equal to v, C = rowsum(A) v^T: the only regime in which
    the reference kernels' output is trustworthy."""
    g = gold("plsym1000")
    csr = csr_of_gold(g)
    m = device_metcf(csr)
    v = np.random.default_rng(3).uniform(-1, 1, 64).astype(np.float32)
    B = np.tile(v, (csr["cols"], 1))
    got = spmm_plain(m, B, 64)
    rs = np.add.reduceat(csr["data"].astype(np.float64),
                         csr["row_ptr"][:-1].astype(np.int64)) if csr["nnz"] else None
    counts = np.diff(csr["row_ptr"].astype(np.int64))
    rs = np.where(counts > 0, rs, 0.0)
    ref = np.outer(rs, v.astype(np.float64))
    assert rel_fro(got[:csr["rows"]], ref) < TOL_TF32_VS_F64


@pytest.mark.slow
def test_scale_workload_properties():
    """The 1M-row workload at K=128: size-independent checks against an FP64
    CSR evaluation of row sums (C 1 = A (B 1)), linearity in B, determinism,
    and exact agreement of the adaptive and plain entry points."""
    rp, ci, vals = synth.powerlaw_local(n=1 << 20, seed=0)
    n = 1 << 20
    csr = dict(rows=n, cols=n, nnz=len(ci), row_ptr=rp, col_idx=ci, data=vals)
    m = device_metcf(csr)
    K = 128
    B1 = torch.rand((n, K), device="cuda") * 2 - 1
    B2 = torch.rand((n, K), device="cuda") * 2 - 1
    C1 = empty_dev(m.c_rows, K)
    C2 = empty_dev(m.c_rows, K)
    C12 = empty_dev(m.c_rows, K)
    m.spmm(B1, C1, K)
    m.spmm(B2, C2, K)
    B12 = (B1 + B2).contiguous()
    m.spmm(B12, C12, K)
    torch.cuda.synchronize()
    lin = (C12 - C1 - C2).norm() / C12.norm()
    assert lin.item() < 2e-3
    # row sums through an FP64 CSR SpMV
    bsum = B1.double().sum(1).cpu().numpy()
    row_of = np.repeat(np.arange(n), np.diff(rp.astype(np.int64)))
    ref = np.bincount(row_of, weights=vals.astype(np.float64) * bsum[ci], minlength=n)
    got = C1.double().sum(1).cpu().numpy()[:n]
    assert rel_fro(got, ref) < TOL_TF32_VS_F64
    C1b = empty_dev(m.c_rows, K)
    m.spmm(B1, C1b, K)
    torch.cuda.synchronize()
    assert torch.equal(C1, C1b)
    a = m.adpbme()
    cr = a.c_rows()
    Ca = empty_dev(cr, K)
    a.spmm(B1, Ca, cr, K)
    torch.cuda.synchronize()
    k = min(cr, m.c_rows)
    assert torch.equal(Ca[:k], C1[:k])


def test_tf32_rounding_is_rna_bit_exact():
    """With A = I, C = rna_tf32(B) exactly (include/ptx_tf32.hpp:19-24 rounds
    both operands with cvt.rna); B covers exact ties in both signs."""
    n, K = 64, 32
    csr = dict(rows=n, cols=n, nnz=n, row_ptr=np.arange(n + 1, dtype=np.uint32),
               col_idx=np.arange(n, dtype=np.uint32), data=np.ones(n, np.float32))
    m = device_metcf(csr)
    rng = np.random.default_rng(9)
    bits = rng.integers(0x30000000, 0x50000000, size=(n, K), dtype=np.uint32)
    bits[:, :8] = (bits[:, :8] & 0xFFFFE000) | 0x1000          # ties
    bits[:, 8:12] = (bits[:, 8:12] & 0xFFFFE000) | 0x0FFF      # just below
    bits[::2] |= 0x80000000                                     # negatives
    B = bits.view(np.float32)
    got = spmm_plain(m, B, K)[:n]
    want = np.vectorize(oracle.tf32_rna, otypes=[np.float32])(B)
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("K", [64, 128])
def test_autotune_picks_a_shape_that_is_used_and_correct(K):
    """At K = 128 the candidates include gathering from a packed B."""
    g = gold("plsym1000")
    csr = csr_of_gold(g)
    m = device_metcf(csr)
    h = m.to_numpy()
    B = np.random.default_rng(8).uniform(-1, 1, (csr["cols"], K)).astype(np.float32)
    dB = torch_dev(B)
    dC = empty_dev(m.c_rows, K)
    try:
        r = m.autotune(dB, dC, K)
        # the default shape is one of the candidates and may win
        assert r["slice_width"] in (32, 64, 128) and r["windows_per_cta"] >= 1
        assert r["candidates"] > 1 and r["best_ms"] <= r["default_ms"] + 1e-6
        assert r["packed_b"] in (-1, 0, 1)
        got = spmm_plain(m, B, K)
        c64 = oracle.spmm_metcf_f64(h, csr["cols"], B)
        assert rel_fro(got, c64) < TOL_TF32_VS_F64
        # the adaptive entry point uses the same tuned shape: identical rows
        a = m.adpbme()
        cr = a.c_rows()
        dCa = empty_dev(cr, K)
        a.spmm(dB, dCa, cr, K)
        torch.cuda.synchronize()
        n = min(cr, got.shape[0])
        np.testing.assert_array_equal(dCa.cpu().numpy()[:n], got[:n])
    finally:
        capi.load().accspmm_autotune_clear()


def test_heaviest_first_schedule_keeps_results_bitwise():
    """Launches of a few waves run their window blocks heaviest first; the
    schedule only changes which CTA runs a block, so plain and adaptive
    results are bitwise equal with and without it."""
    n, K = 16384, 128
    r, c, v = synth.expand_symmetric(*synth.powerlaw_symmetric(n=n, seed=3))
    csr = api.csr_from_coo(n, n, r, c, v)
    m = device_metcf(csr)
    a = m.adpbme()
    cr = a.c_rows()
    B = torch.rand((n, K), device="cuda") * 2 - 1
    got = {}
    for sched in ("1", "0"):
        with capi.option(capi.OPT_SCHEDULE, int(sched)):
            C = empty_dev(m.c_rows, K)
            Ca = empty_dev(cr, K)
            m.spmm(B, C, K)
            a.spmm(B, Ca, cr, K)
            torch.cuda.synchronize()
        got[sched] = (C, Ca)
    assert torch.equal(got["1"][0], got["0"][0])
    assert torch.equal(got["1"][1], got["0"][1])
    assert torch.equal(got["1"][0][:n], got["1"][1][:n])
    ref = oracle.spmm_csr_f64(csr["row_ptr"], csr["col_idx"], csr["data"], B.cpu().numpy())
    assert rel_fro(got["1"][0][:n].cpu().numpy(), ref) < TOL_TF32_VS_F64


def test_schedule_is_forgotten_with_its_matrix():
    """A schedule is kept per library-owned matrix and dropped when the
    matrix is destroyed: matrices built one after another (whose arrays may
    reuse the freed addresses) each get their own."""
    K = 64
    for seed in range(4):
        n = 4096 + 1024 * seed
        r, c, v = synth.expand_symmetric(*synth.powerlaw_symmetric(n=n, seed=10 + seed))
        csr = api.csr_from_coo(n, n, r, c, v)
        m = device_metcf(csr)
        B = np.random.default_rng(seed).uniform(-1, 1, (n, K)).astype(np.float32)
        C = empty_dev(m.c_rows, K)
        m.spmm(torch_dev(B), C, K)
        torch.cuda.synchronize()
        ref = oracle.spmm_csr_f64(csr["row_ptr"], csr["col_idx"], csr["data"], B)
        assert rel_fro(C[:n].cpu().numpy(), ref) < TOL_TF32_VS_F64
        m.destroy()


def test_spmm_calls_capture_into_a_cuda_graph():
    """After one call outside a capture (which derives and keeps the adaptive
    window offsets and the block schedule), the plain, adaptive and epilogue
    entry points can be captured into a CUDA graph; replays with new B
    contents give bitwise the results of direct calls.  A first adaptive call
    inside a capture is refused with a status, not run."""
    n, K = 16384, 128
    r, c, v = synth.expand_symmetric(*synth.powerlaw_symmetric(n=n, seed=5))
    csr = api.csr_from_coo(n, n, r, c, v)
    m = device_metcf(csr)
    a = m.adpbme()
    cr = a.c_rows()
    B = torch.rand((n, K), device="cuda") * 2 - 1
    bias = torch.rand((K,), device="cuda")
    C, Ca, Ce = empty_dev(m.c_rows, K), empty_dev(cr, K), empty_dev(m.c_rows, K)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        m.spmm(B, C, K, stream=s)  # outside any capture: builds the cached state
        a.spmm(B, Ca, cr, K, stream=s)
        m.spmm_bias_act(B, Ce, K, bias, capi.ACT_RELU, stream=s)
    s.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        st = torch.cuda.current_stream()
        m.spmm(B, C, K, stream=st)
        a.spmm(B, Ca, cr, K, stream=st)
        m.spmm_bias_act(B, Ce, K, bias, capi.ACT_RELU, stream=st)
    for seed in range(2):
        B.copy_(torch.rand((n, K), device="cuda", generator=torch.Generator("cuda").manual_seed(seed)) * 2 - 1)
        g.replay()
        torch.cuda.synchronize()
        D, Da, De = empty_dev(m.c_rows, K), empty_dev(cr, K), empty_dev(m.c_rows, K)
        m.spmm(B, D, K)
        a.spmm(B, Da, cr, K)
        m.spmm_bias_act(B, De, K, bias, capi.ACT_RELU)
        torch.cuda.synchronize()
        assert torch.equal(C, D) and torch.equal(Ca, Da) and torch.equal(Ce, De)
    a2 = m.adpbme()
    C2 = empty_dev(cr, K)
    g2 = torch.cuda.CUDAGraph()
    with pytest.raises(capi.AccSpmmError):
        with torch.cuda.graph(g2, stream=s):
            a2.spmm(B, C2, cr, K, stream=torch.cuda.current_stream())
    torch.cuda.synchronize()


@pytest.mark.parametrize("prec", [capi.PREC_TF32, capi.PREC_3XTF32])
@pytest.mark.parametrize("kernel", ["pipe", "bulk", "tma", "lean", "db", "staged"])
@pytest.mark.parametrize("name,K", [("plsym1000", 32), ("plsym1000", 128), ("longwin", 64)])
def test_measurement_kernel_variants(kernel, name, K, prec):
    """The kernel variants kept for measurement in libaccspmm_lab.so
    (ACCSPMM_OPT_KERNEL) compute the same product: bitwise equal to the
    product library's register-direct kernel where they cut the window blocks
    among the same 8 warps (lean, db, staged), within the TF32 emulation
    tolerance where they use 4 warps per CTA (pipe, bulk, tma: their warps'
    pieces, and so the partial-window sums, differ).  The product library
    refuses the variants."""
    lab = capi.load_lab()
    with pytest.raises(capi.AccSpmmError) as e:
        capi.set_option(capi.OPT_KERNEL, capi.KERNELS[kernel])
    assert e.value.status == capi.ERROR_UNSUPPORTED
    g = gold(name)
    csr = csr_of_gold(g)
    m = device_metcf(csr)
    h = m.to_numpy()
    B = np.random.default_rng(K).uniform(-1, 1, (csr["cols"], K)).astype(np.float32)
    dB = torch_dev(B)
    C0 = empty_dev(m.c_rows, K)
    m.spmm(dB, C0, K, prec)
    C1 = empty_dev(m.c_rows, K)
    with capi.option(capi.OPT_KERNEL, capi.KERNELS[kernel], lib=lab):
        capi.call_lab("accspmm_spmm_tf32", m.ref, ctypes.c_void_p(dB.data_ptr()),
                      ctypes.c_void_p(C1.data_ptr()), K, prec, None)
    torch.cuda.synchronize()
    capi.call_lab("accspmm_device_status", None)  # raises if a bounded wait expired
    if kernel in ("lean", "db", "staged"):
        assert torch.equal(C0, C1)
    got = C1.cpu().numpy()
    f64 = oracle.spmm_metcf_f64(h, csr["cols"], B)
    if prec == capi.PREC_TF32:
        assert rel_fro(got, oracle.spmm_metcf_tf32(h, csr["cols"], B)) < TOL_TF32_VS_EMU
        assert rel_fro(got, f64) < TOL_TF32_VS_F64
    else:
        assert rel_fro(got, f64) < TOL_3XTF32_VS_F64


def test_concurrent_callers_on_their_own_streams():
    """Host threads calling the plain and adaptive entry points at once, on
    their own streams, on shared and separate matrices (the per-matrix state
    is created under a lock by whichever call comes first): every result
    equals the single-threaded one bit for bit."""
    import threading
    mats = []
    for seed in (21, 22):
        n = 8192 + 4096 * seed % 3
        r, c, v = synth.expand_symmetric(*synth.powerlaw_symmetric(n=n, seed=seed))
        csr = api.csr_from_coo(n, n, r, c, v)
        m = device_metcf(csr)
        a = m.adpbme()
        mats.append((n, m, a, a.c_rows()))
    K = 64
    Bs = [torch.rand((n, K), device="cuda") * 2 - 1 for n, _, _, _ in mats]
    torch.cuda.synchronize()
    jobs = [(i % 2, i) for i in range(8)]
    out = {}

    def work(mi, j):
        n, m, a, cr = mats[mi]
        s = torch.cuda.Stream()
        C = empty_dev(m.c_rows, K)
        Ca = empty_dev(cr, K)
        m.spmm(Bs[mi], C, K, stream=s)
        a.spmm(Bs[mi], Ca, cr, K, stream=s)
        s.synchronize()
        out[j] = (C, Ca)

    threads = [threading.Thread(target=work, args=jb) for jb in jobs]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    for mi, j in jobs:
        n, m, a, cr = mats[mi]
        C = empty_dev(m.c_rows, K)
        Ca = empty_dev(cr, K)
        m.spmm(Bs[mi], C, K)
        a.spmm(Bs[mi], Ca, cr, K)
        torch.cuda.synchronize()
        assert torch.equal(out[j][0], C) and torch.equal(out[j][1], Ca)


def test_matmul_returns_a_tensor():
    """DeviceMETCF.matmul: the PyTorch-facing form of the plain entry point."""
    g = gold("rand203")
    csr = csr_of_gold(g)
    m = device_metcf(csr)
    B = torch.rand((csr["cols"], 36), device="cuda") * 2 - 1
    C = m.matmul(B)
    assert tuple(C.shape) == (csr["rows"], 36)
    D = empty_dev(m.c_rows, 36)
    m.spmm(B, D, 36)
    torch.cuda.synchronize()
    assert torch.equal(C, D[:csr["rows"]])
    with pytest.raises(ValueError):
        m.matmul(B[:10])


@pytest.mark.slow
def test_products_past_32_bit_element_offsets():
    """cols * K and rows * K beyond 2^32 elements (33.6 M rows at K = 128, a 17 GB
    B and C): every offset into B and C is a 64-bit product (the reference's
    32-bit `vint` offsets wrap there).  One entry per row, value 1, at column
    (7919 i) mod n, and B values exact in TF32, so C[i] must equal
    B[(7919 i) mod n] bit for bit -- checked on sampled rows, all rows past
    row 2^25 (whose offsets exceed 2^32) and the rows around that boundary."""
    n, K = (1 << 25) + 1024, 128
    i = np.arange(n, dtype=np.int64)
    col = ((i * 7919) % n).astype(np.uint32)
    csr = dict(rows=n, cols=n, nnz=n, row_ptr=np.arange(n + 1, dtype=np.uint32), col_idx=col,
               data=np.ones(n, np.float32))
    m = device_metcf(csr)
    r = (torch.arange(n, device="cuda", dtype=torch.int32) % 1000).float()
    B = torch.empty((n, K), device="cuda")
    torch.add(r[:, None], torch.arange(K, device="cuda", dtype=torch.float32)[None, :], out=B)
    B.div_(8)  # integers below 2048 over 8: exact in TF32
    del r
    C = empty_dev(m.c_rows, K)
    m.spmm(B, C, K)
    torch.cuda.synchronize()
    rng = np.random.default_rng(1)
    rows = np.concatenate([rng.integers(0, n, 4096), np.arange((1 << 25) - 8, n)])
    idx = torch.from_numpy(rows).cuda()
    want = B[torch.from_numpy(col[rows].astype(np.int64)).cuda()]
    assert torch.equal(C[idx], want)
    del B, C
    torch.cuda.empty_cache()


def test_bounded_wait_failure_path_reports_and_recovers():
    """A wait that nothing completes (the self-test kernel's mbarrier) gives up
    after its limit and reports ACCSPMM_ERROR_TIMEOUT through
    accspmm_device_status, which then clears it; no trap, and the context
    keeps working (a product computed right after is correct)."""
    import time
    capi.call("accspmm_device_status", None)  # start from a clear status
    t0 = time.perf_counter()
    capi.call("accspmm_selftest_bounded_wait", 50, None)
    with pytest.raises(capi.AccSpmmError) as e:
        capi.call("accspmm_device_status", None)
    assert e.value.status == capi.ERROR_TIMEOUT
    assert time.perf_counter() - t0 >= 0.05
    capi.call("accspmm_device_status", None)  # cleared
    with pytest.raises(capi.AccSpmmError):
        capi.call("accspmm_selftest_bounded_wait", 0, None)  # limit out of range
    g = gold("plsym1000")
    csr = csr_of_gold(g)
    m = device_metcf(csr)
    B = np.random.default_rng(3).uniform(-1, 1, (csr["cols"], 32)).astype(np.float32)
    C = empty_dev(m.c_rows, 32)
    m.spmm(torch_dev(B), C, 32)
    torch.cuda.synchronize()
    assert rel_fro(C.cpu().numpy()[:csr["rows"]],
                   oracle.spmm_csr_f64(csr["row_ptr"], csr["col_idx"], csr["data"], B)) < TOL_TF32_VS_F64


@pytest.mark.slow
def test_device_builders_match_the_oracle_at_full_size():
    """The 1M-row power-law matrix (32.2 M entries): the GPU METCF and AdpBME
    builders equal the oracle's restatement of the reference's host builders
    array for array, and the GPU balance decision equals the oracle's."""
    n = 1 << 20
    rp, ci, vals = synth.powerlaw_local(n=n, seed=0)
    csr = dict(rows=n, cols=n, nnz=len(ci), row_ptr=rp, col_idx=ci, data=vals)
    m = device_metcf(csr)
    o = oracle.metcf(n, rp, ci, vals)
    h = m.to_numpy()
    for k in ("rwo", "tc_offset", "bits", "a2b", "data"):
        np.testing.assert_array_equal(h[k], o[k], err_msg=k)
    assert m.balance_strategy() == oracle.balance_strategy(o["rwo"])
    a = m.adpbme().to_numpy()
    np.testing.assert_array_equal(a["group_offset"], oracle.adpbme_groups(o["rwo"]))
    np.testing.assert_array_equal(a["row_indices"], oracle.adpbme_row_indices(o["rwo"]))
    for k in ("tc_offset", "bits", "a2b", "data"):
        np.testing.assert_array_equal(a[k], o[k], err_msg=k)


@pytest.mark.slow
def test_packed_b_with_prefetch_is_bit_identical_at_full_size():
    """On the 1M-row power-law matrix (seed 0, K = 128, a 512 MB B) the packed
    kernel returns the same bits with its L2 prefetch of the rows two tile
    groups ahead (the default), without it (ACCSPMM_PREFETCH=0), and reading
    fp32 B directly (ACCSPMM_PACK=0), on the plain and adaptive entry points."""
    n, K = 1 << 20, 128
    rp, ci, vals = synth.powerlaw_local(n=n, seed=0)
    csr = dict(rows=n, cols=n, nnz=len(ci), row_ptr=rp, col_idx=ci, data=vals)
    m = device_metcf(csr)
    a = m.adpbme()
    cr = a.c_rows()
    dB = torch.rand((n, K), device="cuda", generator=torch.Generator(device="cuda").manual_seed(0)) * 2 - 1
    out = {}
    for pf, pk in (("1", "1"), ("0", "1"), ("1", "0")):
        with capi.option(capi.OPT_PREFETCH, int(pf)), capi.option(capi.OPT_PACK, -1 if pk == "1" else 0):
            C, Ca = empty_dev(m.c_rows, K), empty_dev(cr, K)
            m.spmm(dB, C, K)
            a.spmm(dB, Ca, cr, K)
            torch.cuda.synchronize()
        out[pf + pk] = (C, Ca)
    for key in ("01", "10"):
        assert torch.equal(out["11"][0], out[key][0]), key
        assert torch.equal(out["11"][1], out[key][1]), key
    assert torch.isfinite(out["11"][0]).all()


@pytest.mark.parametrize("K", [136, 256])
def test_packed_b_is_bit_identical(K):
    """TF32 launches at 128-column slices whose B is at least 4 MiB first
    pack B to 2.5 bytes a value (rounded to TF32; each 128-column slice of a
    row its halfwords of bits 31..16, then the nibbles of bits 15..12); the
    SpMM on the packed copy returns bitwise what
    the kernel reading B directly returns, on the plain and adaptive entry
    points, within the TF32 tolerance of FP64 on sampled rows."""
    n = 1 << 18
    rp, ci, vals = synth.powerlaw_local(n=n, seed=4)
    csr = dict(rows=n, cols=n, nnz=len(ci), row_ptr=rp, col_idx=ci, data=vals)
    m = device_metcf(csr)
    a = m.adpbme()
    cr = a.c_rows()
    dB = torch.rand((n, K), device="cuda") * 2 - 1
    out = {}
    for pk in ("1", "0"):
        with capi.option(capi.OPT_PACK, -1 if pk == "1" else 0):
            C, Ca = empty_dev(m.c_rows, K), empty_dev(cr, K)
            m.spmm(dB, C, K)
            a.spmm(dB, Ca, cr, K)
            torch.cuda.synchronize()
        out[pk] = (C, Ca)
    assert torch.equal(out["1"][0], out["0"][0]) and torch.equal(out["1"][1], out["0"][1])
    rows = np.sort(np.random.default_rng(K).choice(n, 2048, replace=False))
    sub_rp = np.concatenate([[0], np.cumsum(np.diff(rp.astype(np.int64))[rows])]).astype(np.uint32)
    sub_ci = np.concatenate([ci[rp[r]:rp[r + 1]] for r in rows])
    sub_v = np.concatenate([vals[rp[r]:rp[r + 1]] for r in rows])
    ref = oracle.spmm_csr_f64(sub_rp, sub_ci, sub_v, dB.cpu().numpy())
    got = out["1"][0][torch.from_numpy(rows).cuda()].cpu().numpy()
    assert rel_fro(got, ref) < TOL_TF32_VS_F64


@pytest.mark.gpu
@pytest.mark.parametrize("K", [16, 32, 40, 64, 72, 128, 200])
def test_forced_packing_on_a_small_b_is_bit_identical(K):
    """ACCSPMM_OPT_PACK = 1 packs B wherever the launch shape allows, also below the
    default rule's 4 MiB, in 128-column slices (K = 72, 128, 200), in the
    160-byte 64-column slices of the K <= 64 shape (K = 40, 64) and in the
    80-byte 32-column slices of the K <= 32 shape (K = 16, 32): ragged last
    slices, rows that are not a multiple of the window height, the plain and
    adaptive entry points; with the L2 prefetch of rows two tile groups ahead
    forced on and off (128- and 64-column slices)."""
    n = 5003
    rp, ci, vals = synth.powerlaw_local(n=n, seed=7)
    csr = dict(rows=n, cols=n, nnz=len(ci), row_ptr=rp, col_idx=ci, data=vals)
    m = device_metcf(csr)
    a = m.adpbme()
    cr = a.c_rows()
    dB = torch.rand((n, K), device="cuda") * 2 - 1
    out = {}
    for pk, pf in (("2", -1), ("0", -1), ("2", 1), ("2", 0)):
        with capi.option(capi.OPT_PACK, 1 if pk == "2" else 0), capi.option(capi.OPT_PREFETCH, pf):
            C, Ca = empty_dev(m.c_rows, K), empty_dev(cr, K)
            m.spmm(dB, C, K)
            a.spmm(dB, Ca, cr, K)
            torch.cuda.synchronize()
        out[pk if pf < 0 else f"{pk}pf{pf}"] = (C, Ca)
    for key in ("0", "2pf1", "2pf0"):
        assert torch.equal(out["2"][0], out[key][0]) and torch.equal(out["2"][1], out[key][1]), key
    ref = oracle.spmm_csr_f64(rp, ci, vals, dB.cpu().numpy())
    assert rel_fro(out["2"][0][:n].cpu().numpy(), ref) < TOL_TF32_VS_F64
