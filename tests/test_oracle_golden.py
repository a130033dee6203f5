"""The oracle pinned against the reference's own host code (golden fixtures).

Fixtures in tests/golden/ were produced by the reference's include/mmio.hpp and
include/format.hpp compiled from source (tests/golden/make_golden.py).
"""
import glob
import os

import numpy as np
import pytest

from oracle import oracle

GOLD = os.path.join(os.path.dirname(__file__), "golden")
CASES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLD, "*.npz")))


def load(name):
    return dict(np.load(os.path.join(GOLD, name + ".npz")))


@pytest.mark.parametrize("name", CASES)
def test_reader_matches_reference(name):
    g = load(name)
    st, coo = oracle.read_mtx(os.path.join(GOLD, "inputs", name + ".mtx"))
    assert st == int(g["status"][0])
    if st != 0:
        return
    assert [coo["rows"], coo["cols"], coo["nnz"]] == g["dims"].tolist()
    np.testing.assert_array_equal(coo["row"], g["coo_row"])
    np.testing.assert_array_equal(coo["col"], g["coo_col"])
    np.testing.assert_array_equal(coo["data"], g["coo_data"])


@pytest.mark.parametrize("name", [c for c in CASES if int(load(c)["status"][0]) == 0])
def test_formats_match_reference(name):
    g = load(name)
    rows = int(g["dims"][0])
    rp, ci, v = oracle.csr_from_coo(rows, g["coo_row"], g["coo_col"], g["coo_data"])
    np.testing.assert_array_equal(rp, g["csr_row_ptr"])
    np.testing.assert_array_equal(ci, g["csr_col_idx"])
    np.testing.assert_array_equal(v, g["csr_data"])
    m = oracle.metcf(rows, rp, ci, v)
    np.testing.assert_array_equal(m["rwo"], g["m_rwo"])
    np.testing.assert_array_equal(m["tc_offset"], g["m_tc_offset"])
    np.testing.assert_array_equal(m["bits"], g["m_bits"])
    np.testing.assert_array_equal(m["a2b"], g["m_a2b"])
    np.testing.assert_array_equal(m["data"], g["m_data"])
    assert oracle.balance_strategy(m["rwo"]) == int(g["balance"][0])
    if "a_group_offset" in g:
        np.testing.assert_array_equal(oracle.adpbme_groups(m["rwo"]), g["a_group_offset"])
        np.testing.assert_array_equal(oracle.adpbme_groups(m["rwo"], 2, 3, 5, 4),
                                      g["b_group_offset"])
        np.testing.assert_array_equal(oracle.adpbme_row_indices(m["rwo"]), g["a_row_indices"])
        # AdpBME's per-tile arrays equal METCF's (include/format.hpp:384-427)
        for k in ("tc_offset", "bits", "a2b", "data"):
            np.testing.assert_array_equal(g["a_" + k], g["m_" + k])


def test_known_answer_10x10():
    """The 10x10 symmetric case worked by hand from include/format.hpp:215-274."""
    st, coo = oracle.read_mtx(os.path.join(GOLD, "inputs", "kat10.mtx"))
    assert st == 0
    rp, ci, v = oracle.csr_from_coo(coo["rows"], coo["row"], coo["col"], coo["data"])
    m = oracle.metcf(coo["rows"], rp, ci, v)
    inf = 0xFFFFFFFF
    assert m["a2b"].tolist() == [0, 2, 4, 8, 9, inf, inf, inf, 1, 3, 8, 9, inf, inf, inf, inf]
    assert m["data"].tolist() == [1, 2, 3, 2, 4, 5, 3, 6, 4, 6]
    assert m["rwo"].tolist() == [0, 1, 2]


def test_tf32_rounding():
    # ties away from zero at the 13th bit, NaN/Inf preserved
    import struct
    f = lambda u: struct.unpack("<f", struct.pack("<I", u))[0]
    bits = lambda x: struct.unpack("<I", struct.pack("<f", x))[0]
    assert bits(oracle.tf32_rna(f(0x3F801000))) == 0x3F802000  # tie -> away
    assert bits(oracle.tf32_rna(f(0xBF801000))) == 0xBF802000
    assert bits(oracle.tf32_rna(f(0x3F800FFF))) == 0x3F800000
    assert bits(oracle.tf32_rna(f(0x3F801001))) == 0x3F802000
    assert np.isinf(oracle.tf32_rna(float("inf")))
    assert np.isnan(oracle.tf32_rna(float("nan")))


def test_spmm_oracles_agree():
    g = load("rand203")
    rows, cols = int(g["dims"][0]), int(g["dims"][1])
    m = {"rwo": g["m_rwo"], "tc_offset": g["m_tc_offset"], "bits": g["m_bits"],
         "a2b": g["m_a2b"], "data": g["m_data"]}
    B = np.random.default_rng(0).uniform(-1, 1, (cols, 40)).astype(np.float32)
    c64 = oracle.spmm_metcf_f64(m, cols, B)
    ref = oracle.spmm_csr_f64(g["csr_row_ptr"], g["csr_col_idx"], g["csr_data"], B)
    np.testing.assert_allclose(c64[:rows], ref, rtol=1e-12, atol=1e-12)
    assert not c64[rows:].any()
    ctf = oracle.spmm_metcf_tf32(m, cols, B)
    err = np.linalg.norm(ctf - c64) / np.linalg.norm(c64)
    assert 1e-5 < err < 1e-3
    cpu = np.zeros((rows, 40), np.float32)
    oracle.spmm_csr_f32_omp(g["csr_row_ptr"], g["csr_col_idx"], g["csr_data"], B, cpu)
    assert np.linalg.norm(cpu - ref) / np.linalg.norm(ref) < 1e-6
