"""The library's host builders against the reference's golden fixtures and the
oracle (no GPU needed)."""
import glob
import os

import numpy as np
import pytest

from accspmm_gb300 import api, capi, synth
from oracle import oracle

GOLD = os.path.join(os.path.dirname(__file__), "golden")
CASES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLD, "*.npz")))


def gold(name):
    return dict(np.load(os.path.join(GOLD, name + ".npz")))


def test_library_exports_every_header_function():
    lib = capi.load()
    names = capi.header_functions()
    assert len(names) >= 19
    for n in names:
        assert hasattr(lib, n), n
    assert b"sm_103a" in lib.accspmm_version()


@pytest.mark.parametrize("name", CASES)
def test_reader_matches_reference(name):
    g = gold(name)
    st, coo = api.read_from_mtx(os.path.join(GOLD, "inputs", name + ".mtx"))
    assert st == int(g["status"][0])
    if st != 0:
        assert coo is None
        return
    assert [coo["rows"], coo["cols"], coo["nnz"]] == g["dims"].tolist()
    np.testing.assert_array_equal(coo["row"], g["coo_row"])
    np.testing.assert_array_equal(coo["col"], g["coo_col"])
    np.testing.assert_array_equal(coo["data"], g["coo_data"])


def test_reader_missing_file():
    st, coo = api.read_from_mtx("/nonexistent/file.mtx")
    assert st == capi.MM_LOADING_FILE_ERROR and coo is None


@pytest.mark.parametrize("text", [
    "%%MatrixMarket matrix coordinate real general\n3 3 2\n1 1 1\n",           # truncated
    "%%MatrixMarket matrix coordinate real general\n3 3 1\n4 1 1\n",           # row out of range
    "%%MatrixMarket matrix coordinate real general\n3 3 1\n1 x 1\n",           # not a number
    "%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n",              # dense
])
def test_reader_rejects_malformed(tmp_path, text):
    p = tmp_path / "m.mtx"
    p.write_text(text)
    st, coo = api.read_from_mtx(str(p))
    assert st == capi.ERROR_READ_MTX


@pytest.mark.parametrize("name", [c for c in CASES if int(gold(c)["status"][0]) == 0])
def test_host_builders_match_reference(name):
    g = gold(name)
    rows, cols = int(g["dims"][0]), int(g["dims"][1])
    csr = api.csr_from_coo(rows, cols, g["coo_row"], g["coo_col"], g["coo_data"])
    np.testing.assert_array_equal(csr["row_ptr"], g["csr_row_ptr"])
    np.testing.assert_array_equal(csr["col_idx"], g["csr_col_idx"])
    np.testing.assert_array_equal(csr["data"], g["csr_data"])
    m = api.metcf_from_csr(csr)
    for k, gk in [("rwo", "m_rwo"), ("tc_offset", "m_tc_offset"), ("bits", "m_bits"),
                  ("a2b", "m_a2b"), ("data", "m_data")]:
        np.testing.assert_array_equal(m[k], g[gk], err_msg=k)
    assert api.balance_strategy(m) == int(g["balance"][0])
    if "a_group_offset" in g:
        a = api.adpbme_from_metcf(m)
        for k, gk in [("group_offset", "a_group_offset"), ("tc_offset", "a_tc_offset"),
                      ("row_indices", "a_row_indices"), ("bits", "a_bits"), ("a2b", "a_a2b"),
                      ("data", "a_data")]:
            np.testing.assert_array_equal(a[k], g[gk], err_msg=k)
        b = api.adpbme_from_metcf(m, 2, 3, 5, 4)
        np.testing.assert_array_equal(b["group_offset"], g["b_group_offset"])


@pytest.mark.parametrize("seed", [0, 1])
def test_host_metcf_matches_oracle_on_config1_shape(seed):
    """The 16,384-row symmetric power-law workload, host builder vs oracle."""
    r, c, v = synth.powerlaw_symmetric(n=16384, seed=seed)
    r, c, v = synth.expand_symmetric(r, c, v)
    csr = api.csr_from_coo(16384, 16384, r, c, v)
    rp, ci, vals = oracle.csr_from_coo(16384, r, c, v)
    np.testing.assert_array_equal(csr["row_ptr"], rp)
    np.testing.assert_array_equal(csr["col_idx"], ci)
    m = api.metcf_from_csr(csr)
    o = oracle.metcf(16384, rp, ci, vals)
    for k in ("rwo", "tc_offset", "bits", "a2b", "data"):
        np.testing.assert_array_equal(m[k], o[k], err_msg=k)
    a = api.adpbme_from_metcf(m)
    np.testing.assert_array_equal(a["group_offset"], oracle.adpbme_groups(o["rwo"]))
    assert api.balance_strategy(m) == oracle.balance_strategy(o["rwo"])


def test_host_metcf_unsorted_duplicates_random():
    """Unsorted rows with duplicate entries (the reference keeps both)."""
    rng = np.random.default_rng(5)
    rows, cols, nnz = 333, 120, 4000
    r = np.sort(rng.integers(0, rows, nnz)).astype(np.uint32)
    c = rng.integers(0, cols, nnz).astype(np.uint32)
    v = rng.random(nnz, dtype=np.float32)
    csr = api.csr_from_coo(rows, cols, r, c, v)
    m = api.metcf_from_csr(csr)
    o = oracle.metcf(rows, csr["row_ptr"], csr["col_idx"], csr["data"])
    for k in ("rwo", "tc_offset", "bits", "a2b", "data"):
        np.testing.assert_array_equal(m[k], o[k], err_msg=k)


def test_host_metcf_empty_and_rectangular():
    csr = dict(rows=17, cols=5, nnz=0, row_ptr=np.zeros(18, np.uint32),
               col_idx=np.zeros(0, np.uint32), data=np.zeros(0, np.float32))
    m = api.metcf_from_csr(csr)
    assert m["rwo"].tolist() == [0, 0, 0, 0]
    assert m["tc_offset"].tolist() == [0]
    assert api.balance_strategy(m) == 0
    a = api.adpbme_from_metcf(m)
    assert a["group_offset"].tolist() == [0]


def test_invalid_csr_rejected():
    csr = dict(rows=2, cols=3, nnz=1, row_ptr=np.array([0, 1, 1], np.uint32),
               col_idx=np.array([7], np.uint32), data=np.ones(1, np.float32))
    with pytest.raises(capi.AccSpmmError) as e:
        api.metcf_from_csr(csr)
    assert e.value.status == capi.ERROR_INVALID_VALUE


@pytest.mark.parametrize("params", [(3, 1, 2, 16), (2, 3, 5, 4), (1, 0, 0, 1), (10, 5, 7, 60), (7, 7, 7, 100)])
def test_host_adpbme_groups_match_the_oracle(params):
    """The host AdpBME packing equals the oracle's greedy walk for the
    reference's parameters and for other cost settings (one-tile groups,
    large targets)."""
    rng = np.random.default_rng(sum(params))
    rows, cols, nnz = 4000, 3000, 60000
    r = np.sort(rng.integers(0, rows, nnz)).astype(np.uint32)
    c = rng.integers(0, cols, nnz).astype(np.uint32)
    v = rng.random(nnz, dtype=np.float32)
    csr = api.csr_from_coo(rows, cols, r, c, v)
    m = api.metcf_from_csr(csr)
    a = api.adpbme_from_metcf(m, *params)
    np.testing.assert_array_equal(a["group_offset"], oracle.adpbme_groups(m["rwo"], *params))
    np.testing.assert_array_equal(a["row_indices"], oracle.adpbme_row_indices(m["rwo"]))
