"""Binary METCF / AdpBME files (no GPU needed): round trips are bit-exact
against the reference's golden formats, and damaged files -- truncated, wrong
magic, flipped payload bits, consistent checksums over inconsistent arrays --
are refused with ACCSPMM_ERROR_FORMAT before any array is returned."""
import os
import struct

import numpy as np
import pytest

from accspmm_gb300 import api, capi, synth
from tests.helpers import GOLD, gold

CASES = ["kat10", "longwin", "plsym1000", "rand203", "ragged_unsorted"]


def metcf_of(g):
    rows, cols, nnz = (int(x) for x in g["dims"])
    return dict(rows=rows, cols=cols, nnz=nnz, rwo=g["m_rwo"], tc_offset=g["m_tc_offset"],
                bits=g["m_bits"], a2b=g["m_a2b"], data=g["m_data"])


def adp_of(g):
    rows, cols, nnz = (int(x) for x in g["dims"])
    return dict(rows=rows, cols=cols, nnz=nnz, group_offset=g["a_group_offset"],
                tc_offset=g["a_tc_offset"], row_indices=g["a_row_indices"], bits=g["a_bits"],
                a2b=g["a_a2b"], data=g["a_data"])


@pytest.mark.parametrize("name", CASES)
def test_metcf_round_trip_is_bit_exact(name, tmp_path):
    g = gold(name)
    m = metcf_of(g)
    p = str(tmp_path / "m.metcf")
    api.save_metcf(m, p)
    back = api.load_metcf(p)
    for k in ("rwo", "tc_offset", "bits", "a2b", "data"):
        np.testing.assert_array_equal(back[k], m[k], err_msg=k)
    assert (back["rows"], back["cols"], back["nnz"]) == (m["rows"], m["cols"], m["nnz"])


@pytest.mark.parametrize("name", CASES)
def test_adpbme_round_trip_is_bit_exact(name, tmp_path):
    a = adp_of(gold(name))
    p = str(tmp_path / "a.adpbme")
    api.save_adpbme(a, p)
    back = api.load_adpbme(p)
    for k in ("group_offset", "tc_offset", "row_indices", "bits", "a2b", "data"):
        np.testing.assert_array_equal(back[k], a[k], err_msg=k)


def test_round_trip_of_a_built_power_law_matrix(tmp_path):
    rp, ci, v = synth.powerlaw_local(n=20000, mean=12.0, d_max=512, seed=3)
    csr = dict(rows=20000, cols=20000, nnz=len(ci), row_ptr=rp, col_idx=ci, data=v)
    m = api.metcf_from_csr(csr)
    p = str(tmp_path / "pl.metcf")
    api.save_metcf(m, p)
    back = api.load_metcf(p)
    for k in ("rwo", "tc_offset", "bits", "a2b", "data"):
        np.testing.assert_array_equal(back[k], m[k], err_msg=k)


def expect_format_error(fn, *args):
    with pytest.raises(capi.AccSpmmError) as e:
        fn(*args)
    assert e.value.status == capi.ERROR_FORMAT, str(e.value)
    return str(e.value)


def saved(tmp_path, name="plsym1000"):
    p = str(tmp_path / "m.metcf")
    api.save_metcf(metcf_of(gold(name)), p)
    return p


def test_missing_file_is_open_error(tmp_path):
    with pytest.raises(capi.AccSpmmError) as e:
        api.load_metcf(str(tmp_path / "absent.metcf"))
    assert e.value.status == capi.ERROR_OPEN_FILE


def test_truncated_file_is_refused(tmp_path):
    p = saved(tmp_path)
    data = open(p, "rb").read()
    for cut in (4, 20, len(data) // 2, len(data) - 1):
        open(p, "wb").write(data[:cut])
        expect_format_error(api.load_metcf, p)


def test_wrong_magic_or_kind_is_refused(tmp_path):
    p = saved(tmp_path)
    data = bytearray(open(p, "rb").read())
    expect_format_error(api.load_adpbme, p)  # a METCF file is not an AdpBME file
    data[0:8] = b"NOTMETCF"
    open(p, "wb").write(bytes(data))
    assert "magic" in expect_format_error(api.load_metcf, p)


def test_flipped_payload_bit_fails_the_checksum(tmp_path):
    p = saved(tmp_path)
    data = bytearray(open(p, "rb").read())
    data[len(data) // 2] ^= 0x10
    open(p, "wb").write(bytes(data))
    assert "checksum" in expect_format_error(api.load_metcf, p)


@pytest.mark.parametrize("damage", ["tc_offset_past_nnz", "popcount", "column_range", "rwo_order"])
def test_consistent_checksums_over_inconsistent_arrays_are_refused(damage, tmp_path):
    # files written through the library with valid checksums, whose arrays
    # would send a kernel out of bounds: the loader's validation refuses them
    m = metcf_of(gold("plsym1000"))
    m = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in m.items()}
    if damage == "tc_offset_past_nnz":
        m["tc_offset"][-1] += 8
    elif damage == "popcount":
        b = int(m["bits"][3])
        free = next(i for i in range(64) if not (b >> i) & 1)
        m["bits"][3] = np.uint64(b | (1 << free))  # more set bits than values
    elif damage == "column_range":
        m["a2b"][5] = m["cols"] + 3
    elif damage == "rwo_order":
        m["rwo"][4], m["rwo"][5] = m["rwo"][5] + 1, m["rwo"][4]
    p = str(tmp_path / "bad.metcf")
    api.save_metcf(m, p)
    expect_format_error(api.load_metcf, p)


def test_adpbme_with_unsorted_row_indices_is_refused(tmp_path):
    a = adp_of(gold("plsym1000"))
    a = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in a.items()}
    a["row_indices"][10], a["row_indices"][11] = a["row_indices"][11] + 8, a["row_indices"][10]
    p = str(tmp_path / "bad.adpbme")
    api.save_adpbme(a, p)
    expect_format_error(api.load_adpbme, p)


def test_header_fields_are_little_endian_sizes(tmp_path):
    g = gold("kat10")
    p = saved(tmp_path, "kat10")
    data = open(p, "rb").read()
    assert data[:8] == b"ACSPMTCF"
    ver, nf = struct.unpack("<II", data[8:16])
    fields = struct.unpack("<5I", data[16:36])
    assert (ver, nf) == (1, 5)
    assert fields == (10, 10, int(g["dims"][2]), len(g["m_rwo"]) - 1, len(g["m_bits"]))


@pytest.mark.gpu
def test_device_save_and_load_give_the_same_spmm(tmp_path):
    torch = pytest.importorskip("torch")
    from tests.helpers import empty_dev, torch_dev
    g = gold("plsym1000")
    csr = dict(rows=int(g["dims"][0]), cols=int(g["dims"][1]), nnz=int(g["dims"][2]),
               row_ptr=g["csr_row_ptr"], col_idx=g["csr_col_idx"], data=g["csr_data"])
    m = api.DeviceMETCF.from_csr(api.DeviceCSR.upload(csr))
    p = str(tmp_path / "d.metcf")
    m.save(p)
    m2 = api.DeviceMETCF.load(p)
    h1, h2 = m.to_numpy(), m2.to_numpy()
    for k in ("rwo", "tc_offset", "bits", "a2b", "data"):
        np.testing.assert_array_equal(h1[k], h2[k], err_msg=k)
    K = 64
    B = torch_dev(np.random.default_rng(1).uniform(-1, 1, (csr["cols"], K)).astype(np.float32))
    c1, c2 = empty_dev(m.c_rows, K), empty_dev(m2.c_rows, K)
    m.spmm(B, c1, K)
    m2.spmm(B, c2, K)
    torch.cuda.synchronize()
    assert torch.equal(c1, c2)
