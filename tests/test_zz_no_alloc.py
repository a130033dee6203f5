"""The allocation-free adaptive SpMM entry point.

Some callers cannot allocate device memory when they call the library:
plugins inside a host application that owns all device memory through its own
pool, latency-critical loops in which cudaFree's device-wide synchronisation
would stall other streams, and processes with a device-memory budget fixed at
start-up.  For them
accspmm_spmm_adaptive_noalloc keeps its scratch in an array compiled into the
library.  These tests call it through the C ABI and check that it returns
bit for bit what accspmm_spmm_adaptive returns (both sum partial windows in
the same fixed order), on two calls in a row (the shared scratch keeps the
previous call's contents), also when the second call needs fewer windows
than the first, on a B large enough that accspmm_spmm_adaptive packs it and
this entry point does not; that inconsistent rowIndices are reported by
accspmm_device_status; and that sizes past its limit are refused.  The file
is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

from accspmm_gb300 import api, capi, synth
from tests.helpers import empty_dev, gold, torch_dev

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def device_adpbme(name):
    if name == "powerlaw256k":  # 262,144 rows: a B of 128 MiB at K = 128
        rp, ci, v = synth.powerlaw_local(n=1 << 18, seed=11)
        csr = dict(rows=1 << 18, cols=1 << 18, nnz=len(ci), row_ptr=rp, col_idx=ci, data=v)
    else:
        g = gold(name)
        csr = dict(rows=int(g["dims"][0]), cols=int(g["dims"][1]), nnz=int(g["dims"][2]),
                   row_ptr=g["csr_row_ptr"], col_idx=g["csr_col_idx"], data=g["csr_data"])
    m = api.DeviceMETCF.from_csr(api.DeviceCSR.upload(csr))
    a = m.adpbme()
    torch.cuda.synchronize()
    return m, a, csr["cols"]


def noalloc(a, B, C_out, c_rows, K, prec=capi.PREC_TF32):
    capi.call("accspmm_spmm_adaptive_noalloc", a.ref, C.c_void_p(B.data_ptr()),
              C.c_void_p(C_out.data_ptr()), c_rows, K, prec, None)


@pytest.fixture(autouse=True)
def clean_status():
    capi.load().accspmm_device_status(None)  # findings of earlier tests are not this file's
    yield


@pytest.mark.parametrize("prec", [capi.PREC_TF32, capi.PREC_3XTF32])
@pytest.mark.parametrize("K", [64, 128])
def test_noalloc_matches_adaptive_on_two_calls(prec, K):
    # plsym1000 needs more windows than longwin: its scratch contents stay
    # behind when longwin's calls follow
    for name in ("plsym1000", "longwin"):
        m, a, cols = device_adpbme(name)
        c_rows = a.c_rows()
        B = torch_dev(np.random.default_rng(4).uniform(-1, 1, (cols, K)).astype(np.float32))
        ref = empty_dev(c_rows, K)
        a.spmm(B, ref, c_rows, K, prec)
        for _ in range(2):  # the second call reuses the scratch left by the first
            out = empty_dev(c_rows, K)
            noalloc(a, B, out, c_rows, K, prec)
            torch.cuda.synchronize()
            assert torch.equal(out, ref)
    capi.call("accspmm_device_status", None)


def test_noalloc_matches_adaptive_on_a_large_b():
    """A 128 MiB B at K = 128: accspmm_spmm_adaptive packs it to 2.5-byte TF32
    rows, the allocation-free entry reads it directly; the same bits."""
    m, a, cols = device_adpbme("powerlaw256k")
    K = 128
    c_rows = a.c_rows()
    B = torch.rand((cols, K), device="cuda", generator=torch.Generator(device="cuda").manual_seed(5)) * 2 - 1
    assert B.numel() * 4 >= 128 << 20
    ref = empty_dev(c_rows, K)
    a.spmm(B, ref, c_rows, K)
    for _ in range(2):
        out = empty_dev(c_rows, K)
        noalloc(a, B, out, c_rows, K)
        torch.cuda.synchronize()
        assert torch.equal(out, ref)
    capi.call("accspmm_device_status", None)


def test_noalloc_reports_inconsistent_row_indices():
    """A c_rows that leaves the last tiles' windows out, and rowIndices that
    decrease, are found in stream order and reported by
    accspmm_device_status (the call itself does not wait)."""
    m, a, cols = device_adpbme("plsym1000")
    h = a.to_numpy()
    K = 32
    B = torch_dev(np.random.default_rng(6).uniform(-1, 1, (cols, K)).astype(np.float32))
    out = empty_dev(a.c_rows(), K)
    noalloc(a, B, out, int(h["row_indices"][-1]), K)  # one window short
    st = capi.load().accspmm_device_status(None)
    assert st == capi.ERROR_INVALID_VALUE
    assert "c_rows" in capi.load().accspmm_last_error().decode()
    assert capi.load().accspmm_device_status(None) == capi.SUCCESS
    # a caller-filled AdpBME whose rowIndices decrease
    ri = h["row_indices"].copy()
    t = int(np.nonzero(np.diff(ri.astype(np.int64)) > 0)[0][0])
    ri[t] = ri[t + 1] + 8
    keep = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in
            (("go", h["group_offset"].view(np.int32)), ("tco", h["tc_offset"].view(np.int32)),
             ("ri", ri.view(np.int32)), ("bits", h["bits"].view(np.int64)), ("a2b", h["a2b"].view(np.int32)),
             ("data", h["data"]))}

    def p(key, ct):
        return C.cast(C.c_void_p(keep[key].data_ptr()), C.POINTER(ct))

    bad = capi.ADPBME(h["rows"], h["cols"], h["nnz"], len(h["bits"]), len(h["group_offset"]) - 1,
                      p("go", C.c_uint32), p("tco", C.c_uint32), p("ri", C.c_uint32), p("bits", C.c_uint64),
                      p("a2b", C.c_uint32), p("data", C.c_float), capi.DEVICE, 0)
    capi.call("accspmm_spmm_adaptive_noalloc", C.byref(bad), C.c_void_p(B.data_ptr()),
              C.c_void_p(out.data_ptr()), a.c_rows(), K, capi.PREC_TF32, None)
    assert capi.load().accspmm_device_status(None) == capi.ERROR_INVALID_VALUE
    assert "non-decreasing" in capi.load().accspmm_last_error().decode()


def test_noalloc_rejects_sizes_past_its_limit():
    m, a, cols = device_adpbme("kat10")
    limit = capi.load().accspmm_noalloc_max_c_rows()
    assert limit == 8 * ((1 << 20) - 2)
    B = empty_dev(cols, 32, 0.0)
    out = empty_dev(8, 32)
    with pytest.raises(capi.AccSpmmError) as e:
        noalloc(a, B, out, limit + 8, 32)
    assert e.value.status == capi.ERROR_INVALID_VALUE
    assert "allocation-free maximum" in str(e.value)
