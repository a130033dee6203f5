"""The adaptive path checks the rowIndices it derives window offsets from.

The reference sizes the adaptive C as max(8 G, rowIndices.back() + 8) rows
(src/mma_tf32.cu:112) and its CSR2AdpBME writes rowIndices as the first row
of each tile's window, window by window (include/format.hpp:364).  A c_rows
that leaves the last tiles' windows out, or rowIndices that are not
non-decreasing multiples of 8, must not pass silently:
 - a library-owned AdpBME derives its offsets once, with a host wait, so the
   call itself returns ACCSPMM_ERROR_INVALID_VALUE;
 - an AdpBME the caller filled is checked on every call in stream order, and
   the finding is reported (and cleared) by accspmm_device_status.
"""
import ctypes as C

import numpy as np
import pytest

from accspmm_gb300 import api, capi
from tests.helpers import empty_dev, gold, torch_dev

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def owned(name):
    g = gold(name)
    csr = dict(rows=int(g["dims"][0]), cols=int(g["dims"][1]), nnz=int(g["dims"][2]),
               row_ptr=g["csr_row_ptr"], col_idx=g["csr_col_idx"], data=g["csr_data"])
    m = api.DeviceMETCF.from_csr(api.DeviceCSR.upload(csr))
    a = m.adpbme()
    torch.cuda.synchronize()
    return m, a, csr["cols"]


class CallerAdpBME:
    """A device AdpBME whose arrays the caller owns (owned = 0), built from a
    host copy with rowIndices replaced."""

    def __init__(self, h: dict, row_indices=None):
        ri = h["row_indices"] if row_indices is None else row_indices
        self.t = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in
                  (("go", h["group_offset"].astype(np.int32)), ("tco", h["tc_offset"].astype(np.int32)),
                   ("ri", np.asarray(ri, np.uint32).astype(np.int32)), ("bits", h["bits"].view(np.int64)),
                   ("a2b", h["a2b"].view(np.int32)), ("data", h["data"]))}

        def p(key, ct):
            return C.cast(C.c_void_p(self.t[key].data_ptr()), C.POINTER(ct))

        self.s = capi.ADPBME(h["rows"], h["cols"], h["nnz"], len(h["bits"]), len(h["group_offset"]) - 1,
                             p("go", C.c_uint32), p("tco", C.c_uint32), p("ri", C.c_uint32),
                             p("bits", C.c_uint64), p("a2b", C.c_uint32), p("data", C.c_float),
                             capi.DEVICE, 0)

    @property
    def ref(self):
        return C.byref(self.s)


def adaptive(ref, B, out, c_rows, K, fn="accspmm_spmm_adaptive"):
    return getattr(capi.load(), fn)(ref, C.c_void_p(B.data_ptr()), C.c_void_p(out.data_ptr()),
                                    c_rows, K, capi.PREC_TF32, None)


def status():
    return capi.load().accspmm_device_status(None)


@pytest.fixture(autouse=True)
def clean_status():
    status()  # a finding left by an earlier test is not this test's
    yield
    status()


def test_owned_adpbme_refuses_c_rows_one_window_short():
    m, a, cols = owned("plsym1000")
    h = a.to_numpy()
    short = int(h["row_indices"][-1])  # one window short of rowIndices.back() + 8
    K = 64
    B = torch_dev(np.random.default_rng(0).uniform(-1, 1, (cols, K)).astype(np.float32))
    out = empty_dev(a.c_rows(), K)
    for _ in range(2):  # the finding is kept with the derived offsets
        assert adaptive(a.ref, B, out, short, K) == capi.ERROR_INVALID_VALUE
        assert "c_rows" in capi.load().accspmm_last_error().decode()
    assert adaptive(a.ref, B, out, a.c_rows(), K) == capi.SUCCESS
    assert status() == capi.SUCCESS


def test_caller_filled_adpbme_reports_inconsistent_row_indices():
    m, a, cols = owned("plsym1000")
    h = a.to_numpy()
    cr = a.c_rows()
    K = 64
    B = torch_dev(np.random.default_rng(1).uniform(-1, 1, (cols, K)).astype(np.float32))
    want = empty_dev(cr, K)
    a.spmm(B, want, cr, K)
    # consistent: same bits as the library-owned object, nothing reported
    good = CallerAdpBME(h)
    out = empty_dev(cr, K)
    assert adaptive(good.ref, B, out, cr, K) == capi.SUCCESS
    assert status() == capi.SUCCESS
    assert torch.equal(out, want)
    # c_rows one window short: the call is enqueued, the status reports it once
    assert adaptive(good.ref, B, out, int(h["row_indices"][-1]), K) == capi.SUCCESS
    assert status() == capi.ERROR_INVALID_VALUE
    assert "c_rows" in capi.load().accspmm_last_error().decode()
    assert status() == capi.SUCCESS
    # a decreasing rowIndices
    ri = h["row_indices"].copy()
    t = int(np.nonzero(np.diff(ri.astype(np.int64)) > 0)[0][0])  # ri[t] < ri[t + 1]
    ri[t] = ri[t + 1] + 8  # still a window start, now above its successor
    bad = CallerAdpBME(h, ri)
    assert adaptive(bad.ref, B, out, cr, K) == capi.SUCCESS
    assert status() == capi.ERROR_INVALID_VALUE
    assert "non-decreasing" in capi.load().accspmm_last_error().decode()
    # an entry that is not a window start
    ri2 = h["row_indices"].copy()
    ri2[len(ri2) // 2] += 3
    odd = CallerAdpBME(h, ri2)
    assert adaptive(odd.ref, B, out, cr, K) == capi.SUCCESS
    assert status() == capi.ERROR_INVALID_VALUE
    assert status() == capi.SUCCESS


def test_host_entry_reports_inconsistent_row_indices():
    m, a, cols = owned("longwin")
    h = a.to_numpy()
    ri = h["row_indices"].copy()
    ri[-1] += 1
    bad = CallerAdpBME(h, ri)
    K = 32
    Bh = torch.rand((cols, K), dtype=torch.float32).pin_memory()
    Ch = torch.empty((8 * ((h["rows"] + 7) // 8), K), dtype=torch.float32).pin_memory()
    st = capi.load().accspmm_spmm_host(None, bad.ref, C.c_void_p(Bh.data_ptr()), C.c_void_p(Ch.data_ptr()),
                                       K, capi.PREC_TF32, None)
    assert st == capi.SUCCESS
    assert status() == capi.ERROR_INVALID_VALUE
