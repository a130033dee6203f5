"""The allocation-free adaptive SpMM entry point.

Some callers cannot allocate device memory when they call the library:
plugins inside a host application that owns all device memory through its own
pool, latency-critical loops in which cudaFree's device-wide synchronisation
would stall other streams, and processes with a device-memory budget fixed at
start-up.  For them
accspmm_spmm_adaptive_noalloc keeps its scratch in an array compiled into the
library.  These tests call it through the C ABI and check that it returns
what accspmm_spmm_adaptive returns, on two calls in a row (the shared scratch
keeps the previous call's contents), and that sizes past its limit are
refused.  The file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

from accspmm_gb300 import api, capi
from tests.helpers import TOL_TF32_VS_EMU, empty_dev, gold, rel_fro, torch_dev

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def device_adpbme(name):
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


@pytest.mark.parametrize("prec", [capi.PREC_TF32, capi.PREC_3XTF32])
def test_noalloc_matches_adaptive_on_two_calls(prec):
    K = 64
    for name in ("longwin", "plsym1000"):
        m, a, cols = device_adpbme(name)
        c_rows = a.c_rows()
        B = torch_dev(np.random.default_rng(4).uniform(-1, 1, (cols, K)).astype(np.float32))
        ref = empty_dev(c_rows, K)
        a.spmm(B, ref, c_rows, K, prec)
        for _ in range(2):  # the second call reuses the scratch left by the first
            out = empty_dev(c_rows, K)
            noalloc(a, B, out, c_rows, K, prec)
            torch.cuda.synchronize()
            got = out.cpu().numpy()
            want = ref.cpu().numpy()
            assert np.isfinite(got).all()
            assert rel_fro(got, want) < TOL_TF32_VS_EMU
    capi.call("accspmm_device_status", None)


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
