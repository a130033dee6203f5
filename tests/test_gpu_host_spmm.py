"""accspmm_spmm_host: SpMM with B and C in host memory, pipelined by feature
slice.  Its result must be bit-identical to the device entry points on the
same inputs, whether C is written by the kernel straight into page-locked
host memory or staged on the device and copied back (pageable or unaligned
C), for the plain and the adaptive path, both precisions, and K that is not
a multiple of the slice width."""
import ctypes

import numpy as np
import pytest

from accspmm_gb300 import api, capi, synth
from tests.helpers import empty_dev, gold, torch_dev

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def device_matrix(name):
    if name == "powerlaw40k":
        rp, ci, v = synth.powerlaw_local(n=40000, mean=16.0, d_max=1024, seed=5)
        csr = dict(rows=40000, cols=40000, nnz=len(ci), row_ptr=rp, col_idx=ci, data=v)
    else:
        g = gold(name)
        csr = dict(rows=int(g["dims"][0]), cols=int(g["dims"][1]), nnz=int(g["dims"][2]),
                   row_ptr=g["csr_row_ptr"], col_idx=g["csr_col_idx"], data=g["csr_data"])
    m = api.DeviceMETCF.from_csr(api.DeviceCSR.upload(csr))
    torch.cuda.synchronize()
    return m, csr["cols"]


def pinned(shape, fill=np.nan):
    t = torch.empty(shape, dtype=torch.float32, pin_memory=True)
    t.fill_(fill)
    return t


@pytest.mark.parametrize("name", ["plsym1000", "longwin", "powerlaw40k"])
@pytest.mark.parametrize("K", [64, 100, 128])
def test_plain_host_entry_matches_device_entry_bitwise(name, K):
    m, cols = device_matrix(name)
    Bn = np.random.default_rng(K).uniform(-1, 1, (cols, K)).astype(np.float32)
    dB = torch_dev(Bn)
    want = empty_dev(m.c_rows, K)
    m.spmm(dB, want, K)
    Bh = pinned((cols, K))
    Bh.copy_(torch.from_numpy(Bn))
    Ch = pinned((m.c_rows, K))
    s = torch.cuda.Stream()
    m.spmm_host(Bh, Ch, K, capi.PREC_TF32, s)
    s.synchronize()
    assert torch.equal(Ch, want.cpu())


@pytest.mark.parametrize("prec", [capi.PREC_TF32, capi.PREC_3XTF32])
def test_adaptive_host_entry_matches_device_entry_bitwise(prec):
    m, cols = device_matrix("powerlaw40k")
    a = m.adpbme()
    cr = a.c_rows()
    K = 128
    Bn = np.random.default_rng(9).uniform(-1, 1, (cols, K)).astype(np.float32)
    want = empty_dev(cr, K)
    a.spmm(torch_dev(Bn), want, cr, K, prec)
    Bh = pinned((cols, K))
    Bh.copy_(torch.from_numpy(Bn))
    Ch = pinned((m.c_rows, K))
    a.spmm_host(Bh, Ch, K, prec)
    torch.cuda.synchronize()
    assert torch.equal(Ch, want[:m.c_rows].cpu())


def test_pageable_and_unaligned_c_are_staged_with_the_same_bits():
    m, cols = device_matrix("powerlaw40k")
    K = 64
    Bn = np.random.default_rng(2).uniform(-1, 1, (cols, K)).astype(np.float32)
    want = empty_dev(m.c_rows, K)
    m.spmm(torch_dev(Bn), want, K)
    want = want.cpu().numpy()
    # pageable B and C (numpy arrays)
    Cn = np.full((m.c_rows, K), np.nan, np.float32)
    m.spmm_host(Bn, Cn, K)
    torch.cuda.synchronize()
    assert np.array_equal(Cn, want)
    # page-locked C that is not 16-byte aligned: staged, not written directly
    buf = pinned((m.c_rows * K + 1,))
    Cu = buf[1:].view(m.c_rows, K)
    assert Cu.data_ptr() % 16 == 4
    m.spmm_host(Bn, Cu, K)
    torch.cuda.synchronize()
    assert np.array_equal(Cu.numpy(), want)


def test_repeated_calls_on_one_stream_reuse_the_pool():
    m, cols = device_matrix("longwin")
    K = 128
    s = torch.cuda.Stream()
    outs = []
    for seed in range(3):
        Bh = pinned((cols, K))
        Bh.copy_(torch.from_numpy(np.random.default_rng(seed).uniform(-1, 1, (cols, K)).astype(np.float32)))
        Ch = pinned((m.c_rows, K))
        m.spmm_host(Bh, Ch, K, capi.PREC_TF32, s)
        outs.append((Bh, Ch))
    s.synchronize()
    for Bh, Ch in outs:
        want = empty_dev(m.c_rows, K)
        m.spmm(Bh.cuda(), want, K)
        torch.cuda.synchronize()
        assert torch.equal(Ch, want.cpu())


def test_argument_errors():
    m, cols = device_matrix("kat10")
    Bh, Ch = pinned((cols, 8)), pinned((m.c_rows, 8))
    lib = capi.load()
    st = lib.accspmm_spmm_host(None, None, Bh.data_ptr(), Ch.data_ptr(), 8, 0, None)
    assert st == capi.ERROR_INVALID_VALUE
    with pytest.raises(capi.AccSpmmError):
        m.spmm_host(Bh, Ch, 6)


def test_gather_floor_is_a_positive_time_below_the_spmm():
    """The gather floor is a measurement entry point of libaccspmm_lab.so;
    the product library refuses it."""
    m, cols = device_matrix("powerlaw40k")
    K = 128
    B = torch_dev(np.random.default_rng(3).uniform(-1, 1, (cols, K)).astype(np.float32))
    ms = ctypes.c_float(0.0)
    st = capi.load().accspmm_gather_floor(m.ref, ctypes.c_void_p(B.data_ptr()), K, 0, 3, ctypes.byref(ms), None)
    assert st == capi.ERROR_UNSUPPORTED
    floor = m.gather_floor(B, K, 5)
    assert floor > 0
    for w in (32, 64, 128):
        assert m.gather_floor(B, K, 3, slice_width=w) > 0
    with pytest.raises(capi.AccSpmmError):
        m.gather_floor(B, K, 3, slice_width=48)
    C = empty_dev(m.c_rows, K)
    t = api.time_spmm(m, None, B, C, m.c_rows, K, capi.PREC_TF32, 2, 5)
    assert floor < 1.5 * t


def test_adaptive_window_offsets_cached_per_object_and_forgotten_on_destroy():
    # repeated adaptive calls on a library-owned AdpBME reuse its derived
    # window offsets; destroying it and building another (whose arrays may
    # land at the same addresses) must not reuse stale offsets
    K = 64
    outs = []
    for name in ("powerlaw40k", "plsym1000", "powerlaw40k", "longwin"):
        m, cols = device_matrix(name)
        a = m.adpbme()
        cr = a.c_rows()
        B = torch_dev(np.random.default_rng(11).uniform(-1, 1, (cols, K)).astype(np.float32))
        want = empty_dev(m.c_rows, K)
        m.spmm(B, want, K)
        for _ in range(2):
            got = empty_dev(cr, K)
            a.spmm(B, got, cr, K)
            torch.cuda.synchronize()
            assert torch.equal(got[:m.c_rows], want)
        outs.append(want.cpu())
        a.destroy()
        m.destroy()
    assert torch.equal(outs[0], outs[2])
