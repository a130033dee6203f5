"""The continuous-batching request server: results equal to the plain entry
point, the same bits alone and in a mix, chains, admission by HBM budget."""
import numpy as np
import pytest

from accspmm_gb300 import api, capi
from tests.test_gpu_batch import csr_of_gold, device_metcf_from_csr, random_csr

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def pinned(shape, fill=None):
    t = torch.empty(shape, dtype=torch.float32, pin_memory=True)
    if fill is not None:
        t.fill_(fill)
    return t


@pytest.fixture(scope="module")
def graphs():
    mats = [csr_of_gold("longwin"), csr_of_gold("plsym1000"), random_csr(3000, 3000, 10.0, 5),
            random_csr(20000, 20000, 8.0, 6)]
    return [device_metcf_from_csr(c) for c in mats]


def plain(m, B_host, K, prec=capi.PREC_TF32):
    dB = B_host.cuda()
    dC = torch.empty((m.c_rows, K), device="cuda")
    m.spmm(dB, dC, K, prec)
    torch.cuda.synchronize()
    return dC.cpu()


def test_server_alone_and_in_mix_are_bitwise_equal(graphs):
    srv = api.Server(graphs, hbm_budget_bytes=1 << 30, max_batch=16, streams=3)
    rng = np.random.default_rng(0)
    g0, K0 = 1, 64
    B0 = pinned((graphs[g0].struct.cols, K0))
    B0.copy_(torch.from_numpy(rng.uniform(-1, 1, B0.shape).astype(np.float32)))
    C_alone = pinned((graphs[g0].c_rows, K0), float("nan"))
    assert srv.wait(srv.submit(g0, B0, C_alone, K0)) == 0
    np.testing.assert_array_equal(C_alone.numpy(), plain(graphs[g0], B0, K0).numpy())
    # a mix: other graphs, widths and precisions, with the same request inside
    reqs = []
    for i in range(40):
        if i % 5 == 2:
            C = pinned((graphs[g0].c_rows, K0), float("nan"))
            reqs.append(("same", srv.submit(g0, B0, C, K0), C, None))
            continue
        g = int(rng.integers(0, len(graphs)))
        K = int(rng.choice([32, 36, 64, 128, 256]))
        prec = capi.PREC_3XTF32 if i % 7 == 3 else capi.PREC_TF32
        B = pinned((graphs[g].struct.cols, K))
        B.copy_(torch.from_numpy(rng.uniform(-1, 1, B.shape).astype(np.float32)))
        C = pinned((graphs[g].c_rows, K), float("nan"))
        reqs.append(((g, K, prec, B), srv.submit(g, B, C, K, prec), C, None))
    for kind, rid, C, _ in reqs:
        assert srv.wait(rid, 60000) == 0
        if kind == "same":
            np.testing.assert_array_equal(C.numpy(), C_alone.numpy())
        else:
            g, K, prec, B = kind
            np.testing.assert_array_equal(C.numpy(), plain(graphs[g], B, K, prec).numpy())
    st = srv.stats()
    assert st["completed"] == 41 and st["submitted"] == 41
    assert 0 < st["p50_ms"] <= st["p99_ms"] <= st["max_ms"]
    assert st["launches"] >= 1 and st["mean_batch"] >= 1.0
    srv.destroy()


def test_server_two_layer_chain(graphs):
    srv = api.Server(graphs, hbm_budget_bytes=1 << 30)
    m = graphs[2]  # square
    K = 32
    B = pinned((m.struct.cols, K))
    B.copy_(torch.rand(B.shape) * 2 - 1)
    C = pinned((m.c_rows, K), float("nan"))
    assert srv.wait(srv.submit(2, B, C, K, capi.PREC_TF32, chain=2)) == 0
    T = plain(m, B, K)
    want = plain(m, T[: m.struct.cols].contiguous(), K)
    np.testing.assert_array_equal(C.numpy(), want.numpy())
    srv.destroy()


def test_server_admission_budget(graphs):
    m = graphs[3]
    K = 128
    need = (m.struct.cols + m.c_rows) * K * 4
    # room for exactly one request of this size at a time
    srv = api.Server(graphs, hbm_budget_bytes=need + need // 2, max_batch=8, streams=4)
    B = pinned((m.struct.cols, K), 1.0)
    outs = [pinned((m.c_rows, K), float("nan")) for _ in range(6)]
    ids = [srv.submit(3, B, C, K) for C in outs]
    for rid in ids:
        assert srv.wait(rid, 60000) == 0
    ref = plain(m, B, K).numpy()
    for C in outs:
        np.testing.assert_array_equal(C.numpy(), ref)
    st = srv.stats()
    assert st["peak_bytes"] <= need + need // 2
    with pytest.raises(capi.AccSpmmError) as e:
        srv.submit(3, B, outs[0], 2048)
    assert e.value.status == capi.ERROR_ADMISSION
    srv.destroy()


def test_server_cancel_and_bad_requests(graphs):
    m = graphs[3]
    K = 256
    need = (m.struct.cols + m.c_rows) * K * 4
    srv = api.Server(graphs, hbm_budget_bytes=need, max_batch=1, streams=1)
    B = pinned((m.struct.cols, K), 1.0)
    outs = [pinned((m.c_rows, K)) for _ in range(8)]
    ids = [srv.submit(3, B, C, K) for C in outs]
    last = ids[-1]
    rc = srv.cancel(last)
    statuses = [srv.wait(r, 60000) for r in ids]
    assert all(s == 0 for s in statuses[:-1])
    if rc == 0:
        assert statuses[-1] == capi.ERROR_CANCELLED
    else:
        assert statuses[-1] == 0
    with pytest.raises(capi.AccSpmmError):
        srv.submit(99, B, outs[0], K)
    with pytest.raises(capi.AccSpmmError):
        srv.submit(0, B, outs[0], 30)
    with pytest.raises(capi.AccSpmmError):
        srv.submit(0, B, outs[0], 32, chain=2)  # graph 0 is not square
    srv.destroy()


def test_server_wait_limit_and_unknown_request(graphs):
    """A wait whose limit passes before the request is done returns
    ACCSPMM_ERROR_TIMEOUT and leaves the request running; waiting again
    without a limit returns its status.  Requests queue behind a one-slot,
    one-request budget, so the last of several is still pending when waited
    for with a zero limit."""
    m = graphs[3]
    K = 256
    need = (m.struct.cols + m.c_rows) * K * 4
    srv = api.Server(graphs, hbm_budget_bytes=need, max_batch=1, streams=1)
    B = pinned((m.struct.cols, K), 1.0)
    outs = [pinned((m.c_rows, K)) for _ in range(6)]
    ids = [srv.submit(3, B, C, K) for C in outs]
    assert srv.wait(ids[-1], 0) == capi.ERROR_TIMEOUT
    assert all(srv.wait(r, -1) == 0 for r in ids)
    want = plain(m, B, K)
    assert all(torch.equal(C, want) for C in outs)
    srv.destroy()
