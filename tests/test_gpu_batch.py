"""Batched SpMM: many matrices of different sizes and widths in one
persistent launch give the same bits as one plain launch per matrix."""
import numpy as np
import pytest

from accspmm_gb300 import api, capi, synth
from tests.helpers import empty_dev, gold, torch_dev

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def device_metcf_from_csr(csr):
    m = api.DeviceMETCF.from_csr(api.DeviceCSR.upload(csr))
    torch.cuda.synchronize()
    return m


def csr_of_gold(name):
    g = gold(name)
    return dict(rows=int(g["dims"][0]), cols=int(g["dims"][1]), nnz=int(g["dims"][2]),
                row_ptr=g["csr_row_ptr"], col_idx=g["csr_col_idx"], data=g["csr_data"])


def random_csr(rows, cols, mean_deg, seed):
    rng = np.random.default_rng(seed)
    deg = synth.powerlaw_degrees(rows, 2.1, mean_deg, min(cols, 512), rng)
    r = np.repeat(np.arange(rows, dtype=np.int64), deg)
    c = rng.integers(0, cols, size=r.size)
    r, c = synth._dedupe_sorted(r, c, cols)
    v = rng.random(r.size, dtype=np.float32)
    rp, ci, vals = synth.coo_to_csr(rows, r, c, v)
    return dict(rows=rows, cols=cols, nnz=len(ci), row_ptr=rp, col_idx=ci, data=vals)


def build_items(ks, seed=0):
    mats = [csr_of_gold("longwin"), csr_of_gold("plsym1000"), csr_of_gold("rand203"),
            csr_of_gold("ragged_unsorted"), random_csr(5000, 4000, 12.0, seed),
            random_csr(777, 9000, 30.0, seed + 1), random_csr(20000, 20000, 6.0, seed + 2)]
    items = []
    for i, csr in enumerate(mats):
        K = ks[i % len(ks)]
        m = device_metcf_from_csr(csr)
        B = torch_dev(np.random.default_rng(100 + i).uniform(-1, 1, (csr["cols"], K)).astype(np.float32))
        C = empty_dev(m.c_rows, K)
        items.append((m, B, C, K))
    return items


def plain_results(items, prec):
    out = []
    for m, B, _, K in items:
        C = empty_dev(m.c_rows, K)
        m.spmm(B, C, K, prec)
        out.append(C)
    torch.cuda.synchronize()
    return [c.cpu().numpy() for c in out]


@pytest.mark.parametrize("ks", [(64,), (128,), (64, 128), (32, 36, 200)])
@pytest.mark.parametrize("prec", [capi.PREC_TF32, capi.PREC_3XTF32])
def test_batch_matches_plain_launches_bitwise(ks, prec):
    items = build_items(ks)
    ref = plain_results(items, prec)
    b = api.Batch(items, prec)
    n, work, fs = b.info()
    assert n == len(items) and work > 0
    for rep in range(2):
        for _, _, C, _ in items:
            C.fill_(float("nan"))
        b.run()
        torch.cuda.synchronize()
        for (m, _, C, _), r in zip(items, ref):
            np.testing.assert_array_equal(C.cpu().numpy(), r)


def test_batch_graph_replay():
    items = build_items((64, 128))
    ref = plain_results(items, capi.PREC_TF32)
    b = api.Batch(items)
    s = torch.cuda.Stream()
    b.run(s)          # sets kernel attributes outside the capture
    s.synchronize()
    b.capture(s)
    for _ in range(3):
        for _, _, C, _ in items:
            C.fill_(float("nan"))
        torch.cuda.synchronize()
        b.launch_graph(s)
        s.synchronize()
        for (_, _, C, _), r in zip(items, ref):
            np.testing.assert_array_equal(C.cpu().numpy(), r)
    # new B contents are picked up by the replay
    m, B, C, K = items[0]
    B.mul_(2.0)
    b.launch_graph(s)
    s.synchronize()
    np.testing.assert_allclose(C.cpu().numpy(), 2.0 * ref[0], rtol=0, atol=0)


def test_batch_rejects_bad_items():
    items = build_items((64,))[:1]
    m, B, C, K = items[0]
    with pytest.raises(capi.AccSpmmError):
        api.Batch([(m, B, C, 30)])
    with pytest.raises(capi.AccSpmmError):
        api.Batch([(m, B.data_ptr() + 4, C, 64)])


def test_batch_with_packed_b_matches_plain_bitwise():
    """TF32 items whose B the plan packs (all with K > 32 under
    ACCSPMM_OPT_PACK = 1, small ones included; 128-column slices for K > 64,
    64-column ones for K = 40, 64) run in their own persistent launches over
    packed copies the plan owns, packed again on every run: the
    results equal one plain launch per matrix bit for bit, also from a graph
    replay after B has changed."""
    with capi.option(capi.OPT_PACK, 1):
        items = build_items((128, 200, 64, 40))
        ref = plain_results(items, capi.PREC_TF32)
        b = api.Batch(items)
        s = torch.cuda.Stream()
        b.run(s)
        s.synchronize()
        for (_, _, C, _), r in zip(items, ref):
            np.testing.assert_array_equal(C.cpu().numpy(), r)
        b.capture(s)
        for _, B, C, _ in items:
            B.mul_(2.0)
            C.fill_(float("nan"))
        torch.cuda.synchronize()
        b.launch_graph(s)
        s.synchronize()
        for (_, _, C, _), r in zip(items, ref):
            np.testing.assert_array_equal(C.cpu().numpy(), 2.0 * r)
