"""Launch options (accspmm_set_option / accspmm_get_option): host logic only,
no GPU.  Each option starts from its environment variable, read once; the
product library refuses the measurement kernels, the measurement build
(libaccspmm_lab.so) accepts them."""
import json
import os
import subprocess
import sys

import pytest

from accspmm_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

DEFAULTS = {capi.OPT_PACK: -1, capi.OPT_PREFETCH: -1, capi.OPT_SCHEDULE: 1, capi.OPT_SLICE_WIDTH: 0,
            capi.OPT_CTAS_PER_SM: 0, capi.OPT_TILE_RING: -1, capi.OPT_WINDOWS_PER_CTA: 0,
            capi.OPT_HOST_SLICE_WIDTH: 0, capi.OPT_HOST_DIRECT_C: 1, capi.OPT_KERNEL: 0}


def run_fresh(env: dict, lab: bool = False) -> dict:
    """Option values seen by a fresh process with `env` added."""
    code = ("import json, sys; sys.path.insert(0, %r)\n"
            "from accspmm_gb300 import capi\n"
            "lib = capi.load_lab() if %r else capi.load()\n"
            "print(json.dumps({o: capi.get_option(o, lib) for o in range(10)}))") % (ROOT, lab)
    e = {k: v for k, v in os.environ.items() if not k.startswith("ACCSPMM_")}
    e.update(env)
    r = subprocess.run([sys.executable, "-c", code], env=e, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    return {int(k): v for k, v in json.loads(r.stdout.strip().splitlines()[-1]).items()}


def test_defaults_without_environment():
    assert run_fresh({}) == DEFAULTS


def test_environment_is_read_once_at_first_use():
    got = run_fresh({"ACCSPMM_PACK": "0", "ACCSPMM_FS": "64", "ACCSPMM_PREFETCH": "0", "ACCSPMM_WB": "8",
                     "ACCSPMM_HOST_DIRECT": "0"})
    assert got[capi.OPT_PACK] == 0 and got[capi.OPT_SLICE_WIDTH] == 64
    assert got[capi.OPT_PREFETCH] == 0 and got[capi.OPT_WINDOWS_PER_CTA] == 8
    assert got[capi.OPT_HOST_DIRECT_C] == 0
    assert run_fresh({"ACCSPMM_PACK": "2"})[capi.OPT_PACK] == 1
    # values outside the listed ones keep the default
    bad = run_fresh({"ACCSPMM_FS": "48", "ACCSPMM_OCC": "5", "ACCSPMM_KERNEL": "pipe"})
    assert bad[capi.OPT_SLICE_WIDTH] == 0 and bad[capi.OPT_CTAS_PER_SM] == 0
    assert bad[capi.OPT_KERNEL] == 0  # the product library has no measurement kernels


def test_set_get_round_trip_and_refusals():
    lib = capi.load()
    old = capi.get_option(capi.OPT_SLICE_WIDTH)
    try:
        capi.set_option(capi.OPT_SLICE_WIDTH, 32)
        assert capi.get_option(capi.OPT_SLICE_WIDTH) == 32
        for opt, val in ((capi.OPT_SLICE_WIDTH, 48), (capi.OPT_PACK, 2), (capi.OPT_TILE_RING, 3),
                         (capi.OPT_WINDOWS_PER_CTA, 2000), (capi.OPT_PREFETCH, 2), (42, 0), (-1, 0)):
            assert lib.accspmm_set_option(opt, val) == capi.ERROR_INVALID_VALUE
        assert capi.get_option(capi.OPT_SLICE_WIDTH) == 32
        for k in ("pipe", "bulk", "lean", "db", "tma", "staged"):
            assert lib.accspmm_set_option(capi.OPT_KERNEL, capi.KERNELS[k]) == capi.ERROR_UNSUPPORTED
            assert "libaccspmm_lab.so" in lib.accspmm_last_error().decode()
        assert lib.accspmm_set_option(capi.OPT_KERNEL, 7) == capi.ERROR_INVALID_VALUE
        assert lib.accspmm_get_option(capi.OPT_PACK, None) == capi.ERROR_INVALID_VALUE
    finally:
        capi.set_option(capi.OPT_SLICE_WIDTH, old)
    with capi.option(capi.OPT_PACK, 0):
        assert capi.get_option(capi.OPT_PACK) == 0
    assert capi.get_option(capi.OPT_PACK) == DEFAULTS[capi.OPT_PACK]


def test_measurement_build_accepts_the_variants():
    if not os.path.exists(capi.LAB_PATH):
        pytest.skip("libaccspmm_lab.so not built")
    lab = capi.load_lab()
    assert run_fresh({"ACCSPMM_KERNEL": "staged"}, lab=True)[capi.OPT_KERNEL] == capi.KERNELS["staged"]
    for k, v in capi.KERNELS.items():
        with capi.option(capi.OPT_KERNEL, v, lib=lab):
            assert capi.get_option(capi.OPT_KERNEL, lab) == v
    # the two libraries keep separate options
    assert capi.get_option(capi.OPT_KERNEL) == 0
