"""The `mma <matrix> <feature_dim>` command (src/mma_tf32.cu:185-243): argv,
exit codes and the result.csv line."""
import os
import subprocess

import pytest

from tests.helpers import GOLD

MMA = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                   "accspmm_gb300", "bin", "mma")


def run(args, cwd):
    return subprocess.run([MMA] + args, cwd=cwd, capture_output=True, text=True, timeout=300)


def test_usage_exit_code(tmp_path):
    r = run([], tmp_path)
    assert r.returncode == 4
    assert "Usage" in r.stdout
    r = run(["only_one_arg.mtx"], tmp_path)
    assert r.returncode == 4


def test_unreadable_matrix_exit_code(tmp_path):
    r = run([str(tmp_path / "missing.mtx"), "32"], tmp_path)
    assert r.returncode == 3
    r = run([os.path.join(GOLD, "inputs", "bad_banner.mtx"), "32"], tmp_path)
    assert r.returncode == 3
    assert not (tmp_path / "result.csv").exists()


@pytest.mark.gpu
@pytest.mark.parametrize("name,k", [("plsym1000", 64), ("longwin", 128), ("rand203", 32)])
def test_full_run_appends_result_line(tmp_path, name, k):
    path = os.path.join(GOLD, "inputs", name + ".mtx")
    for _ in range(2):
        r = run([path, str(k)], tmp_path)
        assert r.returncode == 0, r.stderr
    lines = (tmp_path / "result.csv").read_text().splitlines()
    assert len(lines) == 2
    fields = lines[0].split(",")
    assert fields[0] == name + ".mtx" and fields[1] == str(k)
    assert float(fields[2]) > 0 and float(fields[3]) > 0
    r = run([path, str(k), "--precision", "3xtf32", "--host-build"], tmp_path)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_metcf_cache_is_written_then_reused(tmp_path):
    import shutil

    import numpy as np

    from accspmm_gb300 import api
    from tests.helpers import gold
    mtx = str(tmp_path / "g.mtx")
    shutil.copy(os.path.join(GOLD, "inputs", "plsym1000.mtx"), mtx)
    r = run([mtx, "64", "--metcf-cache"], tmp_path)
    assert r.returncode == 0, r.stderr
    assert "m_tmp" in r.stdout and os.path.exists(mtx + ".metcf")
    back = api.load_metcf(mtx + ".metcf")
    np.testing.assert_array_equal(back["a2b"], gold("plsym1000")["m_a2b"])
    r = run([mtx, "64", "--metcf-cache"], tmp_path)
    assert r.returncode == 0, r.stderr
    assert "loaded" in r.stdout and "m_tmp" not in r.stdout
    a, b = (tmp_path / "result.csv").read_text().splitlines()
    assert a.split(",")[:2] == b.split(",")[:2]
