"""The ABI is plain C: a C99 program (tests/abi/consumer.c) that includes
only include/accspmm.h compiles with -pedantic -Werror, links
libaccspmm.so and runs the reference's host path on the 10 x 10 known-answer
matrix (entries (1,1)=1, (3,1)=2, (9,2)=3, (10,4)=4, (5,5)=5, (10,9)=6,
symmetric), reproducing its METCF: two windows, two tiles, sparseA2B
0 2 4 8 9 - - - | 1 3 8 9 - - - -, data 1 2 3 2 4 5 | 3 6 4 6, one AdpBME
group and the plain path."""
import os
import shutil
import subprocess

import pytest

from accspmm_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

KAT10 = """%%MatrixMarket matrix coordinate real symmetric
10 10 6
1 1 1
3 1 2
9 2 3
10 4 4
5 5 5
10 9 6
"""


@pytest.fixture(scope="module")
def consumer(tmp_path_factory):
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    if not os.path.exists(build.LIB):
        build.build()
    exe = str(tmp_path_factory.mktemp("abi") / "consumer")
    lib_dir = os.path.dirname(build.LIB)
    cmd = ["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", build.INCLUDE,
           os.path.join(ROOT, "tests", "abi", "consumer.c"), "-o", exe, "-L" + lib_dir, "-laccspmm",
           "-Wl,-rpath," + lib_dir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_c_program_reproduces_the_known_answer(consumer, tmp_path):
    mtx = tmp_path / "kat10.mtx"
    mtx.write_text(KAT10)
    r = subprocess.run([consumer, str(mtx)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.splitlines()
    # one AdpBME group (groupOffset 0 2) and the plain path, as the
    # reference's host code gives for this matrix (tests/golden/kat10.npz)
    assert lines[0] == "rows 10 cols 10 nnz 10 windows 2 tiles 2 groups 1 adaptive 0"
    assert lines[1] == "a2b 0 2 4 8 9 - - - 1 3 8 9 - - - -"
    assert lines[2] == "data 1 2 3 2 4 5 3 6 4 6"


def test_c_program_gets_the_reference_status_codes(consumer, tmp_path):
    r = subprocess.run([consumer, str(tmp_path / "missing.mtx")], capture_output=True, text=True,
                       timeout=60)
    assert r.returncode != 0 and "read" in r.stderr
    bad = tmp_path / "bad.mtx"
    bad.write_text("not a matrix market file\n")
    r = subprocess.run([consumer, str(bad)], capture_output=True, text=True, timeout=60)
    assert r.returncode != 0 and "read" in r.stderr
