"""Host-built bispectrum tables (mld_gb300/csrc/bso4_tables.cpp): the invariants the descriptor
kernel relies on, checked by tests/tables_check.cc compiled with the host compiler (no GPU).

Covered: every Z term in exactly one round lane; rounds of one inner extent, outer extents
descending, padding lanes empty and last; the terms' c and CG indices in range; slot scales
inside the kernel's 16 x 16 table and slot positions unique; contraction rows whole tiles per
layer with unique destinations and a rank-0 row per triple; recursion references inside the
previous half layer and non-negative coefficients."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _cuda_include():
    for d in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if d and os.path.exists(os.path.join(d, "include", "cuda_runtime.h")):
            return os.path.join(d, "include")
    nv = shutil.which("nvcc")
    if nv:
        d = os.path.join(os.path.dirname(os.path.dirname(nv)), "include")
        if os.path.exists(os.path.join(d, "cuda_runtime.h")):
            return d
    return None


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    inc = _cuda_include()
    if not cxx or not inc:
        pytest.skip("needs a host C++ compiler and the CUDA headers")
    exe = str(tmp_path_factory.mktemp("tables") / "tables_check")
    cmd = [cxx, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), "-I", inc,
           os.path.join(ROOT, "tests", "tables_check.cc"), os.path.join(ROOT, "mld_gb300", "csrc", "bso4_tables.cpp"),
           "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


@pytest.mark.parametrize("j_max", [0.5, 1.0, 1.5, 2.0, 2.5, 3.0, 3.5, 4.0, 4.5, 5.0])
def test_table_invariants(checker, j_max):
    r = subprocess.run([checker, str(j_max)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout + r.stderr


def test_jmax4_schedule_sizes(checker):
    """The j_max = 4 schedule: 77 rounds of 32 Z terms, 140 contraction rows."""
    r = subprocess.run([checker, "4.0"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    assert "K=55 rounds=77 rows=140" in r.stdout, r.stdout
