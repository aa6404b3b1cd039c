"""Shared-memory plan of the descriptor kernel (mld_gb300/csrc/bispectrum.cu), checked on the host
by tests/plan_check.cu (compiled with nvcc; no GPU).

At j_max = 4 the FP32 kernel is register-limited to two CTAs per SM, and a plan that fits only
one costs about a third of its speed.  So the plan must fit two: with one channel, with Y in
shared memory and geometry records for the Fe benchmark's neighbour counts; with two or three
weighted channels, with Y in global slices.  The FP64 kernel must fit one."""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def plans(tmp_path_factory):
    from mld_gb300 import build as B
    try:
        nvcc = B.nvcc()
    except RuntimeError:
        pytest.skip("needs nvcc")
    if not shutil.which("g++") and not shutil.which("c++"):
        pytest.skip("needs a host C++ compiler")
    exe = str(tmp_path_factory.mktemp("plan") / "plan_check")
    cmd = [nvcc, *B.ARCH, "-std=c++17", "-O1", "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "plan_check.cu"), os.path.join(ROOT, "mld_gb300", "csrc", "bso4_tables.cpp"),
           "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([exe, "4.0"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    out = {}
    for line in r.stdout.splitlines():
        m = re.match(r"eb=(\d) nch=(\d) y=(\w+) g1=(\d+) geo_cap=(\d+) bytes=(\d+) ctas=(\d+)", line)
        assert m, line
        eb, nch, y, g1, cap, nbytes, ctas = m.groups()
        out[(int(eb), int(nch))] = dict(y=y, g1=int(g1), geo_cap=int(cap), bytes=int(nbytes), ctas=int(ctas))
    return out


def test_fp32_one_channel_two_ctas_shared_y(plans):
    p = plans[(4, 1)]
    assert p["ctas"] == 2 and p["y"] == "shared", p
    assert p["g1"] == 6, p            # 40 neighbours per phase-1 pass
    assert p["geo_cap"] >= 48, p      # the Fe set's atoms keep every neighbour's record


@pytest.mark.parametrize("nch", [2, 3])
def test_fp32_weighted_channels_two_ctas(plans, nch):
    p = plans[(4, nch)]
    assert p["ctas"] == 2 and p["y"] == "global", p


@pytest.mark.parametrize("nch", [1, 2, 3])
def test_fp64_fits(plans, nch):
    assert plans[(8, nch)]["ctas"] >= 1, plans[(8, nch)]
