"""The C-ABI library builds for sm_103a and exports every entry point declared in include/mld_gpu.h
(no GPU needed: only symbols are inspected)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "mld_gpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(mld_gpu_\w+)\s*\(", txt)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "mld_gpu_fit" in syms and "mld_gpu_create" in syms
    assert len(syms) >= 16


def test_library_exports_all_declared(lib):
    for s in declared_symbols():
        assert hasattr(lib, s), s


def test_python_binding_lists_all(lib):
    from mld_gb300 import _lib
    assert set(declared_symbols()) <= set(_lib.EXPORTED)


def test_fortran_module_binds_every_entry_point():
    """The ISO_C_BINDING module declares every C entry point, and its mld_gpu_config type has
    the C struct's fields in the same order (no Fortran compiler here: checked as text)."""
    from mld_gb300 import _lib
    src = open(os.path.join(ROOT, "mld_gb300", "fortran", "mld_gpu_mod.F90")).read()
    bound = set(re.findall(r'name="(mld_gpu_\w+)"', src))
    assert set(declared_symbols()) <= bound, sorted(set(declared_symbols()) - bound)
    body = re.search(r"type, bind\(C\), public :: mld_gpu_config(.*?)end type", src, flags=re.S).group(1)
    fields = re.findall(r"::\s*(\w+)", body)
    assert fields == [f[0] for f in _lib.MldGpuConfig._fields_]


def test_config_defaults_match_namelist():
    from mld_gb300 import _lib
    c = _lib.default_config()
    assert c.descriptor_type == 9 and c.j_max == 1.5 and c.r_cut == 5.0
    assert abs(c.inv_r0_input - (1 - 0.02 / 3.141592653589793)) < 1e-15
    assert c.lambda_krr == -1.0 and c.svd_rcond == -1.0 and c.imm_neigh == 300
    assert c.r_cut_width_in == 0.4 and c.sign_stress == 1.0 and c.sign_stress_big_box == 1.0
