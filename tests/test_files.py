"""Parameter (.pot) and descriptor (.eml) files: byte-identical round trips of MILADY's own files.

The fixtures under tests/golden/files/ are files the reference's regression fits wrote (made by
tests/golden/make_file_fixtures.py); each is read and written back with mld_gb300.potfile.
"""
import os

import numpy as np
import pytest

from mld_gb300 import potfile as pf

FILES = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "files")


def _bytes(p):
    with open(p, "rb") as f:
        return f.read()


@pytest.mark.parametrize("fit,name", [("fit03", "bso4_qnml1_params.pot"), ("fit08", "bso4_snap1_params.pot"),
                                      ("fit13", "bso4_snap1_params.pot")])
def test_pot_round_trip(tmp_path, fit, name):
    src = os.path.join(FILES, f"{fit}_{name}")
    w = pf.read_milady_pot(src)
    out = tmp_path / name
    pf.write_milady_pot(str(out), w)
    assert _bytes(out) == _bytes(src)

    src_l = os.path.join(FILES, f"{fit}_lammps_{name}")
    L = pf.read_lammps_pot(src_l)
    assert np.array_equal(L["w"], w)
    assert L["descriptor_type"] == 9 and L["ndetails"] == 4
    out_l = tmp_path / ("lammps_" + name)
    pf.write_lammps_pot(str(out_l), L["w"], L["elements"], j_max=L["j_max"], r_cut=L["r_cut"],
                        mld_order=L["mld_order"], nchannels=L["nchannels"], weights=L["weights"],
                        weights_3ch=L["weights_3ch"], ref_energy=L["ref_energy"])
    assert _bytes(out_l) == _bytes(src_l)  # masses from the element table, as the reference writes them


def test_pot_header_fields():
    L = pf.read_lammps_pot(os.path.join(FILES, "fit08_lammps_bso4_snap1_params.pot"))
    assert L["nchannels"] == 3 and L["elements"] == ["Ta", "Ti", "V", "W"]
    assert L["j_max"] == 4.0 and L["r_cut"] == 5.0 and L["mld_order"] == 1
    assert L["w"].shape == (166,)  # 1 + 3 channels x 55
    L = pf.read_lammps_pot(os.path.join(FILES, "fit03_lammps_bso4_qnml1_params.pot"))
    assert L["mld_order"] == 2 and L["w"].shape == (211,)  # 1 + 14 + 14^2 (j_max = 2)


@pytest.mark.parametrize("name", ["12_111_000005.eml", "02_111_000001.eml"])
def test_eml_round_trip(tmp_path, name, fit17):
    src = os.path.join(FILES, "fit17_" + name)
    idx, B = pf.read_eml(src)
    assert np.array_equal(idx, np.arange(1, B.shape[0] + 1))
    out = tmp_path / name
    pf.write_eml(str(out), B)
    assert _bytes(out) == _bytes(src)
    # the dump holds the same descriptors as the packed fit17 fixture
    i = list(fit17["names"]).index(name[:-4])
    assert np.array_equal(B, fit17[f"B_{i}"])


def test_eml_append(tmp_path):
    B = np.random.default_rng(1).standard_normal((5, 7))
    p = str(tmp_path / "x.eml")
    pf.write_eml(p, B[:2])
    pf.write_eml(p, B[2:], first_atom=3, append=True)
    idx, got = pf.read_eml(p)
    assert np.array_equal(idx, np.arange(1, 6))
    assert np.abs(got - B).max() <= 1e-17 * np.abs(B).max() * 10


def test_kernel_pot_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    Z = rng.standard_normal((7, 55))
    w = rng.standard_normal(1 + 55 + 7)
    p_mld, p_lmp = pf.write_potential(str(tmp_path), w, ["Fe"], j_max=4.0, r_cut=5.0, mld_order=pf.MLD_KERNEL,
                                      kernel_points=Z, sigma_kernel=0.0, length_kernel=np.sqrt(0.5),
                                      kernel_power=2.0)
    assert os.path.basename(p_mld) == "bso4_kernl_params.pot"
    assert os.path.basename(p_lmp) == "lammps_bso4_kernl_params.pot"
    L = pf.read_lammps_pot(p_lmp)
    assert L["ndetails"] == 7 and L["kernel_type"] == 4
    assert L["kernel_points"].shape == (7, 55)
    # ES25.15 keeps 16 significant digits
    assert np.abs(L["w"] - w).max() <= 1e-15 * np.abs(w).max()
    assert np.abs(L["kernel_points"] - Z).max() <= 1e-15 * np.abs(Z).max()
    assert (L["sigma_kernel"], L["kernel_power"]) == (0.0, 2.0)
    assert abs(L["length_kernel"] - np.sqrt(0.5)) < 1e-15
    assert np.array_equal(pf.read_milady_pot(p_mld), L["w"])


def test_fortran_edit_descriptors():
    assert pf._es(0.0, 25, 15) == "   0.000000000000000E+000"
    assert pf._es(-9.9999999999999999e-101, 25, 15) == "  -1.000000000000000E-100"
    assert pf._es(1.0, 30, 18) == "     1.000000000000000000E+000"
    assert pf._e(1.0, 20, 10) == "    0.1000000000E+01"
    assert pf._e(-0.00123, 20, 10) == "   -0.1230000000E-02"
    assert pf._e(0.0, 20, 10) == "    0.0000000000E+00"
