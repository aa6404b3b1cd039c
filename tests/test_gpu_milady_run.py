"""The ``milady_run`` host mirror end to end on a small POSCAR database: descriptor dump
(ml_type -1), linear and quadratic fits (ml_type 0) and kernel ridge (ml_type 1), each writing the
reference's files (.eml, .pot, train_*.out, kernel_matrix.dat)."""
import os

import numpy as np
import pytest

import oracle
from mld_gb300 import _lib, poscar, potfile, synth

pytestmark = pytest.mark.gpu

NL = """&input_ml
ml_type={ml_type}
mld_order={order}
descriptor_type=9
j_max={j_max}
r_cut=4.7d0
desc_forces=.true.
chemical_elements="Fe"
lambda_krr=1.d-6
np_kernel_ref=24
np_kernel_full=0
db_path="DB/"
&end
"""


@pytest.fixture()
def database(tmp_path):
    ds = synth.fe_bcc_fixed(n_struct=8, reps=2, seed=7)
    db = tmp_path / "DB"
    db.mkdir()
    for k, s in enumerate(ds.structures):
        poscar.write_poscar(str(db / f"01_111_{k + 1:06d}.poscar"), s)
    (tmp_path / "db_model.in").write_text("01   111    8   6   T T T   1.e0 1.e0 1.e0 1.e0 1.e0 1.e0\n")
    return tmp_path, ds


def _run(tmp_path, ml_type, order=1, j_max=4.0, precision=_lib.PLAIN_FP64):
    from mld_gb300.milady_run import milady_run
    inp = tmp_path / f"in_{ml_type}_{order}.ml"
    inp.write_text(NL.format(ml_type=ml_type, order=order, j_max=j_max))
    return milady_run(str(inp), str(tmp_path / "db_model.in"), str(tmp_path / "DB"), str(tmp_path),
                      precision=precision)


def test_descriptor_dump(lib, database):
    tmp_path, ds = database
    r = _run(tmp_path, -1)
    assert len(r.files) == 8
    for k, s in enumerate(ds.structures):
        idx, B = potfile.read_eml(str(tmp_path / "descDB" / f"01_111_{k + 1:06d}.eml"))
        d = oracle.bispectrum(s.positions, s.cell, s.types, 4.7, 4.0, want_deriv=False)
        assert np.array_equal(idx, np.arange(1, s.nat + 1))
        assert np.abs(B - d["B"]).max() <= 1e-10 * np.abs(d["B"]).max()


@pytest.mark.parametrize("order,j_max,tag", [(1, 4.0, "snap1"), (2, 2.0, "qnml1")])
def test_fit_writes_parameter_files(lib, database, order, j_max, tag):
    tmp_path, _ = database
    r = _run(tmp_path, 0, order, j_max)
    assert r.n_train == 6 and r.n_test == 2
    assert os.path.basename(r.files["pot"]) == f"bso4_{tag}_params.pot"
    w = potfile.read_milady_pot(r.files["pot"])
    L = potfile.read_lammps_pot(r.files["lammps_pot"])
    assert np.array_equal(w, L["w"]) and w.shape == r.w.shape
    assert L["mld_order"] == order and L["elements"] == ["Fe"] and L["j_max"] == j_max
    assert np.abs(w - r.w).max() <= 1e-15 * np.abs(r.w).max()
    rows = open(r.files["train_energy"]).read().splitlines()
    assert len(rows) == 6
    assert np.all(np.isfinite(r.rmse_train)) and np.all(np.isfinite(r.rmse_test))


def test_kernel_fit_selects_and_reuses_points(lib, database):
    tmp_path, _ = database
    r1 = _run(tmp_path, 1)
    assert "kernel_matrix" in r1.files
    Z = potfile.read_kernel_matrix(r1.files["kernel_matrix"])
    # the CUR selection keeps atom j with probability min(1, 24 p_j): about 24 of the 128 atoms of
    # class 01, none from np_kernel_full = 0
    nk = Z.shape[0]
    assert 10 <= nk <= 40 and Z.shape[1] == 55
    L = potfile.read_lammps_pot(r1.files["lammps_pot"])
    assert L["mld_order"] == potfile.MLD_KERNEL and L["kernel_points"].shape == (nk, 55)
    assert L["w"].shape == (1 + 55 + nk,)
    # a second run reads kernel_matrix.dat instead of selecting again: the same model, bitwise
    # (every sum of the FP64 path has a fixed order)
    r2 = _run(tmp_path, 1)
    assert "kernel_matrix" not in r2.files
    assert np.array_equal(r2.w, r1.w)
    assert np.array_equal(r2.rmse_train, r1.rmse_train)
