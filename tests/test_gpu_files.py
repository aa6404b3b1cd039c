"""GPU-fitted potentials and GPU descriptors through the reference's file formats."""
import os

import numpy as np
import pytest

from mld_gb300 import potfile as pf

pytestmark = pytest.mark.gpu

FILES = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "files")


def _handle(precision=0, quadratic=False):
    from mld_gb300 import _lib
    c = _lib.default_config()
    c.j_max = 4.0 if not quadratic else 2.0
    c.r_cut = 4.7
    c.precision = precision
    c.lambda_krr = 1e-6
    if quadratic:
        c.mld_order = 2
    return _lib.Handle(c)


@pytest.mark.parametrize("precision,quadratic", [(0, False), (1, False), (0, True)])
def test_fitted_potential_round_trip(lib, tmp_path, precision, quadratic):
    from mld_gb300 import synth
    ds = synth.fe_bcc_batched(n_struct=6, nmin=16, nmax=200, seed=11)
    h = _handle(precision, quadratic)
    nat, pos, cell, types = ds.arrays()
    h.set_structures(nat, pos, cell, types)
    E, F, S, has = ds.labels()
    h.set_labels(E, F, S, has, np.ones((len(nat), 3)))
    w, _ = h.fit()
    order = pf.MLD_QUADRATIC if quadratic else pf.MLD_LINEAR
    p_mld, p_lmp = pf.write_potential(str(tmp_path), w, ["Fe"], j_max=h.cfg.j_max, r_cut=4.7, mld_order=order)
    w_mld = pf.read_milady_pot(p_mld)
    L = pf.read_lammps_pot(p_lmp)
    assert np.array_equal(w_mld, L["w"]) and w_mld.shape == w.shape
    assert np.abs(w_mld - w).max() <= 2e-16 * np.abs(w).max() * 8
    # the mixed method recomputes FP32 descriptors with atomics on every call: runs differ by ~1e-7
    tol = 1e-12 if precision == 0 else 1e-6
    e0, f0, s0 = h.predict(w)
    e1, f1, s1 = h.predict(w_mld)
    assert np.abs(e1 - e0).max() <= tol * np.abs(e0).max()
    assert np.abs(f1 - f0).max() <= tol * 10 * max(np.abs(f0).max(), 1e-300)
    h.close()


def test_gpu_descriptor_dump_matches_reference_eml(lib, tmp_path, fit17):
    i = list(fit17["names"]).index("02_111_000001")
    h = _handle(0)
    h.set_structures([fit17[f"pos_{i}"].shape[0]], fit17[f"pos_{i}"], fit17[f"cell_{i}"][None],
                     fit17[f"types_{i}"])
    B, _ = h.descriptors()
    out = str(tmp_path / "02_111_000001.eml")
    pf.write_eml(out, B)
    idx, got = pf.read_eml(out)
    _, ref = pf.read_eml(os.path.join(FILES, "fit17_02_111_000001.eml"))
    assert np.array_equal(idx, np.arange(1, B.shape[0] + 1))
    assert np.abs(got - ref).max() <= 1e-10 * np.abs(ref).max()
    h.close()
