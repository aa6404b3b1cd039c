"""Host-side mirror of the reference interface: db_model selection, namelist, POSCAR, synthetic data."""
import json
import os
import tempfile

import numpy as np
import pytest

from mld_gb300 import db_model, namelist, poscar, synth

HERE = os.path.dirname(os.path.abspath(__file__))


def test_park_miller_known_answers():
    # documented sequence of the minimal-standard generator for seed 12345
    r, s = db_model.r8_uniform_01(12345)
    assert s == 207482415 and abs(r - 0.096616) < 1e-6
    r, s = db_model.r8_uniform_01(s)
    assert s == 1790989824 and abs(r - 0.833995) < 1e-6
    r, s = db_model.r8_uniform_01(s)
    assert s == 2035175616 and abs(r - 0.947702) < 1e-6


def test_rks2_properties():
    a, _ = db_model.rks2(30, 28, 38)
    assert len(a) == 28 and a == sorted(a) and len(set(a)) == 28 and a[0] >= 1 and a[-1] <= 30
    assert db_model.rks2(10, 0, 5)[0] == []
    assert db_model.rks2(5, 5, 5)[0] == [1, 2, 3, 4, 5]


@pytest.mark.parametrize("name", ["fit01", "fit08", "fit13", "fit17"])
def test_selection_matches_reference_lists(name):
    fx = json.load(open(os.path.join(HERE, "golden", "db_selection.json")))[name]
    with tempfile.NamedTemporaryFile("w", suffix=".in", delete=False) as fh:
        fh.write(fx["db_model"])
    lines = db_model.read_db_model(fh.name, fx["selection_type"])
    cf = db_model.select(lines, fx["selection_type"], fx["seed"], db_path="")
    os.unlink(fh.name)
    assert [c.filename for c in cf if c.train] == fx["train"]
    if name != "fit17":  # fit17's REF/test_files.milady is not produced by its own db_model.in
        assert [c.filename for c in cf if not c.train] == fx["test"]


def test_namelist_defaults_and_parse(tmp_path):
    p = tmp_path / "x.ml"
    p.write_text("&input_ml\n ml_type=-1 ! desc\n r_cut=4.7d0\n j_max=4.0\n weighted=.true.\n"
                 " chemical_elements=\" Ta Ti V W \"\n snap_order=1\n lambda_krr=1.d-8\n&end\n")
    nl = namelist.read_input_ml(str(p))
    assert nl["ml_type"] == -1 and nl["r_cut"] == 4.7 and nl["j_max"] == 4.0 and nl["weighted"] is True
    assert namelist.elements(nl) == ["Ta", "Ti", "V", "W"] and nl["mld_order"] == 1
    assert nl["lambda_krr"] == 1e-8 and nl["seed"] == 14792435 and nl["selection_type"] == 3
    assert abs(nl["inv_r0_input"] - (1 - 0.02 / np.pi)) < 1e-15


def test_poscar_roundtrip(tmp_path):
    ds = synth.fe_bcc_fixed(n_struct=1)
    s = ds.structures[0]
    p = tmp_path / "a.poscar"
    poscar.write_poscar(str(p), s, masses=[56])
    t = poscar.read_poscar(str(p))
    assert np.allclose(t.positions, s.positions) and np.allclose(t.cell, s.cell)
    assert np.allclose(t.forces, s.forces) and np.allclose(t.stress, s.stress)
    assert t.elements == ["Fe"] and t.has_energy and t.has_force and t.has_stress


def test_synthetic_forces_are_gradients():
    ds = synth.fe_bcc_fixed(n_struct=1)
    s = ds.structures[0]
    _, F, _ = synth.morse_labels(s.positions, s.cell, s.types, 4.7)
    h = 1e-6
    for c in range(3):
        p1 = s.positions.copy(); p1[3, c] += h
        p2 = s.positions.copy(); p2[3, c] -= h
        fd = -(synth.morse_labels(p1, s.cell, s.types, 4.7)[0] - synth.morse_labels(p2, s.cell, s.types, 4.7)[0]) / (2 * h)
        assert abs(fd - F[3, c]) < 1e-5 * max(1.0, abs(F[3, c]))


def test_batched_set_is_deterministic():
    a = synth.fe_bcc_batched(n_struct=5, seed=3)
    b = synth.fe_bcc_batched(n_struct=5, seed=3)
    assert all(np.array_equal(x.positions, y.positions) for x, y in zip(a.structures, b.structures))
    assert all(16 <= x.nat <= 1024 for x in a.structures)


def test_kernel_reference_selection_is_seeded_and_prefers_leverage():
    from mld_gb300 import kernel_select
    rng = np.random.default_rng(0)
    B = rng.normal(size=(2000, 6))
    B[:10] *= 50.0  # ten high-leverage atoms
    a = kernel_select.select(B, 100, seed=7)
    b = kernel_select.select(B, 100, seed=7)
    assert np.array_equal(a, b) and len(a) == 100 and len(set(a.tolist())) == 100
    lev, k = kernel_select.leverage_scores(B)
    assert k == 6 and abs(lev.sum() - 1.0) < 1e-9
    assert len(set(range(10)) & set(a.tolist())) >= 9


def _cur_cases():
    rng = np.random.default_rng(1)
    L = rng.normal(size=(12, 12)) * np.logspace(0, -3, 12)[None, :]
    synth_B = rng.normal(size=(300, 12)) @ L.T + 3.0
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "fit17_bso4.npz"))
    fit17_B = np.concatenate([z[k] for k in sorted(z.files) if k.startswith("B_")])
    return [(synth_B, 6, 4), (synth_B, 10, -1), (synth_B, 40, 3), (synth_B, 200, -1), (fit17_B, 20, -1),
            (fit17_B, 60, -1)]


@pytest.mark.parametrize("case", range(6))
def test_cur_selection_matches_oracle(case):
    """The CUR selection of kernel reference atoms (QR-coordinate products) against the oracle's
    explicit restatement with full matrices and pseudo-inverses, on the same uniform draws:
    leverage scores, k and r, every trial's score, the winner and its atoms.  The fit17 cases use
    MILADY's golden descriptors of 20 W structures (1301 atoms, K = 55)."""
    import oracle
    from mld_gb300 import kernel_select
    B, c, r = _cur_cases()[case]
    seed = 5 + case
    res = kernel_select.cur_select(B, c, seed=seed, r=r)
    g = np.random.default_rng(seed)
    ucol = g.random((kernel_select.CUR_TRIALS, B.shape[0]))
    urow = g.random((kernel_select.CUR_TRIALS, B.shape[1]))
    sels, pcol, prow, k, rr, scores, _ = oracle.cur_decomposition(B, c, ucol, urow, r=r)
    assert (res.k, res.r) == (k, rr)
    assert np.abs(res.pcol - pcol).max() <= 1e-10 * pcol.max()
    assert np.abs(res.prow - prow).max() <= 1e-12
    assert np.array_equal(res.n_col, [len(s) for s in sels])
    A = B - B.mean(axis=0)
    norm_a = np.sqrt((A * A).sum())
    assert np.abs(res.scores - scores).max() <= 1e-10 * norm_a
    # the oracle's scores with the same tie rule (rounding-level scores are equal)
    win = int(np.flatnonzero(scores <= scores.min() + kernel_select.TIE_REL * norm_a)[0])
    assert res.winner == win and np.array_equal(res.selected, sels[win])


def test_cur_kernel_points_carry_k_and_r():
    from mld_gb300 import kernel_select
    B = _cur_cases()[4][0]
    first, second = kernel_select.cur_kernel_points(B[:600], B, 50, 80, seed=3)
    assert (first.k, first.r) == (second.k, second.r) == (55, int(55 * np.log(55)))
    assert abs(len(first.selected) - 50) < 25 and abs(len(second.selected) - 80) < 30
    assert first.selected.max() < 600
