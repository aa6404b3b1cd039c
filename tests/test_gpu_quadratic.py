"""Quadratic model (mld_order = 2, QNML two-stage fit) on the GPU against the oracle.

The GPU keeps the symmetric quadratic block once (upper triangle, sqrt(2) off the diagonal);
rows are exported in the reference's full K*K layout and compared with the oracle's
restatement of mld_energy/forces/stress.  Fits compare predictions: min-norm and ridge
solutions of the full and the deduplicated layouts give identical predictions.
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300))


def _dataset():
    from mld_gb300 import synth
    return synth.fe_bcc_batched(n_struct=5, nmin=16, nmax=200, seed=9)


def _handle(j_max, lam, precision=0, weights=None):
    from mld_gb300 import _lib
    c = _lib.default_config()
    c.j_max, c.r_cut, c.lambda_krr, c.precision, c.mld_order = j_max, 4.7, lam, precision, 2
    if weights is not None:
        c.weighted = 1
        c.n_elements = len(weights)
        for i, w in enumerate(weights):
            c.weight_per_element[i] = w
    return _lib.Handle(c)


def _oracle(ds, j_max, chw=None):
    rows, ys = [], []
    for s in ds.structures:
        d = oracle.bispectrum(s.positions, s.cell, s.types, ds.rcut, j_max, channel_weights=chw)
        e, f, st = oracle.quadratic_rows(d, s.cell)
        rows += [e[None, :], f, st]
        ys += [np.array([s.energies[1]]), s.forces.reshape(-1), s.stress]
    return np.concatenate(rows), np.concatenate(ys)


@pytest.mark.parametrize("precision,tol", [(0, 1e-10), (1, 2e-5)])
def test_quadratic_rows(lib, precision, tol):
    ds = _dataset()
    A_ref, y_ref = _oracle(ds, 1.5)
    h = _handle(1.5, 1e-8, precision)
    nat, pos, cell, types = ds.arrays()
    h.set_structures(nat, pos, cell, types)
    E, F, S, has = ds.labels()
    h.set_labels(E, F, S, has, np.ones((len(nat), 3)))
    A, y, w = h.design_matrix()
    assert A.shape == A_ref.shape
    assert _rel(A, A_ref) < tol
    h.close()


def test_quadratic_rows_weighted(lib):
    from mld_gb300 import synth
    ds = _dataset()
    # two element types alternate; per-element weights of the second channel
    for s in ds.structures:
        s.types = (np.arange(s.nat) % 2).astype(np.int32)
    chw = np.array([[1.0, 1.0], [0.7, 1.3]])
    A_ref, _ = _oracle(ds, 1.0, chw)
    h = _handle(1.0, 1e-8, 0, weights=[0.7, 1.3])
    nat, pos, cell, types = ds.arrays()
    h.set_structures(nat, pos, cell, types)
    E, F, S, has = ds.labels()
    h.set_labels(E, F, S, has, np.ones((len(nat), 3)))
    A, _, _ = h.design_matrix()
    assert _rel(A, A_ref) < 1e-10
    h.close()


def test_qnml_fit_predictions(lib):
    ds = _dataset()
    A_ref, y_ref = _oracle(ds, 1.5)
    KK = 8
    lam = 1e-6
    h = _handle(1.5, lam)
    nat, pos, cell, types = ds.arrays()
    h.set_structures(nat, pos, cell, types)
    E, F, S, has = ds.labels()
    h.set_labels(E, F, S, has, np.ones((len(nat), 3)))
    w, rmse = h.fit()
    assert w.shape[0] == 1 + KK + KK * KK
    w_or = oracle.fit_qnml(A_ref, y_ref, np.ones(len(y_ref)), lam, 1 + KK)
    p, p_or = A_ref @ w, A_ref @ w_or
    assert _rel(p, p_or) < 1e-10
    # predictions through the serving entry point use the same full-layout weights
    Ep, Fp, Sp = h.predict(w)
    rows_E = np.cumsum([0] + [1 + 3 * s.nat + 6 for s in ds.structures])[:-1]
    assert _rel(Ep, p[rows_E]) < 1e-10
    h.close()


def test_large_dense_solve_cholesky(lib):
    """D above the Jacobi limit goes through the blocked Cholesky with refinement."""
    from mld_gb300 import _lib
    rng = np.random.default_rng(1)
    D = 300
    X = rng.normal(size=(2000, D))
    G = X.T @ X
    h_ = rng.normal(size=D)
    c = _lib.default_config()
    c.lambda_krr = 1e-3
    with _lib.Handle(c) as h:
        w, _ = h.solve(G, h_)
    w_ref = np.linalg.solve(G + 1e-3 * np.eye(D), h_)
    assert _rel(w, w_ref) < 1e-10


def test_weighted_descriptors_fp64_two_and_three_channels(lib):
    """Two- and three-channel FP64 descriptors at j_max = 4 keep their Z blocks in global scratch
    (they exceed shared memory); the descriptors must still match the oracle."""
    from mld_gb300 import _lib, synth
    ds = synth.hea_bcc_batched(n_struct=2, reps=3, seed=5)
    s = ds.structures[0]
    for three in (0, 1):
        chw = np.array([list(synth.HEA_WEIGHTS)] * (2 + three))
        chw[0] = 1.0
        if three:
            chw[2] = np.array(synth.HEA_WEIGHTS) ** 2
        c = _lib.default_config()
        c.j_max, c.r_cut, c.weighted, c.weighted_3ch = 4.0, 5.0, 1, three
        c.n_elements = 5
        for i, wv in enumerate(synth.HEA_WEIGHTS):
            c.weight_per_element[i] = wv
            c.weight_per_element_3ch[i] = wv ** 2
        with _lib.Handle(c) as h:
            h.set_structures(np.array([s.nat], np.int32), s.positions, s.cell[None], s.types)
            B, _ = h.descriptors()
        ref = oracle.bispectrum(s.positions, s.cell, s.types, 5.0, 4.0, channel_weights=chw, want_deriv=False)
        assert _rel(B, ref["B"]) < 1e-10
