"""Kernel ridge regression (ml_type = 1, normalised polynomial kernel) on the GPU against the
oracle's restatement of compute_kernel.F90 / the kernel packing of mld_energy, mld_forces and
mld_stress, and the lambda^2 ridge of parameters.F90:1217-1395."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300))


def _dataset():
    from mld_gb300 import synth
    return synth.fe_bcc_batched(n_struct=4, nmin=16, nmax=120, seed=17)


def _refs(ds, j_max, nk, seed=3):
    d = oracle.bispectrum(ds.structures[-1].positions, ds.structures[-1].cell, ds.structures[-1].types, ds.rcut,
                          j_max, want_deriv=False)
    rng = np.random.default_rng(seed)
    idx = rng.choice(d["B"].shape[0], size=nk, replace=False)
    return d["B"][idx]


def _oracle(ds, j_max, Z, power, length, sigma):
    rows, ys = [], []
    for s in ds.structures:
        d = oracle.bispectrum(s.positions, s.cell, s.types, ds.rcut, j_max)
        e, f, st = oracle.kernel_rows(d, s.cell, Z, power=power, length=length, sigma=sigma)
        rows += [e[None, :], f, st]
        ys += [np.array([s.energies[1]]), s.forces.reshape(-1), s.stress]
    return np.concatenate(rows), np.concatenate(ys)


def _handle(j_max, lam, precision, power=2.0, length=np.sqrt(0.5), sigma=0.0):
    from mld_gb300 import _lib
    c = _lib.default_config()
    c.j_max, c.r_cut, c.lambda_krr, c.precision, c.ml_type = j_max, 4.7, lam, precision, 1
    c.kernel_power, c.length_kernel, c.sigma_kernel = power, length, sigma
    return _lib.Handle(c)


def _stage(h, ds, Zraw):
    nat, pos, cell, types = ds.arrays()
    h.set_structures(nat, pos, cell, types)
    E, F, S, has = ds.labels()
    h.set_labels(E, F, S, has, np.ones((len(nat), 3)))
    h.set_kernel_points(Zraw)


@pytest.mark.parametrize("precision,tol,power,sigma", [(0, 1e-10, 2.0, 0.0), (0, 1e-10, 3.0, 0.4),
                                                       (1, 2e-4, 2.0, 0.0)])
def test_kernel_rows(lib, precision, tol, power, sigma):
    ds = _dataset()
    Zraw = _refs(ds, 1.5, 9)
    Z, _, _ = oracle.kernel_points(Zraw)
    length = 0.9
    A_ref, _ = _oracle(ds, 1.5, Z, power, length, sigma)
    with _handle(1.5, 1e-6, precision, power, length, sigma) as h:
        _stage(h, ds, Zraw)
        assert h.dim_design_line == A_ref.shape[1]
        A, y, w = h.design_matrix()
    # compare per block: linear part and kernel part have different scales
    KK = Zraw.shape[1]
    assert _rel(A[:, :1 + KK], A_ref[:, :1 + KK]) < tol
    assert _rel(A[:, 1 + KK:], A_ref[:, 1 + KK:]) < tol


def test_kernel_fit_predictions(lib):
    ds = _dataset()
    Zraw = _refs(ds, 1.5, 9)
    Z, _, _ = oracle.kernel_points(Zraw)
    lam = 1e-3
    A_ref, y_ref = _oracle(ds, 1.5, Z, 2.0, np.sqrt(0.5), 0.0)
    w_or = oracle.fit_kernel(A_ref, y_ref, np.ones(len(y_ref)), lam)
    with _handle(1.5, lam, 0) as h:
        _stage(h, ds, Zraw)
        w, rmse = h.fit()
        Ep, Fp, Sp = h.predict(w)
    p, p_or = A_ref @ w, A_ref @ w_or
    assert _rel(p, p_or) < 1e-6
    rows_E = np.cumsum([0] + [1 + 3 * s.nat + 6 for s in ds.structures])[:-1]
    assert _rel(Ep, p[rows_E]) < 1e-9
    with _handle(1.5, lam, 1) as h32:
        _stage(h32, ds, Zraw)
        w32, r32 = h32.fit()
    assert abs(r32[1] - rmse[1]) <= 0.01 * rmse[1]


def test_kernel_points_validation(lib):
    from mld_gb300 import _lib
    ds = _dataset()
    Zraw = _refs(ds, 1.5, 5)
    Zraw[:, 2] = 1.0  # a component without spread
    with _handle(1.5, 1e-6, 0) as h:
        with pytest.raises(_lib.MldError) as ei:
            h.set_kernel_points(Zraw)
        assert ei.value.code == 1
        nat, pos, cell, types = ds.arrays()
        h.set_structures(nat, pos, cell, types)
        E, F, S, has = ds.labels()
        h.set_labels(E, F, S, has, np.ones((len(nat), 3)))
        with pytest.raises(_lib.MldError) as ei:
            h.design_matrix()  # no reference points yet
        assert ei.value.code == 6
