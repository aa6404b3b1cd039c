"""Parity of the CUDA path (through the C ABI) against the oracle and MILADY's golden vectors.

Tolerances: plain FP64 method <= 1e-10 relative to the largest magnitude of each compared array
(the reference's own bar for the FP64 path); mixed method (FP32 descriptors) <= 2e-5.
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

TOL64 = 1e-10
TOL32 = 2e-5


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _handle(j_max=4.0, r_cut=4.7, precision=0, lam=-1.0, n_el=1, weights=None):
    from mld_gb300 import _lib
    c = _lib.default_config()
    c.j_max = j_max
    c.r_cut = r_cut
    c.n_elements = n_el
    c.lambda_krr = lam
    c.precision = precision
    c.desc_forces = 1
    if weights is not None:
        c.weighted = 1
        for i, w in enumerate(weights):
            c.weight_per_element[i] = w
    return _lib.Handle(c)


def _fit17_batch(fit17, idx=None):
    idx = range(len(fit17["names"])) if idx is None else idx
    nat = [fit17[f"pos_{i}"].shape[0] for i in idx]
    pos = np.concatenate([fit17[f"pos_{i}"] for i in idx])
    cell = np.stack([fit17[f"cell_{i}"] for i in idx])
    types = np.concatenate([fit17[f"types_{i}"] for i in idx])
    return nat, pos, cell, types


@pytest.mark.parametrize("precision,tol", [(0, TOL64), (1, TOL32)])
def test_fit17_descriptors(lib, fit17, precision, tol):
    nat, pos, cell, types = _fit17_batch(fit17)
    h = _handle(precision=precision)
    h.set_structures(nat, pos, cell, types)
    B, nn = h.descriptors()
    ref = np.concatenate([fit17[f"B_{i}"] for i in range(len(nat))])
    assert B.shape == ref.shape
    assert _rel(B, ref) < tol
    h.close()


@pytest.mark.parametrize("precision,tol", [(0, TOL64), (1, TOL32)])
def test_fit19_three_channel_descriptors(lib, fit19, precision, tol):
    """Weighted 3-channel descriptors (weighted_auto channel weights) against fit19's golden B."""
    from mld_gb300 import _lib, elements
    els = [str(e) for e in fit19["elements"]]
    w2, w3 = elements.auto_channel_weights(els)
    c = _lib.default_config()
    c.j_max, c.r_cut, c.precision, c.n_elements = 4.0, 4.7, precision, len(els)
    c.weighted, c.weighted_3ch = 1, 1
    for i in range(len(els)):
        c.weight_per_element[i] = w2[i]
        c.weight_per_element_3ch[i] = w3[i]
    idx = range(len(fit19["names"]))
    nat = [fit19[f"pos_{i}"].shape[0] for i in idx]
    with _lib.Handle(c) as h:
        h.set_structures(nat, np.concatenate([fit19[f"pos_{i}"] for i in idx]),
                         np.stack([fit19[f"cell_{i}"] for i in idx]),
                         np.concatenate([fit19[f"types_{i}"] for i in idx]))
        B, _ = h.descriptors()
    ref = np.concatenate([fit19[f"B_{i}"] for i in idx])
    assert B.shape == ref.shape == (sum(nat), 165)
    assert _rel(B, ref) < tol


@pytest.mark.parametrize("fit", ["fit03", "fit08"])
@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("evaluate", [False, True])
def test_reference_run_predictions(lib, predictions, fit, precision, evaluate):
    """mld_gpu_predict (design rows x weights) and mld_gpu_evaluate (no rows) with a reference
    run's .pot weights reproduce that run's train_*.out."""
    from mld_gb300 import _lib
    from conftest import channel_weights_for
    d = predictions
    j_max, r_cut, order = d[f"{fit}_params"]
    els = [str(e) for e in d[f"{fit}_elements"]]
    c = _lib.default_config()
    c.j_max, c.r_cut, c.mld_order, c.precision, c.n_elements = float(j_max), float(r_cut), int(order), precision, len(els)
    if len(els) > 1:
        chw = channel_weights_for(els)
        c.weighted, c.weighted_3ch = 1, 1
        for k in range(len(els)):
            c.weight_per_element[k], c.weight_per_element_3ch[k] = chw[1, k], chw[2, k]
    n = len(d[f"{fit}_names"])
    nat = [d[f"{fit}_pos_{i}"].shape[0] for i in range(n)]
    with _lib.Handle(c) as h:
        h.set_structures(nat, np.concatenate([d[f"{fit}_pos_{i}"] for i in range(n)]),
                         np.stack([d[f"{fit}_cell_{i}"] for i in range(n)]),
                         np.concatenate([d[f"{fit}_types_{i}"] for i in range(n)]))
        E, F, S = h.evaluate(d[f"{fit}_w"]) if evaluate else h.predict(d[f"{fit}_w"])
    # plain: the printed precision of es20.10; mixed: FP32 descriptors and rows
    tol = 1e-9 if precision == 0 else 2e-4
    scaleE = max(np.abs([d[f"{fit}_E_{i}"][0] for i in range(n)]).max(), 1.0)
    a0 = 0
    for i in range(n):
        Er, Fr, Sr = d[f"{fit}_E_{i}"], d[f"{fit}_F_{i}"], d[f"{fit}_S_{i}"]
        assert abs(E[i] - Er[0]) <= tol * scaleE, (i, E[i], Er[0])
        if Fr.size:
            assert np.abs(F[a0:a0 + nat[i]].reshape(-1) - Fr).max() <= tol * max(np.abs(Fr).max(), 1.0)
        if Sr.size:
            assert np.abs(S[i] - Sr).max() <= tol * max(np.abs(Sr).max(), 0.1)
        a0 += nat[i]


def _small_dataset(seed=5):
    from mld_gb300 import synth
    rng = np.random.default_rng(seed)
    ds = synth.fe_bcc_batched(n_struct=6, nmin=16, nmax=300, seed=seed)
    return ds


def _oracle_rows(ds, j_max=4.0):
    rowsA, ys, ws = [], [], []
    for s in ds.structures:
        d = oracle.bispectrum(s.positions, s.cell, s.types, ds.rcut, j_max)
        e, f, st = oracle.linear_rows(d, s.cell)
        rowsA += [e[None, :], f, st]
        ys += [np.array([s.energies[1]]), s.forces.reshape(-1), s.stress]
        ws += [np.ones(1), np.ones(3 * s.nat), np.ones(6)]
    return np.concatenate(rowsA), np.concatenate(ys), np.concatenate(ws)


def _stage(h, ds):
    nat, pos, cell, types = ds.arrays()
    h.set_structures(nat, pos, cell, types)
    E, F, S, has = ds.labels()
    h.set_labels(E, F, S, has, np.ones((len(nat), 3)))


@pytest.mark.parametrize("precision,tol", [(0, TOL64), (1, TOL32)])
def test_descriptor_derivatives(lib, precision, tol):
    ds = _small_dataset()
    h = _handle(precision=precision)
    nat, pos, cell, types = ds.arrays()
    h.set_structures(nat, pos, cell, types)
    B, nn = h.descriptors()
    nbr, u, dB = h.descriptor_derivatives(int(nn.sum()) + 8)
    p = 0
    a0 = 0
    for s in ds.structures:
        d = oracle.bispectrum(s.positions, s.cell, s.types, ds.rcut, 4.0)
        for i in range(s.nat):
            n = d["nn"][i]
            assert nn[a0 + i] == n
            assert np.array_equal(nbr[p:p + n] - a0, d["nbr"][i, :n])
            assert np.allclose(u[p:p + n], d["u"][i, :n], rtol=0, atol=1e-12)
            got = dB[p:p + n]
            want = d["dB"][i, :n]
            assert _rel(got, want) < tol
            p += n
        assert _rel(B[a0:a0 + s.nat], d["B"]) < tol
        a0 += s.nat
    h.close()


@pytest.mark.parametrize("precision,tol", [(0, TOL64), (1, TOL32)])
def test_design_rows(lib, precision, tol):
    ds = _small_dataset()
    A_ref, y_ref, w_ref = _oracle_rows(ds)
    h = _handle(precision=precision)
    _stage(h, ds)
    A, y, w = h.design_matrix()
    assert A.shape == A_ref.shape
    assert np.array_equal(y, y_ref) and np.array_equal(w, w_ref)
    for lo, hi, name in [(0, 1, "E")]:
        assert _rel(A[lo:hi], A_ref[lo:hi]) < tol, name
    assert _rel(A, A_ref) < tol
    h.close()


def test_gram_and_solve_plain(lib):
    ds = _small_dataset()
    A_ref, y_ref, w_ref = _oracle_rows(ds)
    h = _handle(lam=1e-8)
    _stage(h, ds)
    G, rhs = h.gram()
    G_ref = A_ref.T @ (A_ref * w_ref[:, None])
    rhs_ref = A_ref.T @ (w_ref * y_ref)
    assert _rel(G, G_ref) < TOL64
    assert _rel(rhs, rhs_ref) < TOL64
    w, rank = h.solve(G_ref, rhs_ref)
    phi = G_ref + 1e-8 * np.eye(G_ref.shape[0])
    w_ref_fit = oracle.solve_gelsd(phi, rhs_ref)
    pred, pred_ref = A_ref @ w, A_ref @ w_ref_fit
    # predictions within the FP64 bar; coefficients within the rounding of the normal matrix
    # (eps) times its condition number (about 1e11 here)
    assert _rel(pred, pred_ref) < TOL64
    assert _rel(w, w_ref_fit) < 64 * np.finfo(float).eps * np.linalg.cond(phi)
    h.close()


def test_fit_end_to_end_plain(lib):
    ds = _small_dataset()
    A_ref, y_ref, w_ref = _oracle_rows(ds)
    h = _handle(lam=1e-8)
    _stage(h, ds)
    w, rmse = h.fit()
    w_or = oracle.fit_linear(A_ref, y_ref, w_ref, 1e-8)
    p, p_or = A_ref @ w, A_ref @ w_or
    assert _rel(p, p_or) < TOL64
    kinds = np.concatenate([[0] + [1] * (3 * s.nat) + [2] * 6 for s in ds.structures])
    for k in range(3):
        # the RMSE moves by at most the largest prediction difference
        r_or = oracle.rmse(p_or[kinds == k], y_ref[kinds == k])
        assert abs(rmse[k] - r_or) <= TOL64 * np.abs(p_or).max()
    # predictions through the serving entry point
    E, F, S = h.predict(w)
    rows_E = np.cumsum([0] + [1 + 3 * s.nat + 6 for s in ds.structures])[:-1]
    assert _rel(E, (A_ref @ w)[rows_E]) < 1e-10
    h.close()


def test_fit_mixed_close_to_plain(lib):
    ds = _small_dataset()
    h64 = _handle(lam=1e-8)
    _stage(h64, ds)
    w64, r64 = h64.fit()
    h32 = _handle(lam=1e-8, precision=1)
    _stage(h32, ds)
    w32, r32 = h32.fit()
    # force RMSE of the mixed fit within 1% of the FP64 fit
    assert abs(r32[1] - r64[1]) <= 0.01 * r64[1]
    h64.close()
    h32.close()


def test_neighbour_cap_is_reported(lib):
    from mld_gb300 import _lib
    ds = _small_dataset()
    c = _lib.default_config()
    c.j_max, c.r_cut, c.imm_neigh = 4.0, 4.7, 10
    h = _lib.Handle(c)
    nat, pos, cell, types = ds.arrays()
    h.set_structures(nat, pos, cell, types)
    with pytest.raises(_lib.MldError) as ei:
        h.descriptors()
    assert ei.value.code == 3
    # the handle stays usable after the error
    c2 = _lib.default_config()
    h.close()


@pytest.mark.parametrize("order,j_max", [(1, 4.0), (2, 2.0), (2, 4.0)])
@pytest.mark.parametrize("precision,tol", [(0, 1e-10), (1, 2e-5)])
def test_evaluate_matches_predict(lib, order, j_max, precision, tol):
    """Evaluation without design rows equals rows x weights (both box branches, two channels)."""
    from mld_gb300 import _lib, synth
    ds = synth.hea_bcc_batched(n_struct=5, reps=3, seed=31)
    structs = list(ds.structures) + list(synth.fe_bcc_batched(n_struct=3, nmin=2, nmax=40, seed=3).structures)
    c = _lib.default_config()
    c.j_max, c.r_cut, c.precision, c.mld_order, c.lambda_krr = j_max, 4.7, precision, order, 1e-6
    c.weighted, c.n_elements = 1, len(synth.HEA_ELEMENTS)
    for i, wv in enumerate(synth.HEA_WEIGHTS):
        c.weight_per_element[i] = wv
    sub = synth.Dataset(structs, 4.7, "mix")
    nat, pos, cell, types = sub.arrays()
    with _lib.Handle(c) as h:
        h.set_structures(nat, pos, cell, types)
        rng = np.random.default_rng(7)
        w = rng.standard_normal(h.dim_design_line) * 1e-3
        if order == 2:
            # full layout 1 + KK + KK^2: a symmetric quadratic block as a fit produces
            KK = int(round((-1 + np.sqrt(1 + 4 * (h.dim_design_line - 1))) / 2))
            Wq = rng.standard_normal((KK, KK)) * 1e-5
            w = np.concatenate([rng.standard_normal(1 + KK) * 1e-3, ((Wq + Wq.T) / 2).reshape(-1)])
        E0, F0, S0 = h.predict(w)
        E1, F1, S1 = h.evaluate(w)
    assert _rel(E1, E0) < tol
    assert _rel(F1, F0) < tol
    assert _rel(S1, S0) < tol
