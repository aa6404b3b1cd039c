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


@pytest.mark.parametrize("j_max,r_cut,channels,system", [
    (4.0, 4.7, 2, "hea"),   # K = 110: two K blocks of the tensor-core tiles
    (4.0, 4.7, 3, "hea"),   # K = 165: three K blocks, at most 40 vectors per tile
    (4.0, 6.0, 3, "hea"),   # about 65 vectors per atom: atoms split over two tiles
    (2.0, 6.6, 1, "fe"),    # 89 vectors per atom: split with one K block
])
def test_kernel_force_rows_mixed_vs_plain(lib, j_max, r_cut, channels, system):
    """FP32 kernel rows (force rows on the tensor cores) against the FP64 rows of the same
    handle setup, over K-block counts and atoms split over several tiles."""
    from mld_gb300 import _lib, synth
    if system == "fe":
        ds = synth.fe_bcc_batched(n_struct=3, nmin=16, nmax=60, seed=5)
        els, w2, w3 = ["Fe"], [1.0], [1.0]
    else:
        ds = synth.hea_bcc_batched(n_struct=3, reps=2, seed=11)
        els = list(synth.HEA_ELEMENTS)
        from mld_gb300 import elements as el
        w2, w3 = el.auto_channel_weights(els)
    nat, pos, cell, types = ds.arrays()

    def cfg(precision):
        c = _lib.default_config()
        c.j_max, c.r_cut, c.precision, c.ml_type, c.lambda_krr = j_max, r_cut, precision, 1, 1e-6
        c.kernel_power, c.length_kernel, c.sigma_kernel = 2.0, 1.3, 0.2
        c.n_elements = len(els)
        c.weighted, c.weighted_3ch = int(channels >= 2), int(channels >= 3)
        for i in range(len(els)):
            c.weight_per_element[i], c.weight_per_element_3ch[i] = w2[i], w3[i]
        return c

    c0 = cfg(0)
    c0.ml_type = 0
    with _lib.Handle(c0) as h:
        h.set_structures(nat, pos, cell, types)
        B, nn = h.descriptors()
    assert B.shape[1] == channels * {4.0: 55, 2.0: 14}[j_max]
    idx = np.random.default_rng(2).choice(B.shape[0], size=150, replace=B.shape[0] < 150)
    Zraw = B[idx]
    E, F, S, has = ds.labels()
    out = []
    for precision in (0, 1):
        with _lib.Handle(cfg(precision)) as h:
            h.set_structures(nat, pos, cell, types)
            h.set_labels(E, F, S, has, np.ones((len(nat), 3)))
            h.set_kernel_points(Zraw)
            A, _, _ = h.design_matrix()
        out.append(np.asarray(A, dtype=np.float64))
    KK = B.shape[1]
    kb0, kb1 = out[0][:, 1 + KK:], out[1][:, 1 + KK:]
    assert kb0.shape[1] == 150
    rows_E = np.cumsum([0] + [1 + 3 * n + 6 for n in nat])[:-1]
    fmask = np.ones(kb0.shape[0], bool)
    for r, n in zip(rows_E, nat):
        fmask[r] = False
        fmask[r + 1 + 3 * n: r + 1 + 3 * n + 6] = False
    assert nn.max() + 1 > (40 if channels == 3 else 80) or r_cut < 5
    ef, ea = _rel(kb1[fmask], kb0[fmask]), _rel(kb1, kb0)
    assert ef < 5e-5, (ef, ea)
    assert ea < 2e-4, (ef, ea)


@pytest.mark.parametrize("n_struct", [48, 12])
def test_kernel_fit_sketched_preconditioner(lib, n_struct):
    """A kernel block of D = 783 columns (768 reference points) takes the sketched preconditioner
    of the mixed method: a sparse sign sketch when the design rows exceed 3 D (48 structures),
    the weighted rows themselves otherwise (12 structures).  The mixed fit solves the same
    normal equations as the FP64 fit, so their training RMSEs and predictions agree."""
    from mld_gb300 import _lib, synth
    ds = synth.fe_bcc_batched(n_struct=n_struct, nmin=16, nmax=40, seed=23)
    nat, pos, cell, types = ds.arrays()
    E, F, S, has = ds.labels()
    c0 = _lib.default_config()
    c0.j_max, c0.r_cut, c0.precision, c0.ml_type = 2.0, 4.7, 0, 0
    with _lib.Handle(c0) as h:
        h.set_structures(nat, pos, cell, types)
        B, _ = h.descriptors()
    idx = np.random.default_rng(5).choice(B.shape[0], size=768, replace=B.shape[0] < 768)
    Zraw = B[idx] + np.random.default_rng(6).normal(scale=1e-6, size=(768, B.shape[1]))
    out = {}
    for precision in (0, 1):
        c = _lib.default_config()
        c.j_max, c.r_cut, c.precision, c.ml_type, c.lambda_krr = 2.0, 4.7, precision, 1, 1e-6
        with _lib.Handle(c) as h:
            h.set_structures(nat, pos, cell, types)
            h.set_labels(E, F, S, has, np.ones((len(nat), 3)))
            h.set_kernel_points(Zraw)
            assert h.dim_design_line == 1 + 14 + 768
            rows = h.num_rows()
            w, rmse = h.fit()
            Ep, Fp, Sp = h.predict(w)
            info = h.solve_info()
        out[precision] = (rmse, Ep, Fp, info, rows)
    (r0, E0, F0, _, rows), (r1, E1, F1, info1, _) = out[0], out[1]
    assert (rows > 3 * 783) == (n_struct == 48)
    # converged CG (not the iteration cap), RMSE within 1 % of FP64
    assert info1["pcg_iterations"][0] < 150, info1
    assert abs(r1[1] - r0[1]) <= 0.01 * r0[1], (r0, r1)
    assert abs(r1[0] - r0[0]) <= 0.01 * max(r0[0], 1e-3), (r0, r1)
    assert _rel(F1, F0) < 2e-2
