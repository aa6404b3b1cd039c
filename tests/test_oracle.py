"""CPU tests of the oracle: pinned against MILADY's own golden descriptors (fit17) and checked
for internal consistency (derivatives vs finite differences, CG identities)."""
import numpy as np
import pytest

import oracle


def test_dimensions_jmax4():
    K = oracle.init(4.0)
    assert K == 55                                   # 55 B components (fit17 .eml: 56 columns)
    L = oracle.lib()
    assert L.orc_num_u() == 285                      # sum_{j<=8} (j+1)^2
    assert [L.orc_num_cg(i) for i in range(3)] == [34946, 34946, 34946]


def test_cg_orthonormality():
    oracle.init(4.0)
    # sum_{m1,m2} <j1 m1 j2 m2|j m><j1 m1 j2 m2|j' m'> = delta_jj' delta_mm'  (doubled indices)
    for j1, j2 in [(2, 2), (3, 1), (4, 2), (3, 3)]:
        for j in range(abs(j1 - j2), j1 + j2 + 1, 2):
            for jp in range(abs(j1 - j2), j1 + j2 + 1, 2):
                for m in range(-min(j, jp), min(j, jp) + 1, 2):
                    s = sum(oracle.cg(j1, m1, j2, m - m1, j, m) * oracle.cg(j1, m1, j2, m - m1, jp, m)
                            for m1 in range(-j1, j1 + 1, 2) if abs(m - m1) <= j2)
                    assert abs(s - (1.0 if j == jp else 0.0)) < 1e-12


def test_fit17_golden_descriptors(fit17):
    """The oracle reproduces REF/descDB/*.eml of MILADY's fit17 test (small and large boxes)."""
    worst = 0.0
    kinds = set()
    for i, name in enumerate(fit17["names"]):
        d = oracle.bispectrum(fit17[f"pos_{i}"], fit17[f"cell_{i}"], fit17[f"types_{i}"], 4.7, 4.0,
                              want_deriv=False)
        ref = fit17[f"B_{i}"]
        kinds.add(d["small"])
        worst = max(worst, np.abs(d["B"] - ref).max() / np.abs(ref).max())
    assert kinds == {True, False}
    assert worst < 1e-13


def _energy_row_sum(pos, cell, types):
    return oracle.bispectrum(pos, cell, types, 4.7, 4.0, want_deriv=False)["B"].sum(0)


def test_fit19_golden_three_channel_descriptors(fit19):
    """The oracle reproduces MILADY's fit19 REF/descDB (Ta-Ti-V-W, weighted + weighted_3ch with
    weighted_auto): channel 2 weights Z / rms(Z), channel 3 (m^2 + r_cov^2) / mean, masses at the
    reference's single precision."""
    from mld_gb300 import elements
    els = [str(e) for e in fit19["elements"]]
    w2, w3 = elements.auto_channel_weights(els)
    chw = np.stack([np.ones(len(els)), w2, w3])
    for i in range(len(fit19["names"])):
        d = oracle.bispectrum(fit19[f"pos_{i}"], fit19[f"cell_{i}"], fit19[f"types_{i}"], 4.7, 4.0,
                              channel_weights=chw, want_deriv=False)
        ref = fit19[f"B_{i}"]
        assert d["B"].shape == ref.shape
        assert np.abs(d["B"] - ref).max() / np.abs(ref).max() < 1e-13
    # with the masses in double precision channel 3 misses by ~1e-8: the binary32 rounding is real
    m64 = np.array([elements.TABLE[e][1] for e in els])
    rc = np.array([elements.covalent_radius(e) for e in els])
    w3_64 = (m64 ** 2 + rc ** 2) / np.mean(m64 ** 2 + rc ** 2)
    assert 1e-9 < np.abs(w3_64 - w3).max() < 1e-6


@pytest.mark.parametrize("fit", ["fit03", "fit08"])
def test_reference_run_predictions(predictions, fit):
    """Design rows x the .pot weights of a reference run reproduce that run's train_*.out
    predictions (es20.10): fit03 quadratic QNML incl. 1-atom small-box stresses, fit08 3-channel
    weighted linear."""
    from conftest import channel_weights_for
    d = predictions
    j_max, r_cut, order = d[f"{fit}_params"]
    els = [str(e) for e in d[f"{fit}_elements"]]
    chw = channel_weights_for(els) if len(els) > 1 else None
    rows = oracle.quadratic_rows if int(order) == 2 else oracle.linear_rows
    w = d[f"{fit}_w"]
    for i in range(len(d[f"{fit}_names"])):
        desc = oracle.bispectrum(d[f"{fit}_pos_{i}"], d[f"{fit}_cell_{i}"], d[f"{fit}_types_{i}"], float(r_cut),
                                 float(j_max), channel_weights=chw)
        e, f, st = rows(desc, d[f"{fit}_cell_{i}"])
        E, F, S = d[f"{fit}_E_{i}"], d[f"{fit}_F_{i}"], d[f"{fit}_S_{i}"]
        assert abs(e @ w - E[0]) <= 1e-9 * max(abs(E[0]), 1.0)
        if F.size:
            assert np.abs(f @ w - F).max() <= 1e-9 * max(np.abs(F).max(), 1.0)
        if S.size:
            assert np.abs(st @ w - S).max() <= 1e-10 * max(np.abs(S).max(), 1.0)


@pytest.mark.parametrize("idx", [2, 9])
def test_force_rows_are_negative_gradient(fit17, idx):
    pos = fit17[f"pos_{idx}"].copy()
    cell, types = fit17[f"cell_{idx}"], fit17[f"types_{idx}"]
    d = oracle.bispectrum(pos, cell, types, 4.7, 4.0)
    _, rowF, _ = oracle.linear_rows(d, cell)
    h = 1e-5
    for a in (0, 1):
        for c in range(3):
            p1 = pos.copy(); p1[a, c] += h
            p2 = pos.copy(); p2[a, c] -= h
            fd = -(_energy_row_sum(p1, cell, types) - _energy_row_sum(p2, cell, types)) / (2 * h)
            an = rowF[3 * a + c, 1:]
            assert np.abs(fd - an).max() <= 1e-6 * np.abs(an).max() + 1e-9


def test_weighted_channels_scale():
    """A weighted channel with all element weights 1 equals the plain channel."""
    from mld_gb300 import synth
    pos, cell = synth.bcc(2, 2, 2, 3.2)
    rng = np.random.default_rng(3)
    pos = pos + rng.normal(0, 0.05, pos.shape)
    types = np.array([0, 1] * 8, np.int32)
    chw = np.array([[1.0, 1.0], [1.0, 1.0]])
    d = oracle.bispectrum(pos, cell, types, 5.0, 4.0, channel_weights=chw)
    assert np.allclose(d["B"][:, :55], d["B"][:, 55:], rtol=0, atol=1e-12)
    chw2 = np.array([[1.0, 1.0], [0.5, 2.0]])
    d2 = oracle.bispectrum(pos, cell, types, 5.0, 4.0, channel_weights=chw2)
    assert np.allclose(d2["B"][:, :55], d["B"][:, :55])
    assert not np.allclose(d2["B"][:, 55:], d["B"][:, 55:])


def test_gelsd_min_norm_on_rank_deficient():
    rng = np.random.default_rng(0)
    A = rng.normal(size=(50, 6))
    A[:, 5] = A[:, 4]                     # duplicate column -> rank 5
    y = rng.normal(size=50)
    w = oracle.fit_linear(A, y, np.ones(50), -1.0)
    assert abs(w[4] - w[5]) < 1e-10       # minimum norm splits the duplicate evenly


def test_kernel_rows_are_gradients_of_the_energy_row():
    """Kernel force rows equal minus the position gradient of the kernel energy row, the
    convention of the linear rows (compute_kernel.F90:91-150 with the mld_forces packing)."""
    from mld_gb300 import synth
    ds = synth.fe_bcc_batched(n_struct=1, nmin=16, nmax=40, seed=4)
    s = ds.structures[0]
    d = oracle.bispectrum(s.positions, s.cell, s.types, 4.7, 1.5)
    Z, _, _ = oracle.kernel_points(d["B"][:6])
    E, F, S = oracle.kernel_rows(d, s.cell, Z, power=2.0, length=0.8, sigma=0.3)
    h = 1e-5
    for atom, comp in ((0, 0), (3, 2)):
        rows = []
        for sgn in (1, -1):
            p = s.positions.copy()
            p[atom, comp] += sgn * h
            dd = oracle.bispectrum(p, s.cell, s.types, 4.7, 1.5)
            rows.append(oracle.kernel_rows(dd, s.cell, Z, power=2.0, length=0.8, sigma=0.3)[0])
        fd = (rows[0] - rows[1]) / (2 * h)
        assert np.abs(fd + F[3 * atom + comp]).max() <= 1e-6 * max(1.0, np.abs(fd).max())
