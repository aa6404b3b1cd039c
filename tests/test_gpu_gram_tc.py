"""Tensor-core Gram (tcgen05, BF16 split precision) and the mixed-method solve.

The Gram of the mixed method is x'_i x'_j ~= hi_i hi_j + hi_i lo_j + lo_i hi_j with
x' = sqrt(w) x = hi + lo (bf16), accumulated in FP32 per row split and in FP64 across splits.
It is checked (a) against a NumPy emulation of exactly that split (products exact in FP64), to
the FP32 accumulation tolerance, and (b) against the FP64 Gram, to the split's truncation
tolerance.  Tolerances are relative to sqrt(G_ii G_jj).  The mixed fit then refines with
conjugate gradients on FP64-accumulated matvecs over X and must reproduce the FP64 fit.
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

TOL_EMULATED = 3e-6   # tensor-core FP32 accumulation (short chains, compensated sums) vs exact BF16x3
TOL_FP64 = 6e-5       # BF16x3 (lo*lo and the 17th+ mantissa bits dropped) vs FP64


def _bf16(x):
    x = np.ascontiguousarray(x, dtype=np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def _emulate(X, w):
    v = (X.astype(np.float64) * np.sqrt(w)[:, None]).astype(np.float32)
    hi = _bf16(v)
    lo = _bf16(v - hi)
    h, l = hi.astype(np.float64), lo.astype(np.float64)
    return h.T @ h + h.T @ l + l.T @ h


def _scaled_err(G, Gref):
    d = np.sqrt(np.maximum(np.diag(Gref), 1e-300))
    return float(np.abs((G - Gref) / np.outer(d, d)).max())


def _rows(M, D, ldx, seed, dtype):
    rng = np.random.default_rng(seed)
    # columns of very different scales and a shared component, like descriptor columns
    scale = 10.0 ** rng.uniform(-3, 2, size=D)
    base = rng.normal(size=(M, 1))
    X = (rng.normal(size=(M, D)) + 0.7 * base) * scale
    Xp = np.zeros((M, ldx), dtype=dtype)
    Xp[:, :D] = X
    w = rng.uniform(0.2, 3.0, size=M)
    y = rng.normal(size=M)
    return Xp, w, y


@pytest.mark.parametrize("M,D,ldx,fp32", [
    (1000, 56, 56, True),
    (70001, 300, 304, True),
    (5000, 129, 132, True),
    (64, 1, 4, True),
    (130, 257, 260, True),
    (20000, 1024, 1024, True),
    (9000, 200, 201, False),
])
def test_gram_rows_tensor_cores(lib, M, D, ldx, fp32):
    import torch
    from mld_gb300 import _lib
    Xp, w, y = _rows(M, D, ldx, seed=M + D, dtype=np.float32 if fp32 else np.float64)
    dev = torch.device("cuda:0")
    tX = torch.from_numpy(Xp).to(dev)
    tw = torch.from_numpy(w).to(dev)
    ty = torch.from_numpy(y).to(dev)
    tG = torch.empty((D, D), dtype=torch.float64, device=dev)
    th = torch.empty(D, dtype=torch.float64, device=dev)
    _lib.gram_rows(_lib.MIXED, tX.data_ptr(), fp32, M, D, ldx, tw.data_ptr(), ty.data_ptr(), tG.data_ptr(),
                   th.data_ptr())
    G, h = tG.cpu().numpy(), th.cpu().numpy()
    X = Xp[:, :D].astype(np.float64)
    G64 = X.T @ (X * w[:, None])
    h64 = X.T @ (w * y)
    assert np.array_equal(G, G.T)
    e_emu = _scaled_err(G, _emulate(Xp[:, :D], w))
    e_64 = _scaled_err(G, G64)
    assert e_emu < TOL_EMULATED, e_emu
    assert e_64 < TOL_FP64, e_64
    assert np.abs(h - h64).max() <= 1e-11 * np.abs(X * w[:, None] * y[:, None]).sum(0).max()
    # the plain method of the same entry point is FP64 throughout
    _lib.gram_rows(_lib.PLAIN_FP64, tX.data_ptr(), fp32, M, D, ldx, tw.data_ptr(), ty.data_ptr(), tG.data_ptr(),
                   th.data_ptr())
    assert _scaled_err(tG.cpu().numpy(), G64) < 1e-12


def test_gram_rows_rejects_bad_arguments(lib):
    from mld_gb300 import _lib
    with pytest.raises(_lib.MldError) as ei:
        _lib.gram_rows(_lib.MIXED, 0, True, 10, 4, 4, 0, 0, 0)
    assert ei.value.code == 1


def _fe_dataset():
    from mld_gb300 import synth
    return synth.fe_bcc_batched(n_struct=6, nmin=16, nmax=140, seed=21)


def _stage(h, ds):
    nat, pos, cell, types = ds.arrays()
    h.set_structures(nat, pos, cell, types)
    E, F, S, has = ds.labels()
    h.set_labels(E, F, S, has, np.ones((len(nat), 3)))


def _handle(precision, order=1, j_max=4.0, lam=1e-8):
    from mld_gb300 import _lib
    c = _lib.default_config()
    c.j_max, c.r_cut, c.lambda_krr, c.precision, c.mld_order = j_max, 4.7, lam, precision, order
    return _lib.Handle(c)


def test_handle_gram_mixed_uses_split_precision(lib):
    ds = _fe_dataset()
    with _handle(1) as h:
        _stage(h, ds)
        G, rhs = h.gram()
        A, y, w = h.design_matrix()
    A = A.astype(np.float64)
    G64 = A.T @ (A * w[:, None])
    assert _scaled_err(G, G64) < TOL_FP64
    # the FP32 force rows are accumulated with atomics, so two builds of X differ in the last bits
    # (and their bf16 splits by up to one unit of lo): a looser bound than for identical rows
    assert _scaled_err(G, _emulate(A.astype(np.float32), w)) < 5 * TOL_EMULATED
    assert np.abs(rhs - A.T @ (w * y)).max() <= 2e-6 * np.abs(A.T @ np.abs(w * y)).max()


def test_mixed_linear_fit_reaches_fp64_solution(lib):
    ds = _fe_dataset()
    with _handle(0) as h64:
        _stage(h64, ds)
        w64, r64 = h64.fit()
        A, y, wr = h64.design_matrix()
    with _handle(1) as h32:
        _stage(h32, ds)
        w32, r32 = h32.fit()
        info = h32.solve_info()
    assert 1 <= info["pcg_iterations"][0] < 60
    assert info["pcg_residual"][0] < 1e-6
    p64, p32 = A @ w64, A @ w32
    # predictions of the two fits on the FP64 rows agree far better than the 1% RMSE target
    assert np.abs(p32 - p64).max() <= 1e-4 * np.abs(p64).max()
    for k in range(3):
        assert abs(r32[k] - r64[k]) <= 1e-3 * r64[k]


def test_mixed_qnml_fit_force_rmse_within_one_percent(lib):
    from mld_gb300 import synth
    ds = synth.fe_bcc_batched(n_struct=5, nmin=16, nmax=200, seed=9)
    lam = 1e-6
    with _handle(0, order=2, j_max=1.5, lam=lam) as h64:
        _stage(h64, ds)
        w64, r64 = h64.fit()
    with _handle(1, order=2, j_max=1.5, lam=lam) as h32:
        _stage(h32, ds)
        w32, r32 = h32.fit()
        info = h32.solve_info()
    assert info["pcg_iterations"][1] >= 1
    assert abs(r32[1] - r64[1]) <= 0.01 * r64[1]
    assert abs(r32[0] - r64[0]) <= 0.01 * r64[0] + 1e-9
