"""Python front-end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Loads ``oracle/liboracle.so`` (built from bso4_oracle.c by oracle/Makefile) and restates the
fit step of MILADY in NumPy/SciPy:

* weighted normal matrix  phi = A W A^T + lambda*I (lambda<0 -> 0), rhs = A W y, solved with
  LAPACK ``gelsd`` (SVD, minimum norm, rcond) -- MILADY src/mld/parameters.F90:1018-1099 and
  src/mld/stats_tools.F90:1153-1213 (``serial_lsystem_by_svd``);
* predictions w . row and RMSE -- src/mld/mld.F90:40-86,944-1020, src/mld/stats_tools.F90:1551-1559.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import Dict, Optional, Sequence

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB: Optional[ctypes.CDLL] = None
_STATE = {"j_max": None, "inv_r0": None, "K": 0}

DEFAULT_INV_R0_INPUT = 1.0 - 0.02 / np.pi   # read_ml_file.F90:425


def build() -> str:
    path = os.path.join(_HERE, "liboracle.so")
    src = os.path.join(_HERE, "bso4_oracle.c")
    if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
        subprocess.check_call(["make", "-s", "-C", _HERE])
    return path


def lib() -> ctypes.CDLL:
    global _LIB
    if _LIB is None:
        _LIB = ctypes.CDLL(build())
        d, i, p = ctypes.c_double, ctypes.c_int, ctypes.c_void_p
        _LIB.orc_init.argtypes = [d, d]
        _LIB.orc_init.restype = i
        _LIB.orc_num_u.restype = i
        _LIB.orc_num_cg.argtypes = [i]
        _LIB.orc_num_cg.restype = ctypes.c_long
        _LIB.orc_triples.argtypes = [p, p, p]
        _LIB.orc_cg_value.argtypes = [i] * 6
        _LIB.orc_cg_value.restype = d
        _LIB.orc_volume.argtypes = [p]
        _LIB.orc_volume.restype = d
        _LIB.orc_small_box.argtypes = [p, d, p]
        _LIB.orc_neighbours.argtypes = [i, p, p, d, i, p, p, p, p]
        _LIB.orc_bispectrum.argtypes = [i, p, i, i, p, p, d, d, p, p, p, i, p, p]
        _LIB.orc_rows_linear.argtypes = [i, i, p, p, p, p, p, i, i, d, d, d, p, p, p]
    return _LIB


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def init(j_max: float = 4.0, inv_r0_input: float = DEFAULT_INV_R0_INPUT) -> int:
    L = lib()
    if _STATE["j_max"] != j_max or _STATE["inv_r0"] != inv_r0_input:
        K = L.orc_init(float(j_max), float(inv_r0_input))
        if K < 0:
            raise ValueError(f"orc_init failed ({K})")
        _STATE.update(j_max=j_max, inv_r0=inv_r0_input, K=K)
    return _STATE["K"]


def triples() -> np.ndarray:
    K = _STATE["K"]
    a = np.zeros((3, K), dtype=np.int32)
    lib().orc_triples(_ptr(a[0]), _ptr(a[1]), _ptr(a[2]))
    return a.T.copy()


def cg(j1, m1, j2, m2, j, m) -> float:
    return lib().orc_cg_value(j1, m1, j2, m2, j, m)


def neighbours(positions: np.ndarray, cell: np.ndarray, r_cut: float, cap: int = 300):
    pos = np.ascontiguousarray(positions, dtype=np.float64)
    cel = np.ascontiguousarray(cell, dtype=np.float64)
    nat = pos.shape[0]
    nn = np.zeros(nat, dtype=np.int32)
    nbr = np.zeros((nat, cap), dtype=np.int32)
    u = np.zeros((nat, cap, 3), dtype=np.float64)
    small = ctypes.c_int(0)
    rc = lib().orc_neighbours(nat, _ptr(pos), _ptr(cel), float(r_cut), cap, _ptr(nn), _ptr(nbr), _ptr(u),
                              ctypes.byref(small))
    if rc != 0:
        raise OverflowError("neighbour cap exceeded")
    return nn, nbr, u, bool(small.value)


def bispectrum(positions, cell, types, r_cut: float, j_max: float = 4.0, *,
               channel_weights: Optional[np.ndarray] = None, want_deriv: bool = True,
               inv_r0_input: float = DEFAULT_INV_R0_INPUT, cap: int = 300,
               r_in_pair: Optional[np.ndarray] = None, r_in_width: float = 0.4) -> Dict[str, np.ndarray]:
    """Per-atom B (nat, nch*K) and, if asked, dB (nat, cap, 3, nch*K) plus the neighbour list."""
    K = init(j_max, inv_r0_input)
    types = np.ascontiguousarray(types, dtype=np.int32)
    ntypes = int(types.max()) + 1 if types.size else 1
    if channel_weights is None:
        channel_weights = np.ones((1, ntypes))
    chw = np.ascontiguousarray(channel_weights, dtype=np.float64)
    nch, ntypes = chw.shape
    nn, nbr, u, small = neighbours(positions, cell, r_cut, cap)
    nat = types.shape[0]
    B = np.zeros((nat, nch * K))
    dB = np.zeros((nat, cap, 3, nch * K)) if want_deriv else None
    rin = None if r_in_pair is None else np.ascontiguousarray(r_in_pair, dtype=np.float64)
    lib().orc_bispectrum(nat, _ptr(types), ntypes, nch, _ptr(chw), _ptr(rin), float(r_in_width), float(r_cut),
                         _ptr(nn), _ptr(nbr), _ptr(u), cap, _ptr(B), _ptr(dB))
    return dict(B=B, dB=dB, nn=nn, nbr=nbr, u=u, small=small, cap=cap)


def linear_rows(desc: Dict[str, np.ndarray], cell: np.ndarray, *, sign_stress: float = 1.0,
                sign_big: float = 1.0):
    B, dB = desc["B"], desc["dB"]
    nat, KK = B.shape
    D = 1 + KK
    rowE = np.zeros(D)
    rowF = np.zeros((3 * nat, D))
    rowS = np.zeros((6, D))
    vol = lib().orc_volume(_ptr(np.ascontiguousarray(cell, dtype=np.float64)))
    lib().orc_rows_linear(nat, KK, _ptr(B), _ptr(dB), _ptr(desc["nn"]), _ptr(desc["nbr"]), _ptr(desc["u"]),
                          desc["cap"], int(desc["small"]), float(sign_stress), float(sign_big), float(vol),
                          _ptr(rowE), _ptr(rowF), _ptr(rowS))
    return rowE, rowF, rowS


def solve_gelsd(phi: np.ndarray, rhs: np.ndarray, rcond: float = -1.0) -> np.ndarray:
    """dgelsd on the (D x D) normal matrix, as serial_lsystem_by_svd does."""
    import scipy.linalg
    if rcond is None or rcond < 0:
        rcond = np.finfo(np.float64).eps
    w, *_ = scipy.linalg.lstsq(phi, rhs, cond=rcond, lapack_driver="gelsd")
    return w


def normal_equations(A: np.ndarray, y: np.ndarray, wts: np.ndarray, lam: float):
    """phi = A^T W A + lambda I (lambda<0 -> 0), rhs = A^T W y  (A is rows x D)."""
    lam = 0.0 if lam < 0 else lam
    AW = A * wts[:, None]
    phi = A.T @ AW
    phi[np.diag_indices_from(phi)] += lam
    rhs = AW.T @ y
    return phi, rhs


def fit_linear(A: np.ndarray, y: np.ndarray, wts: np.ndarray, lam: float, rcond: float = -1.0) -> np.ndarray:
    phi, rhs = normal_equations(A, y, wts, lam)
    return solve_gelsd(phi, rhs, rcond)


def rmse(pred: np.ndarray, ref: np.ndarray) -> float:
    d = np.asarray(pred) - np.asarray(ref)
    return float(np.sqrt(np.mean(d * d))) if d.size else 0.0


def quadratic_rows(desc: Dict[str, np.ndarray], cell: np.ndarray, *, sign_stress: float = 1.0,
                   sign_big: float = 1.0):
    """Quadratic design rows in the reference's full layout (1 + KK + KK*KK columns)."""
    L = lib()
    L.orc_rows_quadratic.argtypes = L.orc_rows_linear.argtypes
    B, dB = desc["B"], desc["dB"]
    nat, KK = B.shape
    D = 1 + KK + KK * KK
    rowE = np.zeros(D)
    rowF = np.zeros((3 * nat, D))
    rowS = np.zeros((6, D))
    vol = L.orc_volume(_ptr(np.ascontiguousarray(cell, dtype=np.float64)))
    L.orc_rows_quadratic(nat, KK, _ptr(B), _ptr(dB), _ptr(desc["nn"]), _ptr(desc["nbr"]), _ptr(desc["u"]),
                         desc["cap"], int(desc["small"]), float(sign_stress), float(sign_big), float(vol),
                         _ptr(rowE), _ptr(rowF), _ptr(rowS))
    return rowE, rowF, rowS


def fit_qnml(A: np.ndarray, y: np.ndarray, wts: np.ndarray, lam: float, n_linear: int, rcond: float = -1.0):
    """QNML two-stage fit (parameters.F90:404-421, 476-1015): linear block first, then the
    quadratic block on the residual, both with the linear ridge/gelsd solver."""
    AL, AQ = A[:, :n_linear], A[:, n_linear:]
    wL = fit_linear(AL, y, wts, lam, rcond)
    res = y - AL @ wL
    wQ = fit_linear(AQ, res, wts, lam, rcond)
    return np.concatenate([wL, wQ])


def kernel_points(B_ref: np.ndarray):
    """Standardised reference points of the kernel (compute_kernel.F90:1058-1256, init_kernel):
    z = (z_raw - mean) / std over the reference set (std = population standard deviation)."""
    Br = np.asarray(B_ref, dtype=np.float64)
    mean = Br.mean(axis=0)
    std = np.sqrt(((Br - mean) ** 2).sum(axis=0) / Br.shape[0])
    return (Br - mean) / std, mean, std


def kernel_rows(desc: Dict[str, np.ndarray], cell: np.ndarray, Z: np.ndarray, *, power: float = 2.0,
                length: float = np.sqrt(0.5), sigma: float = 0.0, sign_stress: float = 1.0, sign_big: float = 1.0):
    """Kernel ridge design rows (polynomial kernel) in the reference layout 1 + KK + nk."""
    L = lib()
    d, i, p = ctypes.c_double, ctypes.c_int, ctypes.c_void_p
    L.orc_rows_kernel.argtypes = [i, i, p, p, p, p, p, i, i, d, d, d, i, p, d, d, d, p, p, p]
    B, dB = desc["B"], desc["dB"]
    nat, KK = B.shape
    Zc = np.ascontiguousarray(Z, dtype=np.float64)
    nk = Zc.shape[0]
    D = 1 + KK + nk
    rowE = np.zeros(D)
    rowF = np.zeros((3 * nat, D))
    rowS = np.zeros((6, D))
    vol = L.orc_volume(_ptr(np.ascontiguousarray(cell, dtype=np.float64)))
    L.orc_rows_kernel(nat, KK, _ptr(B), _ptr(dB), _ptr(desc["nn"]), _ptr(desc["nbr"]), _ptr(desc["u"]),
                      desc["cap"], int(desc["small"]), float(sign_stress), float(sign_big), float(vol), nk, _ptr(Zc),
                      float(power), float(length), float(sigma), _ptr(rowE), _ptr(rowF), _ptr(rowS))
    return rowE, rowF, rowS


def fit_kernel(A: np.ndarray, y: np.ndarray, wts: np.ndarray, lam: float, rcond: float = -1.0) -> np.ndarray:
    """Kernel ridge solve (parameters.F90:1217-1395): [sqrt(W) A; lambda I] w ~ [sqrt(W) y; 0], i.e.
    the normal equations with a lambda^2 penalty (lambda < 0 -> 0)."""
    lam = 0.0 if lam < 0 else lam
    phi, rhs = normal_equations(A, y, wts, lam * lam)
    return solve_gelsd(phi, rhs, rcond)


def _pinv_cut(M: np.ndarray, rcond: float) -> np.ndarray:
    """Pseudo-inverse keeping singular values s >= max(s) * rcond
    (scalapack_pseudo_inverse, mld_scalapack.F90:1975-2300)."""
    U, s, Vt = np.linalg.svd(M, full_matrices=False)
    keep = s >= s.max() * rcond
    return (Vt[keep].T / s[keep]) @ U[:, keep].T


def cur_decomposition(B: np.ndarray, c: int, ucol: np.ndarray, urow: np.ndarray, k: int = -1, r: int = -1,
                      eps: float = 1.0, svd_rcond: float = -1.0):
    """Randomised CUR selection of kernel reference atoms, with explicit matrices (small cases):
    compute_cur_decomposition, module_Sigma_matrix.F90:865-1052.  ``ucol`` (trials x atoms) and
    ``urow`` (trials x components) are the uniform draws of the trials, in the reference's order.

    * A = (B - mean)^T, components x atoms (compute_sca_phia :431-490; mean over the same atoms,
      get_dimension_design_Phi_by_class :162-202);
    * leverage (compute_leverage_column_score :322-428): rank = #{s >= svd_rcond} (100 eps when
      negative), k = rank unless cur_kval is set and smaller, p_j = |VT(1:k, j)|^2 / k of A and
      q_i of A^T; r = int(k ln k / eps^2) when negative;
    * trial t selects atom j when min(1, c p_j) >= u (perform_cur_selection :515-560), and
      component i when min(1, r q_i) >= u;
    * score |A - C U R|_F, C = A(:, 1:n_col) / (c sqrt(p)), R = A(1:n_row, :) / (r sqrt(q)),
      U = C^+ A R^+ (compute_full_CUR_matrix :622-862);
    * the winner is minloc of the scores.
    Returns (selected atoms of every trial, pcol, prow, k, r, scores, winner)."""
    B = np.asarray(B, dtype=np.float64)
    A = (B - B.mean(axis=0)).T
    tol = 100.0 * np.finfo(np.float64).eps if svd_rcond < 0 else svd_rcond
    _, s, VT = np.linalg.svd(A, full_matrices=False)
    rank = int(np.sum(np.abs(s) >= tol))
    if k < 0 or k > rank:
        k = rank
    if r < 0:
        r = int(k * np.log(k) / eps ** 2)
    nK, nA = A.shape
    pcol = np.array([np.sum(VT[:k, j] ** 2) / k for j in range(nA)])
    _, s2, VT2 = np.linalg.svd(A.T, full_matrices=False)
    prow = np.array([np.sum(VT2[:k, i] ** 2) / k for i in range(nK)])
    trials = ucol.shape[0]
    sel, scores = [], []
    for t in range(trials):
        selcol = np.array([min(1.0, pcol[j] * c) >= ucol[t, j] for j in range(nA)])
        selrow = np.array([min(1.0, prow[i] * r) >= urow[t, i] for i in range(nK)])
        nc, nr = int(selcol.sum()), int(selrow.sum())
        C = A[:, :nc] / (c * np.sqrt(pcol[:nc]))[None, :]
        R = A[:nr, :] / (r * np.sqrt(prow[:nr]))[:, None]
        U = _pinv_cut(C, tol) @ A @ _pinv_cut(R, tol)
        scores.append(np.linalg.norm(A - C @ U @ R))
        sel.append(np.flatnonzero(selcol))
    win = int(np.argmin(scores))
    return sel, pcol, prow, k, r, np.array(scores), win
