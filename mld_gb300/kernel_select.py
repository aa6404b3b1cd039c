"""Reference points of the kernel model: the reference's randomised CUR selection.

The reference's descriptor analysis (main_descriptors_analysis.F90:316-372, kernel_dump = 3)
picks the kernel's reference atoms twice: from the configurations of the MCD classes
(``classes_for_mcd``, c = ``np_kernel_ref``) and from those of every class (c =
``np_kernel_full``), and concatenates the two lists (duplicates kept).  Each pick is
``compute_cur_decomposition`` (module_Sigma_matrix.F90:865-1052) on A = (descriptors - mean)^T,
components x atoms, the mean taken over the same atoms (compute_sca_phia :431-490,
get_dimension_design_Phi_by_class :162-202):

* leverage scores from the SVD A = U S V^T (compute_leverage_column_score :322-428): singular
  values s >= svd_rcond count towards the rank (an absolute cut; svd_rcond < 0 means 100 eps,
  mld_scalapack.F90:1815-1960), k = cur_kval (the rank when negative or larger),
  p_j = |V_k^T e_j|^2 / k per atom and q_i = |U_k^T e_i|^2 / k per component;
* r = cur_rval, int(k ln k / cur_eps^2) when negative;
* ten trials (cur_no_of_samples, ml_in_ndm_module.F90:245): atom j is selected when
  min(1, c p_j) >= u, component i when min(1, r q_i) >= u (perform_cur_selection :515-560); all
  ten column trials draw first, then the ten row trials;
* a trial's score is |A - C U R|_F with C = A[:, :n_col] / (c sqrt(p)), R = A[:n_row, :] /
  (r sqrt(q)) and U = C^+ A R^+ (compute_full_CUR_matrix :622-862).  The reference builds C and R
  from the LEADING n_col columns and n_row rows, not from the selected ones, so a trial's score
  depends on how many it selected; this is kept as the reference has it.  Pseudo-inverses cut
  singular values below max(s) * svd_rcond (scalapack_pseudo_inverse, mld_scalapack.F90:2120-2140);
* the first trial of lowest score wins and its selected atoms are the reference points.  Trials
  that reconstruct A exactly score at rounding level, where the reference's ``minloc`` follows
  rounding noise; here scores within 1e-9 |A|_F of the lowest are ties and the first one wins.

The uniform draws come from a seeded NumPy generator, not from the Fortran runtime's
``random_number``, so the selected atoms follow the same distribution as the reference's but not
the same stream.  All products are formed in the K-dimensional coordinates of the QR
factorisation of the (atoms x components) matrix: C U R = P_C A P_R with orthogonal projectors
P_C and P_R, and A = R_f^T Q^T, so the score is the Frobenius norm of a K x K residual.  It is
evaluated directly, without subtracting squared norms.

``select`` is a second, fixed-count sampler (weighted reservoir keys over the same leverage
scores) used where a workload needs an exact number of points (the benchmarks).
"""
from __future__ import annotations

import dataclasses
import numpy as np

CUR_TRIALS = 10  # cur_no_of_samples
TIE_REL = 1e-9   # trial scores closer than this times |A|_F are ties (the first one wins)


def _rcond(svd_rcond: float) -> float:
    return 100.0 * np.finfo(np.float64).eps if svd_rcond is None or svd_rcond < 0 else float(svd_rcond)


def _svd_coords(X: np.ndarray):
    """Singular values and right singular vectors of X (atoms x components) through its R factor."""
    R = np.linalg.qr(X, mode="r") if X.shape[0] >= X.shape[1] else X
    _, s, Vt = np.linalg.svd(R, full_matrices=False)
    return R, s, Vt.T


def _pinv_projector_cols(M: np.ndarray, rcond: float) -> np.ndarray:
    """Orthonormal basis of the column space kept by M's pseudo-inverse (s >= max(s) * rcond)."""
    if M.size == 0:
        return np.zeros((M.shape[0], 0))
    U, s, _ = np.linalg.svd(M, full_matrices=False)
    keep = s >= s.max() * rcond if s.size and s.max() > 0 else np.zeros(s.shape, bool)
    if not keep.any():
        raise ValueError("CUR: rank 0 matrix in the pseudo-inverse")
    return U[:, keep]


@dataclasses.dataclass
class CurResult:
    selected: np.ndarray      # atom indices of the winning trial, increasing
    pcol: np.ndarray          # leverage of each atom
    prow: np.ndarray          # leverage of each component
    k: int
    r: int
    rank: int
    n_col: np.ndarray         # atoms selected in each trial
    n_row: np.ndarray         # components selected in each trial
    scores: np.ndarray        # |A - CUR|_F of each trial
    winner: int


def leverage(B: np.ndarray, k: int = -1, svd_rcond: float = -1.0):
    """(pcol, prow, k, rank, X, R) of the descriptor matrix B (atoms x components): X is B centred
    on its mean, R the triangular factor of X."""
    X = np.asarray(B, dtype=np.float64)
    X = X - X.mean(axis=0)
    R, s, V = _svd_coords(X)
    rank = int((np.abs(s) >= _rcond(svd_rcond)).sum())
    if k is None or k < 0 or k > rank:
        k = rank
    if k == 0:
        raise ValueError("CUR: the centred descriptor matrix has rank 0")
    W = V[:, :k] / s[:k]
    P = X @ W
    pcol = (P * P).sum(axis=1) / k
    prow = (V[:, :k] ** 2).sum(axis=1) / k
    return pcol, prow, k, rank, X, R


def cur_select(B: np.ndarray, c: int, seed: int, k: int = -1, r: int = -1, eps: float = 1.0,
               svd_rcond: float = -1.0, trials: int = CUR_TRIALS) -> CurResult:
    """One ``compute_cur_decomposition``: the atoms of B (atoms x components) it selects."""
    pcol, prow, k, rank, X, Rf = leverage(B, k, svd_rcond)
    if r is None or r < 0:
        r = int(k * np.log(k) / eps ** 2)
    N, K = X.shape
    rng = np.random.default_rng(seed)
    ucol = rng.random((trials, N))
    urow = rng.random((trials, K))
    selcol = np.minimum(1.0, pcol * c)[None, :] >= ucol
    selrow = np.minimum(1.0, prow * r)[None, :] >= urow
    rc = _rcond(svd_rcond)
    # A = Xc^T = (Q Rf)^T: in Q coordinates the atoms' side of A is Rf^T (K x K, rows = components)
    if Rf.shape[0] < K:
        Rf = np.vstack([Rf, np.zeros((K - Rf.shape[0], K))])
    At = Rf.T  # K components x K coordinates
    scores = np.zeros(trials)
    ncol = selcol.sum(axis=1)
    nrow = selrow.sum(axis=1)
    with np.errstate(divide="ignore", invalid="ignore"):
        dc = np.where(pcol > 0, 1.0 / (c * np.sqrt(pcol)), 0.0)
        dr = np.where(prow > 0, 1.0 / (r * np.sqrt(prow)), 0.0)
    for t in range(trials):
        nc, nr = int(ncol[t]), int(nrow[t])
        if nc == 0 or nr == 0:
            scores[t] = np.sqrt((At * At).sum())
            continue
        C = X[:nc].T * dc[:nc]                    # K x nc, the leading columns of A
        Pc = _pinv_projector_cols(C, rc)         # K x rc
        Rm = At[:nr] * dr[:nr, None]             # nr x K, the leading rows of A in Q coordinates
        Pr = _pinv_projector_cols(Rm.T, rc)      # K x rr: row space of R
        E = At - Pc @ (Pc.T @ At @ Pr) @ Pr.T
        scores[t] = np.sqrt((E * E).sum())
    # trials that reconstruct A exactly score at rounding level, where the reference's minloc is
    # decided by rounding noise: scores within TIE_REL * |A|_F of the minimum count as equal
    norm_a = float(np.sqrt((At * At).sum()))
    win = int(np.flatnonzero(scores <= scores.min() + TIE_REL * norm_a)[0])
    return CurResult(np.flatnonzero(selcol[win]), pcol, prow, k, r, rank, ncol, nrow, scores, win)


def cur_kernel_points(B_inner: np.ndarray, B_full: np.ndarray, np_kernel_ref: int, np_kernel_full: int,
                      seed: int, k: int = -1, r: int = -1, eps: float = 1.0, svd_rcond: float = -1.0):
    """Both CUR picks: (indices into B_inner, indices into B_full), concatenated by the caller.
    cur_kval and cur_rval set by the first pick carry into the second, as the reference's
    intent(inout) arguments do."""
    first = cur_select(B_inner, np_kernel_ref, seed, k, r, eps, svd_rcond)
    second = cur_select(B_full, np_kernel_full, seed + 1, first.k, first.r, eps, svd_rcond)
    return first, second


def leverage_scores(B: np.ndarray, k: int = -1, rcond: float = -1.0):
    """Column leverage scores of the (uncentred) descriptor matrix, rows of B = atoms, with a
    relative singular-value cut (rcond * s_max)."""
    B = np.asarray(B, dtype=np.float64)
    ev, V = np.linalg.eigh(B.T @ B)
    order = np.argsort(ev)[::-1]
    ev, V = ev[order], V[:, order]
    s = np.sqrt(np.maximum(ev, 0.0))
    rank = int((s > _rcond(rcond) * s[0]).sum()) if s.size and s[0] > 0 else 0
    if k is None or k < 0 or k > rank:
        k = rank
    if k == 0:
        return np.full(B.shape[0], 1.0 / max(B.shape[0], 1)), 0
    P = B @ (V[:, :k] / s[:k])
    return (P * P).sum(axis=1) / k, k


def select(B: np.ndarray, nk: int, seed: int = 20240605, k: int = -1, rcond: float = -1.0) -> np.ndarray:
    """Indices (sorted) of exactly nk atoms drawn without replacement with probabilities
    proportional to their leverage (weighted reservoir keys u^(1/p))."""
    lev, _ = leverage_scores(B, k, rcond)
    n = lev.shape[0]
    if nk >= n:
        return np.arange(n)
    rng = np.random.default_rng(seed)
    p = np.maximum(lev, 1e-300)
    keys = np.log(rng.random(n)) / p
    idx = np.argpartition(-keys, nk - 1)[:nk]
    return np.sort(idx)
