"""Reference points of the kernel model by leverage-score (CUR-style) column selection.

The reference chooses the atoms whose descriptors become the kernel's reference points with a
randomised CUR decomposition of the descriptor matrix (module_Sigma_matrix.F90:322-442 leverage
scores from the top-k right singular vectors, :515-560 Bernoulli selection with probability
min(1, c p_j)), written to kernel_matrix.dat by the descriptor-analysis run.  Here the column
leverage scores of the (components x atoms) descriptor matrix are formed from the eigen-pairs of
its small Gram matrix (components x components): p_j = |Sigma_k^-1 V_k^T b_j|^2 / k over the
singular values above rcond * sigma_max (rcond = 100 eps as in the reference); exactly nk atoms
are then drawn without replacement with probabilities proportional to p_j from a seeded
generator (weighted reservoir keys u^(1/p)).  This is an analysis step run once before a fit; the
descriptors come from the GPU (mld_gpu_descriptors).
"""
from __future__ import annotations

import numpy as np


def leverage_scores(B: np.ndarray, k: int = -1, rcond: float = -1.0):
    """Column leverage scores of the descriptor matrix (rows of B are atoms)."""
    B = np.asarray(B, dtype=np.float64)
    G = B.T @ B
    ev, V = np.linalg.eigh(G)
    order = np.argsort(ev)[::-1]
    ev, V = ev[order], V[:, order]
    sv = np.sqrt(np.maximum(ev, 0.0))
    if rcond is None or rcond < 0:
        rcond = 100.0 * np.finfo(np.float64).eps
    rank = int((sv > rcond * sv[0]).sum()) if sv.size and sv[0] > 0 else 0
    if k is None or k < 0 or k > rank:
        k = rank
    if k == 0:
        return np.full(B.shape[0], 1.0 / max(B.shape[0], 1)), 0
    P = B @ (V[:, :k] / sv[:k])
    lev = (P * P).sum(axis=1) / k
    return lev, k


def select(B: np.ndarray, nk: int, seed: int = 20240605, k: int = -1, rcond: float = -1.0) -> np.ndarray:
    """Indices (sorted) of nk atoms drawn with probabilities proportional to their leverage."""
    lev, _ = leverage_scores(B, k, rcond)
    n = lev.shape[0]
    if nk >= n:
        return np.arange(n)
    rng = np.random.default_rng(seed)
    p = np.maximum(lev, 1e-300)
    keys = np.log(rng.random(n)) / p
    idx = np.argpartition(-keys, nk - 1)[:nk]
    return np.sort(idx)
