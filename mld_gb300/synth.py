"""Seeded synthetic training sets standing in for MILADY's POSCAR databases.

No public dataset is used by the reference for this path; the workloads are bcc supercells with
thermal noise, strain and vacancies, labelled by a Morse pair potential.  Labels:

* energy  E = sum over pairs r < r_c of D[(1-exp(-a(r-r0)))^2 - 1]  (eV)
* forces  F_i = -dE/dx_i
* stress  in the convention of the stress design rows (mld_stress.F90:540-752):
  S_ab = 3/V * sum_{i, n} (1/2) phi'(r) (u_a/r) * uu_b / r, with u = x_n - x_i and
  uu = u for a small box, uu = -u for a large box (sign_stress = sign_stress_big_box = 1), so
  that a model linear in the descriptors can represent it.
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional, Sequence, Tuple

import numpy as np

from .poscar import Structure

FE_A = 2.83
MORSE_FE = (0.4, 1.4, 2.5)  # D [eV], alpha [1/A], r0 [A]


def small_box(cell: np.ndarray, rcut: float) -> Tuple[bool, np.ndarray]:
    """neighbours.F90:787-847: small if int(2 r_c / width_i) + 1 > 1 for some i; image range."""
    bg = np.linalg.inv(cell).T  # rows b_i with a_i . b_k = delta
    widths = 1.0 / np.linalg.norm(bg, axis=1)
    ncell = (2.0 * rcut / widths).astype(int) + 1
    return bool((ncell > 1).any()), ncell // 2 + 1


def pair_list(pos: np.ndarray, cell: np.ndarray, rcut: float):
    """All (i, j, u) with u = x_j(image) - x_i, |u| < r_cut, in the reference's candidate order."""
    nat = pos.shape[0]
    sm, nsz = small_box(cell, rcut)
    if sm:
        rng = [np.arange(-n, n + 1) for n in nsz]
        img = np.stack(np.meshgrid(*rng, indexing="ij"), -1).reshape(-1, 3) @ cell  # (nimg, 3)
        # u[i, j, m] = x_j + img_m - x_i
        u = pos[None, :, None, :] + img[None, None, :, :] - pos[:, None, None, :]
        r2 = (u * u).sum(-1)
        ok = (r2 >= 1e-15) & (r2 <= rcut * rcut) & (np.sqrt(r2) < rcut)
        ii, jj, mm = np.nonzero(ok)
        return ii, jj, u[ii, jj, mm], True
    bg = np.linalg.inv(cell)  # columns b_k
    d = pos[None, :, :] - pos[:, None, :]
    ds = d @ bg
    ds = np.where(np.abs(ds) > 0.5, ds - np.round(ds), ds)
    u = ds @ cell
    r = np.sqrt((u * u).sum(-1))
    ok = r < rcut
    np.fill_diagonal(ok, False)
    ii, jj = np.nonzero(ok)
    return ii, jj, u[ii, jj], False


def morse_labels(pos: np.ndarray, cell: np.ndarray, types: np.ndarray, rcut: float,
                 table: Optional[np.ndarray] = None, params=MORSE_FE):
    """Energy, forces and stress (row convention) of a Morse pair potential."""
    ii, jj, u, sm = pair_list(pos, cell, rcut)
    r = np.sqrt((u * u).sum(-1))
    if table is None:
        Dm, al, r0 = (np.full(r.shape, p) for p in params)
    else:
        t = table[types[ii], types[jj]]
        Dm, al, r0 = t[:, 0], t[:, 1], t[:, 2]
    ex = np.exp(-al * (r - r0))
    phi = Dm * ((1.0 - ex) ** 2 - 1.0)
    dphi = 2.0 * Dm * al * ex * (1.0 - ex)
    E = 0.5 * phi.sum()
    fpair = (0.5 * dphi / r)[:, None] * u  # d(phi/2)/du for the (i, n) half-pair
    F = np.zeros_like(pos)
    np.add.at(F, ii, fpair)      # -dE/dx_i gets +phi'/2 u/r from each neighbour n of i
    np.add.at(F, jj, -fpair)
    vol = abs(np.linalg.det(cell))
    uu = u if sm else -u
    S6 = np.zeros(6)
    pairs = [(0, 0), (1, 1), (2, 2), (1, 2), (0, 2), (0, 1)]
    w = fpair / r[:, None]
    for k, (a, b) in enumerate(pairs):
        S6[k] = 3.0 / vol * (w[:, a] * uu[:, b]).sum()
    return E, F, S6


def bcc(n: int, m: int, k: int, a: float) -> Tuple[np.ndarray, np.ndarray]:
    base = np.array([[0.0, 0.0, 0.0], [0.5, 0.5, 0.5]])
    g = np.stack(np.meshgrid(np.arange(n), np.arange(m), np.arange(k), indexing="ij"), -1).reshape(-1, 3)
    sites = (g[:, None, :] + base[None, :, :]).reshape(-1, 3)   # in units of the cubic cell
    cell = np.diag([n * a, m * a, k * a])
    return sites * a, cell


def strain_cell(rng: np.random.Generator, cell: np.ndarray, amp: float) -> np.ndarray:
    e = rng.uniform(-amp, amp, size=(3, 3))
    e = 0.5 * (e + e.T)
    return cell @ (np.eye(3) + e)


def _dims_for(n_atoms: int) -> Tuple[int, int, int]:
    """Smallest near-cubic n x m x k (2 atoms per cell) holding n_atoms sites."""
    cells = max(1, math.ceil(n_atoms / 2))
    n = max(1, int(round(cells ** (1.0 / 3.0))) - 1)
    while True:
        for dims in ((n, n, n), (n, n, n + 1), (n, n + 1, n + 1), (n + 1, n + 1, n + 1)):
            if dims[0] * dims[1] * dims[2] >= cells:
                return dims
        n += 1


@dataclasses.dataclass
class Dataset:
    structures: List[Structure]
    rcut: float
    name: str

    def arrays(self):
        nat = np.array([s.nat for s in self.structures], np.int32)
        pos = np.concatenate([s.positions for s in self.structures])
        cell = np.stack([s.cell for s in self.structures])
        types = np.concatenate([s.types for s in self.structures]).astype(np.int32)
        return nat, pos, cell, types

    def labels(self, idx: Optional[Sequence[int]] = None):
        ss = self.structures if idx is None else [self.structures[i] for i in idx]
        E = np.array([s.energies[1] for s in ss])
        F = np.concatenate([s.forces for s in ss])
        S = np.stack([s.stress for s in ss])
        has = np.array([[s.has_energy, s.has_force, s.has_stress] for s in ss], np.int32)
        return E, F, S, has

    def n_rows(self) -> int:
        return sum(1 + 3 * s.nat + 6 for s in self.structures)


def fe_bcc_fixed(n_struct: int = 100, reps: int = 4, sigma: float = 0.05, strain: float = 0.01,
                 rcut: float = 4.7, seed: int = 20240601) -> Dataset:
    """Fe bcc a=2.83, reps^3 cubic supercell (128 atoms for reps=4), Gaussian noise, uniform strain."""
    rng = np.random.default_rng(seed)
    out = []
    for s in range(n_struct):
        pos, cell = bcc(reps, reps, reps, FE_A)
        cell2 = strain_cell(rng, cell, strain)
        pos = pos @ np.linalg.solve(cell, cell2)
        pos = pos + rng.normal(0.0, sigma, size=pos.shape)
        types = np.zeros(pos.shape[0], np.int32)
        E, F, S = morse_labels(pos, cell2, types, rcut)
        out.append(Structure(cell=cell2, positions=pos, types=types, elements=["Fe"],
                             energies=np.array([E, E, E]), forces=F, stress=S, name=f"fe_{s:05d}"))
    return Dataset(out, rcut, "fe_bcc_128x100")


def _batched_one(args):
    s, seed, nmin, nmax, sigma, strain, rcut, max_vac = args
    rng = np.random.default_rng(np.random.SeedSequence([seed, s]))
    N = int(round(math.exp(rng.uniform(math.log(nmin), math.log(nmax)))))
    nvac = int(rng.integers(0, max_vac + 1))
    n, m, k = _dims_for(N + nvac)
    pos, cell = bcc(n, m, k, FE_A)
    keep = np.sort(rng.choice(pos.shape[0], size=N, replace=False))
    pos = pos[keep]
    cell2 = strain_cell(rng, cell, strain)
    pos = pos @ np.linalg.solve(cell, cell2)
    pos = pos + rng.normal(0.0, sigma, size=pos.shape)
    types = np.zeros(N, np.int32)
    E, F, S = morse_labels(pos, cell2, types, rcut)
    return Structure(cell=cell2, positions=pos, types=types, elements=["Fe"],
                     energies=np.array([E, E, E]), forces=F, stress=S, name=f"feb_{s:05d}")


def fe_bcc_batched(n_struct: int = 2000, nmin: int = 16, nmax: int = 1024, sigma: float = 0.08,
                   strain: float = 0.02, rcut: float = 4.7, seed: int = 20240602,
                   max_vac: int = 3, workers: int = 0) -> Dataset:
    """Fe bcc supercells with log-uniform atom counts in [nmin, nmax], trimmed to size with
    0..max_vac extra vacancies.  Structure s draws from its own seeded stream, so the set does
    not depend on ``workers`` (0 = serial; >0 = that many spawned processes)."""
    jobs = [(s, seed, nmin, nmax, sigma, strain, rcut, max_vac) for s in range(n_struct)]
    if workers and workers > 1 and n_struct > 8:
        import concurrent.futures as cf
        import multiprocessing as mp
        with cf.ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn")) as ex:
            out = list(ex.map(_batched_one, jobs, chunksize=max(1, n_struct // (4 * workers))))
    else:
        out = [_batched_one(j) for j in jobs]
    return Dataset(out, rcut, f"fe_bcc_batched_{n_struct}")


# ---------------------------------------------------------------------------------------------
# 5-element equiatomic bcc alloy (quadratic-fit workload)
# ---------------------------------------------------------------------------------------------
HEA_ELEMENTS = ["Mo", "Nb", "Ta", "V", "Cr"]
HEA_A = 3.2
# weight_per_element of the weighted (two-channel) bispectrum: Z / 100
HEA_WEIGHTS = (0.42, 0.41, 0.73, 0.23, 0.24)


def hea_morse_table(seed: int = 20240603, r0: float = 2.75) -> np.ndarray:
    """Seeded symmetric element-pair Morse table (5 x 5 x (D, alpha, r0)): D in [0.3, 0.6] eV,
    alpha in [1.2, 1.6] 1/A, r0 at the bcc nearest-neighbour distance of a = 3.2 A."""
    rng = np.random.default_rng(seed)
    n = len(HEA_ELEMENTS)
    t = np.zeros((n, n, 3))
    for i in range(n):
        for j in range(i, n):
            t[i, j] = t[j, i] = (rng.uniform(0.3, 0.6), rng.uniform(1.2, 1.6), r0)
    return t


def _hea_one(args):
    s, seed, reps, sigma, rcut, table = args
    rng = np.random.default_rng(np.random.SeedSequence([seed, s]))
    pos, cell = bcc(reps, reps, reps, HEA_A)
    n = pos.shape[0]
    ne = len(HEA_ELEMENTS)
    types = rng.permutation(np.arange(n) % ne).astype(np.int32)   # equiatomic random occupation
    pos = pos + rng.normal(0.0, sigma, size=pos.shape)
    E, F, S = morse_labels(pos, cell, types, rcut, table=table)
    return Structure(cell=cell, positions=pos, types=types, elements=list(HEA_ELEMENTS),
                     energies=np.array([E, E, E]), forces=F, stress=S, name=f"hea_{s:05d}")


def hea_bcc_batched(n_struct: int = 4000, reps: int = 5, sigma: float = 0.1, rcut: float = 5.0,
                    seed: int = 20240604, workers: int = 0) -> Dataset:
    """(Mo, Nb, Ta, V, Cr) bcc a = 3.2 A, reps^3 cubic cells (250 atoms for reps = 5) with random
    equiatomic occupation, Gaussian noise sigma, labels from the seeded element-pair Morse table.
    Structure s draws from its own seeded stream (independent of ``workers``)."""
    table = hea_morse_table()
    jobs = [(s, seed, reps, sigma, rcut, table) for s in range(n_struct)]
    if workers and workers > 1 and n_struct > 8:
        import concurrent.futures as cf
        import multiprocessing as mp
        with cf.ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn")) as ex:
            out = list(ex.map(_hea_one, jobs, chunksize=max(1, n_struct // (4 * workers))))
    else:
        out = [_hea_one(j) for j in jobs]
    return Dataset(out, rcut, f"hea_bcc_{n_struct}")


def hea_request(rng: np.random.Generator, n_atoms: int, sigma: float = 0.1) -> Structure:
    """One serving request: a random 5-element bcc alloy cell of n_atoms atoms (a near-cubic
    supercell trimmed to size), Gaussian noise sigma; no labels."""
    n, m, k = _dims_for(n_atoms)
    pos, cell = bcc(n, m, k, HEA_A)
    keep = np.sort(rng.choice(pos.shape[0], size=n_atoms, replace=False))
    pos = pos[keep] + rng.normal(0.0, sigma, size=(n_atoms, 3))
    types = rng.integers(0, len(HEA_ELEMENTS), size=n_atoms).astype(np.int32)
    return Structure(cell=cell, positions=pos, types=types, elements=list(HEA_ELEMENTS),
                     energies=np.zeros(3), forces=np.zeros((n_atoms, 3)), stress=np.zeros(6), name="req")
