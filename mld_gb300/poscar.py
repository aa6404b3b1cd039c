"""MILADY-flavoured POSCAR reader/writer.

Mirrors ``read_poscar_sasha`` (MILADY src/mld/build_subdata.F90:2484-2952):

* line 1: ``EFS nb_el (symbol mass)*nb_el E_total E_fit1 E_fit2`` where ``EFS`` is a
  3-character flag string ("111" = has energy, force, stress);
* line 2: lattice scale ``alat``; lines 3-5: lattice vectors (one per line), scaled by alat;
* optional VASP-5 species line, then per-species counts;
* ``Cartesian``/``Direct`` line, then positions (Cartesian positions are NOT wrapped);
* when forces are wanted: a blank line then nat force lines, a blank line then the
  6-component stress (xx yy zz yz xz xy).

Energies are stored as in the reference: ``energy[k] = E_k - sum of reference energies
per element`` (build_subdata.F90:2905-2914); ``iread_energy=2`` selects ``E_fit1``.
"""
from __future__ import annotations

import dataclasses
from typing import List, Optional, Sequence

import numpy as np


@dataclasses.dataclass
class Structure:
    """One atomic configuration in the reference's units (Angstrom, eV)."""

    cell: np.ndarray                 # (3, 3): cell[i] = lattice vector a_i
    positions: np.ndarray            # (nat, 3) Cartesian
    types: np.ndarray                # (nat,) 0-based index into ``elements``
    elements: List[str]
    energies: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(3))  # E_total, E_fit1, E_fit2 (raw)
    forces: Optional[np.ndarray] = None   # (nat, 3)
    stress: Optional[np.ndarray] = None   # (6,)
    has_energy: bool = True
    has_force: bool = True
    has_stress: bool = True
    name: str = ""

    @property
    def nat(self) -> int:
        return int(self.positions.shape[0])

    def volume(self) -> float:
        return float(abs(np.linalg.det(self.cell)))


def _is_number(tok: str) -> bool:
    try:
        float(tok.replace("d", "e").replace("D", "e"))
        return True
    except ValueError:
        return False


def _f(tok: str) -> float:
    return float(tok.replace("d", "e").replace("D", "e"))


def read_poscar(path: str, want_forces: bool = True) -> Structure:
    with open(path) as fh:
        lines = fh.read().splitlines()
    it = iter(lines)
    head = next(it).split()
    efs = head[0]
    nb = int(head[1])
    elements = [head[2 + 2 * i] for i in range(nb)]
    rest = head[2 + 2 * nb:]
    energies = np.array([_f(t) for t in rest[:3]] + [0.0] * max(0, 3 - len(rest)), dtype=np.float64)
    alat = _f(next(it).split()[0])
    cell = np.array([[_f(t) for t in next(it).split()[:3]] for _ in range(3)], dtype=np.float64) * alat
    line = next(it)
    toks = line.split()
    if not _is_number(toks[0]):
        if toks[:nb] != elements:
            raise ValueError(f"{path}: species line {toks} disagrees with header {elements}")
        line = next(it)
        toks = line.split()
    counts = [int(t) for t in toks[:nb]]
    if len(counts) != nb:
        raise ValueError(f"{path}: expected {nb} species counts")
    mode = next(it).strip()
    if not mode or mode[0] not in "cCdD":
        raise ValueError(f"{path}: coordinate mode line must start with C or D, got {mode!r}")
    nat = sum(counts)
    xc = np.array([[_f(t) for t in next(it).split()[:3]] for _ in range(nat)], dtype=np.float64)
    types = np.concatenate([np.full(c, i, dtype=np.int32) for i, c in enumerate(counts)])
    if mode[0] in "dD":
        pos = xc @ cell
    else:
        pos = xc
    forces = None
    stress = None
    if want_forces:
        rem = [l for l in it]
        # blank line, nat force lines, blank, stress line (read with list-directed semantics)
        k = 0
        while k < len(rem) and rem[k].strip() == "":
            k += 1
        try:
            forces = np.array([[_f(t) for t in rem[k + i].split()[:3]] for i in range(nat)], dtype=np.float64)
            k += nat
            while k < len(rem) and rem[k].strip() == "":
                k += 1
            stress = np.array([_f(t) for t in rem[k].split()[:6]], dtype=np.float64)
        except (IndexError, ValueError):
            forces = np.zeros((nat, 3))
            stress = np.zeros(6)
    return Structure(cell=cell, positions=pos, types=types, elements=elements, energies=energies,
                     forces=forces, stress=stress, has_energy=efs[0] == "1",
                     has_force=len(efs) > 1 and efs[1] == "1",
                     has_stress=len(efs) > 2 and efs[2] == "1", name=path)


def write_poscar(path: str, s: Structure, masses: Optional[Sequence[float]] = None) -> None:
    """Write ``s`` in the same layout ``read_poscar`` (and the reference) parses."""
    efs = "".join("1" if f else "0" for f in (s.has_energy, s.has_force, s.has_stress))
    nb = len(s.elements)
    masses = list(masses) if masses is not None else [1] * nb
    head = [efs, str(nb)]
    for e, m in zip(s.elements, masses):
        head += [e, str(int(m))]
    head += ["%.12f" % v for v in s.energies[:3]]
    out = [" ".join(head), " 1.0000000000000000"]
    for v in s.cell:
        out.append("  %.16f  %.16f  %.16f" % tuple(v))
    order = np.argsort(s.types, kind="stable")
    counts = [int((s.types == i).sum()) for i in range(nb)]
    out.append(" ".join(s.elements))
    out.append(" ".join(str(c) for c in counts))
    out.append("Cartesian")
    for i in order:
        out.append("  %.16f  %.16f  %.16f" % tuple(s.positions[i]))
    out.append("")
    f = s.forces if s.forces is not None else np.zeros((s.nat, 3))
    for i in order:
        out.append("  %.16f  %.16f  %.16f" % tuple(f[i]))
    out.append("")
    st = s.stress if s.stress is not None else np.zeros(6)
    out.append("  " + "  ".join("%.16f" % v for v in st))
    out.append("")
    with open(path, "w") as fh:
        fh.write("\n".join(out))
