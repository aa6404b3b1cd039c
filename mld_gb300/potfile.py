"""Potential and descriptor files in the reference's formats, so that GPU-fitted potentials drop
into the reference's tooling and LAMMPS `pair_style milady`.

* MILADY parameter file ``<desc>_<model>_params.pot``: the number of parameters (I12), then one
  weight per line (ES25.15E3) -- module_write_parameters.F90:764-1000 (write_snap_parameters),
  read back by mld.F90:1876-1952.
* LAMMPS parameter file ``lammps_<...>.pot``: six comment lines, then
  ``(I7,I7)`` channels and elements followed on the same line by ``(A4,3E20.10)`` per element
  (symbol, channel-2 weight, channel-3 weight or 1, reference energy), ``(I4,I12,I4)``
  descriptor type / number of parameters / number of detail fields, the masses ``(nF20.4)``,
  the bispectrum details ``(I5,F5.1,2I4)`` (mld_order, j_max, diagonal flag, active patches),
  r_cut ``(F20.4)`` and the weights (ES25.15E3).
* Descriptor dump ``desc<db_path><class>_<klm>_<cnumber>.eml`` (ml_type = -1): per atom
  ``(ES30.18E3, 1X, n ES30.18E3)`` with the 1-based atom index and the descriptor --
  read_write_descriptors.F90:165-190.

Formats are reproduced byte for byte (tests compare against the reference's own files).
"""
from __future__ import annotations

import os
from typing import Dict, Optional, Sequence, Tuple

import numpy as np

from . import elements as elements_table



def _es(v: float, width: int, digits: int, expd: int = 3) -> str:
    """Fortran ESw.dEe: one digit before the point, `digits` after, an exponent of `expd` digits.
    Python's e-format rounds the exact binary value, as gfortran's formatted output does."""
    m, ex = f"{float(v):.{digits}e}".split("e")
    ex = int(ex)
    return f"{m}E{'+' if ex >= 0 else '-'}{abs(ex):0{expd}d}".rjust(width)


def _e(v: float, width: int, digits: int) -> str:
    """Fortran Ew.d: 0.dddE+nn with `digits` significant digits (zero prints with exponent +00)."""
    v = float(v)
    if v == 0.0:
        return ("0." + "0" * digits + "E+00").rjust(width)
    m, ex = f"{v:.{digits - 1}e}".split("e")
    ex = int(ex) + 1
    sign = "-" if m.startswith("-") else ""
    mant = m.lstrip("-").replace(".", "")
    return f"{sign}0.{mant}E{'+' if ex >= 0 else '-'}{abs(ex):02d}".rjust(width)


def write_milady_pot(path: str, w: Sequence[float]) -> None:
    w = np.asarray(w, dtype=np.float64).reshape(-1)
    with open(path, "w") as f:
        f.write(f"{w.shape[0]:12d}\n")
        for v in w:
            f.write(_es(v, 25, 15) + "\n")


def read_milady_pot(path: str) -> np.ndarray:
    with open(path) as f:
        tok = f.read().split()
    n = int(tok[0])
    return np.array([float(t) for t in tok[1:1 + n]])


_LAMMPS_COMMENTS = [
    "# nchannels nelements element_1 weight_1_for_el_1 weight_2_for_el_1 element_2 weight_1_for_el_2 "
    "weight_2_for_el_2 ... etc ",
    "# descriptor type, nparameters_descriptor, ndetails",
    "# mass_1 mass_2 ... mass_nelements",
    "# detail_1 is the mld_order, ..., detail_ndetails (e.g. mld_order no_of_radial_channels no_of_angular_channels)",
    "# r_cut only one for all descriptors",
    "# w_i  with i=1, dim_xdesc, dim_xdesc +1 ...  (nchannel-1)*dim_xdesc ... nchannel*dim_xdesc",
]


MLD_LINEAR, MLD_QUADRATIC, MLD_POLYC, MLD_KERNEL = 1, 2, 3, 7
KERNEL_PO = 4
MODEL_TAG = {MLD_LINEAR: "snap1", MLD_QUADRATIC: "qnml1", MLD_POLYC: "polyc", MLD_KERNEL: "kernl"}


def write_lammps_pot(path: str, w: Sequence[float], elements: Sequence[str], *, j_max: float, r_cut: float,
                     mld_order: int = 1, nchannels: int = 1, weights: Optional[Sequence[float]] = None,
                     weights_3ch: Optional[Sequence[float]] = None, ref_energy: Optional[Sequence[float]] = None,
                     masses: Optional[Sequence[float]] = None, descriptor_type: int = 9, diagonal: int = 0,
                     active_patch: int = 0, kernel_points: Optional[np.ndarray] = None,
                     kernel_type: int = KERNEL_PO, sigma_kernel: float = 0.0, length_kernel: float = 0.0,
                     kernel_power: float = 0.0) -> None:
    """The LAMMPS parameter file (module_write_parameters.F90:870-1085, :1186-1530).  For the kernel
    model (mld_order 7) `kernel_points` holds the standardised reference points (nk x dim_xdesc);
    they follow the weights, then sigma, length and power (E25.15) for the polynomial kernel."""
    w = np.asarray(w, dtype=np.float64).reshape(-1)
    kernel = mld_order == MLD_KERNEL
    if kernel:
        if kernel_points is None:
            raise ValueError("the kernel model needs its reference points")
        kernel_points = np.asarray(kernel_points, dtype=np.float64)
        nk, dim_x = kernel_points.shape
        if kernel_type != KERNEL_PO:
            raise ValueError("only the polynomial kernel (kernel_type 4) is written")
    ne = len(elements)
    wt = list(weights) if weights is not None else [1.0] * ne
    w3 = list(weights_3ch) if weights_3ch is not None else [1.0] * ne
    er = list(ref_energy) if ref_energy is not None else [0.0] * ne
    ms = list(masses) if masses is not None else [elements_table.mass(e) for e in elements]
    with open(path, "w") as f:
        for c in _LAMMPS_COMMENTS:
            f.write(c + "\n")
        line = f"{nchannels:7d}{ne:7d}"
        for i, el in enumerate(elements):
            line += el.ljust(2).rjust(4) + _e(wt[i], 20, 10) + _e(w3[i] if nchannels == 3 else 1.0, 20, 10) + \
                _e(er[i], 20, 10)
        f.write(line + "\n")
        npar = w.shape[0] + (nk * dim_x + 3 if kernel else 0)
        f.write(f"{descriptor_type:4d}{npar:12d}{4 + 3 if kernel else 4:4d}\n")
        f.write("".join(f"{m:20.4f}" for m in ms) + "\n")
        if kernel:
            f.write(f"{mld_order:5d}{j_max:5.1f}{diagonal:4d}{active_patch:6d}{kernel_type:6d}{dim_x:6d}{nk:6d}\n")
        else:
            f.write(f"{mld_order:5d}{j_max:5.1f}{diagonal:4d}{active_patch:4d}\n")
        f.write(f"{r_cut:20.4f}\n")
        for v in w:
            f.write(_es(v, 25, 15) + "\n")
        if kernel:
            for v in kernel_points.reshape(-1):
                f.write(_es(v, 25, 15) + "\n")
            for v in (sigma_kernel, length_kernel, kernel_power):
                f.write(_e(v, 25, 15) + "\n")


def read_lammps_pot(path: str) -> Dict[str, object]:
    with open(path) as f:
        lines = [l for l in f.read().split("\n") if not l.startswith("#")]
    head = lines[0]
    nch, ne = int(head[0:7]), int(head[7:14])
    els, wts, w3, er = [], [], [], []
    pos = 14
    for _ in range(ne):
        els.append(head[pos:pos + 4].strip())
        wts.append(float(head[pos + 4:pos + 24]))
        w3.append(float(head[pos + 24:pos + 44]))
        er.append(float(head[pos + 44:pos + 64]))
        pos += 64
    dtype, npar, ndet = (int(t) for t in lines[1].split())
    masses = [float(t) for t in lines[2].split()]
    det = lines[3].split()
    r_cut = float(lines[4])
    vals = np.array([float(t) for l in lines[5:] for t in l.split()])
    out = {"nchannels": nch, "elements": els, "weights": wts, "weights_3ch": w3, "ref_energy": er,
           "descriptor_type": dtype, "ndetails": ndet, "masses": masses, "mld_order": int(det[0]),
           "j_max": float(det[1]), "details": det, "r_cut": r_cut}
    if dtype == 9 and int(det[0]) == MLD_KERNEL:
        ktype, dim_x, nk = int(det[4]), int(det[5]), int(det[6])
        nw = npar - nk * dim_x - 3
        out.update(w=vals[:nw], kernel_type=ktype, kernel_points=vals[nw:nw + nk * dim_x].reshape(nk, dim_x),
                   sigma_kernel=vals[npar - 3], length_kernel=vals[npar - 2], kernel_power=vals[npar - 1])
    else:
        out["w"] = vals[:npar]
    return out


def write_potential(directory: str, w: Sequence[float], elements: Sequence[str], *, j_max: float, r_cut: float,
                    mld_order: int = MLD_LINEAR, descriptor_tag: str = "bso4", **lammps) -> Tuple[str, str]:
    """Both parameter files of a fitted model, named as the reference names them
    (module_write_parameters.F90:762-780): ``<desc>_<model>_params.pot`` and ``lammps_<...>``."""
    base = f"{descriptor_tag}_{MODEL_TAG[mld_order]}_params.pot"
    p_mld, p_lmp = os.path.join(directory, base), os.path.join(directory, "lammps_" + base)
    write_milady_pot(p_mld, w)
    write_lammps_pot(p_lmp, w, elements, j_max=j_max, r_cut=r_cut, mld_order=mld_order, **lammps)
    return p_mld, p_lmp


def write_eml(path: str, B: np.ndarray, first_atom: int = 1, append: bool = False) -> None:
    """Descriptor dump of one configuration: one line per atom, the 1-based atom index (as a real)
    then the descriptor components (read_write_descriptors.F90:165-190; the reference appends when
    the file exists, for configurations written in atom ranges)."""
    B = np.asarray(B, dtype=np.float64)
    if B.ndim == 1:
        B = B[None, :]
    with open(path, "a" if append else "w") as f:
        for i, row in enumerate(B):
            f.write(_es(float(first_atom + i), 30, 18) + " " + "".join(_es(v, 30, 18) for v in row) + "\n")


def read_eml(path: str):
    """(atom indices, descriptors) of a descriptor dump."""
    data = np.loadtxt(path, ndmin=2)
    return data[:, 0].astype(np.int64), data[:, 1:]


def write_kernel_matrix(path: str, points: np.ndarray, iconf: Sequence[int], iatom: Sequence[int],
                        names: Sequence[str]) -> None:
    """``kernel_matrix.dat``: the raw descriptors of the kernel's reference atoms
    (module_write_parameters.F90:1585-1600): a ``(2I9)`` header (count, dim + 4), then per point
    ``(I6, n E20.10, I6, I6, A15)`` = index, descriptor, configuration, atom, ``"  <class>_<klm>_<n>"``."""
    P = np.asarray(points, dtype=np.float64)
    with open(path, "w") as f:
        f.write(f"{P.shape[0]:9d}{P.shape[1] + 4:9d}\n")
        for k, row in enumerate(P):
            tag = ("  " + names[k])[:15].ljust(15)
            f.write(f"{k + 1:6d}" + "".join(_e(v, 20, 10) for v in row) + f"{iconf[k]:6d}{iatom[k]:6d}" + tag + "\n")


def read_kernel_matrix(path: str) -> np.ndarray:
    """Points of ``kernel_matrix.dat`` (compute_kernel.F90:1106-1160), ordered by their index."""
    with open(path) as f:
        nk, dim4 = (int(t) for t in f.readline().split()[:2])
        dim = dim4 - 4
        P = np.zeros((nk, dim))
        for _ in range(nk):
            line = f.readline()
            k = int(line[:6])
            P[k - 1] = [float(line[6 + 20 * i:26 + 20 * i]) for i in range(dim)]
    return P
