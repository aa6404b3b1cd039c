"""Element data the descriptor path needs: atomic number, mass and covalent radius.

Values are those of the reference's periodic table (ml_in_ndm_module.F90:1675-2343 masses,
:2656-2729 covalent radii in pm).  The reference assigns the masses from default-kind (single
precision) literals into double-precision fields, so the value it computes with is the
binary32 rounding of the printed number; `mass()` returns that value.
"""
from __future__ import annotations

from typing import Dict, Sequence, Tuple

import numpy as np

# symbol: (Z, mass as printed, covalent radius [pm])
TABLE: Dict[str, Tuple[int, float, float]] = {
    "H": (1, 1.008, 79.0), "Li": (3, 6.941, 155.0), "C": (6, 12.011, 91.0), "Al": (13, 26.982, 143.0),
    "Si": (14, 28.086, 132.0), "Ti": (22, 47.867, 147.0), "V": (23, 50.942, 134.0), "Cr": (24, 51.996, 130.0),
    "Mn": (25, 54.938, 135.0), "Fe": (26, 55.845, 126.0), "Co": (27, 58.933, 125.0), "Ni": (28, 58.693, 124.0),
    "Cu": (29, 63.546, 128.0), "Zr": (40, 91.224, 160.0), "Nb": (41, 92.906, 146.0), "Mo": (42, 95.940, 139.0),
    "Hf": (72, 178.490, 167.0), "Ta": (73, 180.948, 149.0), "W": (74, 183.840, 141.0), "Re": (75, 186.207, 137.0),
}


def atomic_number(sym: str) -> int:
    return TABLE[sym][0]


def mass(sym: str) -> float:
    return float(np.float32(TABLE[sym][1]))


def covalent_radius(sym: str) -> float:
    return TABLE[sym][2]


def auto_channel_weights(symbols: Sequence[str]) -> Tuple[np.ndarray, np.ndarray]:
    """Per-element weights of the second and third bispectrum channels with ``weighted_auto``:
    channel 2 starts from Z and channel 3 from mass^2 + covalent_radius^2 (read_ml_file.F90:
    1640-1680); fix_poscar_weights (build_subdata.F90:2964-2988) then divides channel 2 by the
    root mean square and channel 3 by the mean over the element list."""
    z = np.array([atomic_number(s) for s in symbols], dtype=np.float64)
    m = np.array([mass(s) for s in symbols], dtype=np.float64)
    rc = np.array([covalent_radius(s) for s in symbols], dtype=np.float64)
    w2 = z / np.sqrt(np.sum(z * z) / z.size)
    w3 = m * m + rc * rc
    return w2, w3 / (np.sum(w3) / w3.size)
