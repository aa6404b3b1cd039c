"""Build tests/golden/fit19_bso4_3ch.npz from MILADY's regression test fit19.

fit19 (tests/train_tests/fit19 in the MILADY project) writes three-channel weighted
bispectrum-SO(4) descriptors (descriptor_type=9, j_max=4, r_cut=4.7, weighted + weighted_3ch +
weighted_auto, elements Ta Ti V W) to REF/descDB/<name>.eml: column 1 = the 1-based atom index,
columns 2..166 = the 3 x 55 components (unweighted channel, then the two weighted channels),
format es30.18e3.  This script packs three of the structures (a 128-atom relaxed cell and two
100/112-atom molten snapshots), with types mapped to the namelist's element order, so the tests
can run where the MILADY sources are absent.

Usage:  python tests/golden/make_fit19_fixture.py [/path/to/MILADY]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from mld_gb300.poscar import read_poscar  # noqa: E402

NAMES = ["00_001_000001", "28_001_000001", "29_001_000001"]
ELEMENTS = ["Ta", "Ti", "V", "W"]


def main(root: str) -> None:
    t = os.path.join(root, "tests", "train_tests", "fit19")
    out = {"names": np.array(NAMES), "elements": np.array(ELEMENTS)}
    for i, n in enumerate(NAMES):
        s = read_poscar(os.path.join(t, "DB", n + ".poscar"), want_forces=False)
        m = np.array([ELEMENTS.index(e) for e in s.elements], np.int32)
        ref = np.loadtxt(os.path.join(t, "REF", "descDB", n + ".eml"), ndmin=2)
        assert ref.shape == (s.nat, 1 + 165), (n, ref.shape, s.nat)
        out[f"cell_{i}"] = s.cell
        out[f"pos_{i}"] = s.positions
        out[f"types_{i}"] = m[s.types]
        out[f"B_{i}"] = ref[:, 1:]
    out["r_cut"] = np.array(4.7)
    out["j_max"] = np.array(4.0)
    np.savez_compressed(os.path.join(HERE, "fit19_bso4_3ch.npz"), **out)
    print("wrote", len(NAMES), "structures")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {os.path.basename(__file__)} <path of the MILADY source tree>")
    main(sys.argv[1])
