"""Build tests/golden/fit17_bso4.npz from MILADY's own regression test fit17.

fit17 (tests/train_tests/fit17 in the MILADY project) computes bispectrum-SO(4) descriptors
(descriptor_type=9, j_max=4, r_cut=4.7, unweighted, tungsten) for 20 POSCAR files selected by
its db_model.in and writes the reference's per-atom B to REF/descDB/<name>.eml (column 1 = the
1-based atom index, columns 2..56 = B_1..B_55, format es30.18e3).  This script packs, per structure,
the cell, positions, types and the reference's B into one compressed fixture so the tests can
run where the MILADY sources are absent.

Usage:  python tests/golden/make_fit17_fixture.py [/path/to/MILADY]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from mld_gb300.poscar import read_poscar  # noqa: E402


def main(root: str) -> None:
    t = os.path.join(root, "tests", "train_tests", "fit17")
    names = []
    with open(os.path.join(t, "REF", "train_files.milady")) as fh:
        for line in fh:
            if line.strip():
                names.append(os.path.basename(line.split()[0]).replace(".poscar", ""))
    out = {"names": np.array(names)}
    for i, n in enumerate(names):
        s = read_poscar(os.path.join(t, "DB", n + ".poscar"), want_forces=False)
        ref = np.loadtxt(os.path.join(t, "REF", "descDB", n + ".eml"), ndmin=2)
        assert ref.shape[0] == s.nat, (n, ref.shape, s.nat)
        out[f"cell_{i}"] = s.cell
        out[f"pos_{i}"] = s.positions
        out[f"types_{i}"] = s.types
        out[f"B_{i}"] = ref[:, 1:]
        out[f"tag_{i}"] = ref[:, 0]
    out["r_cut"] = np.array(4.7)
    out["j_max"] = np.array(4.0)
    np.savez_compressed(os.path.join(HERE, "fit17_bso4.npz"), **out)
    print("wrote", len(names), "structures")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {os.path.basename(__file__)} <path of the MILADY source tree>")
    main(sys.argv[1])
