"""Copy a few of MILADY's own parameter and descriptor files into tests/golden/files/.

The reference's regression tests keep the files its fits write:
  * fit03 (W, quadratic QNML, j_max=2, r_cut=4.7): bso4_qnml1_params.pot + lammps_bso4_qnml1_params.pot
  * fit08 (Ta-Ti-V-W, three-channel weighted, linear, j_max=4, r_cut=5): bso4_snap1_params.pot + lammps_...
  * fit13 (W, linear, j_max=4, r_cut=5): bso4_snap1_params.pot + lammps_...
  * fit17 (W, descriptor dump): REF/descDB/12_111_000005.eml (1 atom) and 02_111_000001.eml (12 atoms)
The tests read each file and write it back with mld_gb300.potfile, requiring identical bytes.

Usage:  python tests/golden/make_file_fixtures.py [/path/to/MILADY]
"""
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
FILES = [
    ("fit03", "bso4_qnml1_params.pot"), ("fit03", "lammps_bso4_qnml1_params.pot"),
    ("fit08", "bso4_snap1_params.pot"), ("fit08", "lammps_bso4_snap1_params.pot"),
    ("fit13", "bso4_snap1_params.pot"), ("fit13", "lammps_bso4_snap1_params.pot"),
    ("fit17", "REF/descDB/12_111_000005.eml"), ("fit17", "REF/descDB/02_111_000001.eml"),
]


def main(root: str) -> None:
    out = os.path.join(HERE, "files")
    os.makedirs(out, exist_ok=True)
    for fit, name in FILES:
        src = os.path.join(root, "tests", "train_tests", fit, name)
        dst = os.path.join(out, f"{fit}_{os.path.basename(name)}")
        shutil.copyfile(src, dst)
        print(dst, os.path.getsize(dst))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {os.path.basename(__file__)} <path of the MILADY source tree>")
    main(sys.argv[1])
