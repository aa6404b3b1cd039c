"""Build tests/golden/db_selection.json from MILADY's regression tests.

For each listed test directory (tests/train_tests/<fitNN> in the MILADY project) it stores the
db_model.in lines, the selection_type/seed of its namelist and the reference's own
REF/train_files.milady and REF/test_files.milady lists (file names in selection order), so the
db_model selection can be checked where the MILADY sources are absent.

Usage:  python tests/golden/make_db_fixture.py [/path/to/MILADY]
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
TESTS = ["fit01", "fit08", "fit13", "fit17"]


def names(path):
    if not os.path.exists(path):
        return []
    return [os.path.basename(l.split()[0]) for l in open(path) if l.strip()]


def main(root):
    out = {}
    for t in TESTS:
        d = os.path.join(root, "tests", "train_tests", t)
        ml = [f for f in os.listdir(d) if f.endswith(".ml") and not f.startswith("old")]
        txt = open(os.path.join(d, sorted(ml)[0]), "rb").read().decode("latin-1")
        def get(key, default):
            m = re.search(r"^\s*" + key + r"\s*=\s*([^!\s,]+)", txt, flags=re.M | re.I)
            return int(m.group(1)) if m else default
        out[t] = {"db_model": open(os.path.join(d, "db_model.in")).read(),
                  "selection_type": get("selection_type", 3), "seed": get("seed", 14792435),
                  "train": names(os.path.join(d, "REF", "train_files.milady")),
                  "test": names(os.path.join(d, "REF", "test_files.milady"))}
    json.dump(out, open(os.path.join(HERE, "db_selection.json"), "w"), indent=1)
    print("wrote", list(out))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {os.path.basename(__file__)} <path of the MILADY source tree>")
    main(sys.argv[1])
