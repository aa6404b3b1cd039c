"""Reader of MILADY's ``&input_ml`` namelist (the subset the descriptor-to-fit path uses).

Defaults follow src/mld/read_ml_file.F90:307-611; legacy ``snap_*`` aliases map onto the
``mld_*`` names as in read_ml_file.F90:664-691.  Values are parsed with Fortran list-directed
conventions: ``.true./.false./T/F``, ``1.d-8`` exponents, quoted strings, ``!`` comments.
"""
from __future__ import annotations

import math
import re
from typing import Any, Dict

DEFAULTS: Dict[str, Any] = {
    "ml_type": 0,
    "descriptor_type": 1,
    "j_max": 1.5,
    "r_cut": 5.0,
    "inv_r0_input": 1.0 - 0.02 / math.pi,
    "lambda_krr": -1.0,
    "svd_rcond": -1.0,
    "mld_fit_type": 4,
    "mld_order": 1,
    "mld_type_quadratic": 1,
    "kernel_type": 4,
    "kernel_power": 2.0,
    "length_kernel": math.sqrt(0.5),
    "sigma_kernel": 0.0,
    "np_kernel_ref": 200,
    "np_kernel_full": 800,
    "kernel_dump": 1,
    "classes_for_mcd": " 01 02",
    "cur_kval": -1,
    "cur_rval": -1,
    "cur_cval": -1,
    "cur_eps": 1.0,
    "seed": 14792435,
    "selection_type": 3,
    "iread_energy": 2,
    "desc_forces": False,
    "weighted": False,
    "weighted_3ch": False,
    "weighted_auto": False,
    "chemical_elements": "",
    "weight_per_element": "",
    "weight_per_element_3ch": "",
    "fix_no_of_elements": 0,
    "sign_stress": 1.0,
    "sign_stress_big_box": 1.0,
    "factor_energy_error": 1.0,
    "factor_force_error": 1.0,
    "factor_stress_error": 1.0,
    "type_of_loss": 1,
    "r_cut_width_in": 0.4,
    "db_file": "db_model.in",
    "db_path": "DB/",
    "write_desc": False,
    "train_only": False,
}

ALIASES = {"snap_order": "mld_order", "snap_type_quadratic": "mld_type_quadratic", "snap_fit_type": "mld_fit_type"}


def _value(tok: str):
    t = tok.strip()
    if not t:
        return t
    if t[0] in "'\"":
        return t.strip("'\"")
    low = t.lower()
    if low in (".true.", "t", ".t.", "true"):
        return True
    if low in (".false.", "f", ".f.", "false"):
        return False
    try:
        return int(t)
    except ValueError:
        pass
    try:
        return float(low.replace("d", "e"))
    except ValueError:
        return t


def read_input_ml(path: str) -> Dict[str, Any]:
    """Parse ``&input_ml ... &end`` (or ``/``) from ``path`` into a dict over DEFAULTS."""
    with open(path, "rb") as fh:
        text = fh.read().decode("latin-1")
    m = re.search(r"&input_ml(.*?)(?:&end|^\s*/\s*$)", text, flags=re.S | re.I | re.M)
    if not m:
        raise ValueError(f"{path}: no &input_ml group")
    body = m.group(1)
    out = dict(DEFAULTS)
    for raw in body.splitlines():
        line = raw
        # strip comments outside quotes
        q = None
        for i, ch in enumerate(line):
            if ch in "'\"":
                q = None if q == ch else (ch if q is None else q)
            elif ch == "!" and q is None:
                line = line[:i]
                break
        for part in re.finditer(r"(\w+)\s*=\s*('[^']*'|\"[^\"]*\"|[^,\s]+)", line):
            key = part.group(1).lower()
            key = ALIASES.get(key, key)
            out[key] = _value(part.group(2))
    # read_ml_file.F90:332 / parameters.F90:1089: lambda_krr < 0 means no ridge
    return out


def elements(nl: Dict[str, Any]):
    return [e for e in str(nl.get("chemical_elements", "")).split() if e]


def element_weights(nl: Dict[str, Any], key: str = "weight_per_element"):
    ws = [float(str(x).replace("d", "e").replace("D", "e")) for x in str(nl.get(key, "")).split()]
    n = len(elements(nl))
    if not ws:
        ws = [1.0] * n
    return ws
