"""``db_model.in`` reader and the seeded train/test selection of MILADY.

* Line format (build_subdata.F90:1720-1882): ``class klm no_total no_selec E F S w_e w_f w_s``
  (``no_start`` precedes the flags for selection_type=4); ``#`` lines are comments.
* Selection (build_subdata.F90:1884-2110): per line, files ``<class>_<klm>_<nnnnnn>.poscar``;
  selection_type 1 = first no_selec, 2 = last no_selec, 3 = random (``seed`` is incremented
  once per db line, then ``rks2`` draws no_selec of no_total), 4 = first from no_start.
  Selected files are training configurations, the remaining ones test configurations.
* ``rks2`` is the sequential random k-subset algorithm (Bratley, Fox & Schrage) driven by the
  Park-Miller minimal-standard generator seed <- 16807*seed mod (2^31-1), r = seed/(2^31-1),
  evaluated with Schrage's factorisation so that the 32-bit integer arithmetic is exact.
* Per-configuration weights (main_train_regularization.F90:336-390): with type_of_loss=1
  (``loss_init``) w_e_model = w_e * factor_energy_error, and alike for forces and stress.
"""
from __future__ import annotations

import dataclasses
import os
from typing import List, Tuple


@dataclasses.dataclass
class DbLine:
    cls: str
    klm: str
    no_total: int
    no_selec: int
    no_start: int
    has_e: bool
    has_f: bool
    has_s: bool
    w_e: float
    w_f: float
    w_s: float


@dataclasses.dataclass
class Config:
    filename: str
    train: bool
    line: int
    w_e: float
    w_f: float
    w_s: float
    has_e: bool
    has_f: bool
    has_s: bool


def _flag(c: str) -> bool:
    if c in ("T", "t"):
        return True
    if c in ("F", "f"):
        return False
    raise ValueError(f"db_model flag must be T or F, got {c!r}")


def read_db_model(path: str, selection_type: int = 3) -> List[DbLine]:
    out = []
    with open(path) as fh:
        for raw in fh:
            if not raw.strip() or raw.lstrip().startswith("#"):
                continue
            t = raw.split()
            if selection_type == 4:
                cls, klm, tot, sel, start, c1, c2, c3 = t[:8]
                w = t[8:11]
            else:
                cls, klm, tot, sel, c1, c2, c3 = t[:7]
                start = 1
                w = t[7:10]
            w = [float(x.replace("d", "e").replace("D", "e")) for x in w]
            line = DbLine(cls, klm, int(tot), int(sel), int(start), _flag(c1), _flag(c2), _flag(c3), *w)
            if line.no_total < line.no_selec + line.no_start - 1:
                raise ValueError("no_total smaller than the selection in " + raw.strip())
            out.append(line)
    return out


def r8_uniform_01(seed: int) -> Tuple[float, int]:
    """Park-Miller minimal standard step (Schrage's method); returns (r, new_seed)."""
    k = seed // 127773
    seed = 16807 * (seed - k * 127773) - k * 2836
    if seed < 0:
        seed += 2147483647
    return seed * 4.656612875e-10, seed


def rks2(n: int, k: int, seed: int) -> Tuple[List[int], int]:
    """Random k-subset of 1..n in increasing order; returns (subset, new_seed)."""
    if k < 0 or n < k:
        raise ValueError("0 <= k <= n required")
    a: List[int] = []
    if k == 0:
        return a, seed
    c1, c2 = k, n
    for i in range(1, n + 1):
        r, seed = r8_uniform_01(seed)
        if float(c2) * r <= float(c1):
            c1 -= 1
            a.append(i)
            if c1 <= 0:
                break
        c2 -= 1
    return a, seed


def select(lines: List[DbLine], selection_type: int = 3, seed: int = 14792435, db_path: str = "DB/",
           factors=(1.0, 1.0, 1.0)) -> List[Config]:
    """Train configurations first per db line (in selection order), then that line's test ones
    (the ordering of prepare_name_file_from_db)."""
    out: List[Config] = []
    for li, d in enumerate(lines):
        anum = None
        if selection_type == 3:
            seed += 1
            anum, _ = rks2(d.no_total, d.no_selec, seed)
        chosen = []
        for ic in range(d.no_start, d.no_selec + d.no_start):
            if selection_type in (1, 4):
                fn = ic
            elif selection_type == 2:
                fn = d.no_total - d.no_selec + ic
            elif selection_type == 3:
                fn = anum[ic - 1]
            else:
                raise ValueError("selection_type must be 1, 2, 3 or 4")
            chosen.append(fn)
        def cfg(fn, train):
            name = os.path.join(db_path, f"{d.cls}_{d.klm}_{fn:06d}.poscar")
            return Config(name, train, li, d.w_e * factors[0], d.w_f * factors[1], d.w_s * factors[2],
                          d.has_e, d.has_f, d.has_s)
        out += [cfg(fn, True) for fn in chosen]
        if d.no_selec == d.no_total:
            continue
        for ic in range(d.no_start, d.no_total + 1):
            if selection_type == 3:
                if ic in anum:
                    continue
            elif d.no_start <= ic < d.no_start + d.no_selec:
                # the reference marks selection indices, not file numbers, so for
                # selection_type=2 the test files are no_selec+1..no_total (build_subdata.F90:1988-2003)
                continue
            out.append(cfg(ic, False))
    return out
