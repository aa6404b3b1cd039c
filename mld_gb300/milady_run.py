"""``milady_run``: the Python entry of the MILADY fit, driving the GPU path through the C ABI.

Mirrors the documented surface ``milady_run(input, db_model, DB, workdir, output, check)`` of the
reference's Python wrapper (README of the MILADY project): it reads the ``&input_ml`` namelist,
``db_model.in`` and the POSCAR database, then for descriptor_type = 9

* ml_type = -1 writes the descriptors of every selected configuration to
  ``desc<db_path><class>_<klm>_<n>.eml`` (read_write_descriptors.F90:120-200);
* ml_type = 0 (mld_order 1 linear, 2 quadratic QNML) or 1 (kernel ridge, polynomial kernel) fits
  with ``mld_gpu_fit``, writes ``<desc>_<model>_params.pot`` and ``lammps_<...>`` (module_write_
  parameters.F90:762-1530) and the predictions of the training and test configurations in the
  reference's ``train_*.out`` / ``test_*.out`` layout (``es20.10`` predicted and reference values,
  class and file name; mld.F90:944-1020).

The kernel model reads its reference points from ``kernel_matrix.dat`` in ``workdir`` when the
file exists (compute_kernel.F90:1106-1160); otherwise it runs the reference's randomised CUR
selection (mld_gb300.kernel_select; kernel_dump = 3) over the selected configurations and writes
the file.  The Mahalanobis-distance selections (kernel_dump 1, 2, 4) need the MCD statistics,
which this build does not implement, so every kernel_dump value takes the CUR selection.
"""
from __future__ import annotations

import dataclasses
import os
from typing import Dict, List, Optional

import numpy as np

from . import _lib, db_model, elements, kernel_select, namelist, poscar, potfile


@dataclasses.dataclass
class FitResult:
    w: Optional[np.ndarray]
    rmse_train: Optional[np.ndarray]
    rmse_test: Optional[np.ndarray]
    n_train: int
    n_test: int
    files: Dict[str, str]


def _config(nl: dict, precision: int) -> _lib.MldGpuConfig:
    if int(nl["descriptor_type"]) != 9:
        raise ValueError("this build implements descriptor_type = 9 (bispectrum SO(4)) only")
    ml_type, order = int(nl["ml_type"]), int(nl["mld_order"])
    if ml_type not in (-1, 0, 1) or (ml_type == 0 and order not in (1, 2)):
        raise ValueError("this build implements ml_type -1, 0 (mld_order 1 or 2) and 1 (kernel ridge)")
    if ml_type == 1 and int(nl["kernel_type"]) != potfile.KERNEL_PO:
        raise ValueError("the kernel model implements kernel_type = 4 (polynomial) only")
    c = _lib.default_config()
    c.ml_type = max(ml_type, 0)
    c.mld_order = order if ml_type == 0 else 1
    c.j_max = float(nl["j_max"])
    c.r_cut = float(nl["r_cut"])
    c.inv_r0_input = float(nl["inv_r0_input"])
    c.weighted = int(bool(nl["weighted"]))
    c.weighted_3ch = int(bool(nl["weighted_3ch"])) if c.weighted else 0
    els = namelist.elements(nl) or ["X"]
    c.n_elements = len(els)
    w1 = namelist.element_weights(nl, "weight_per_element")
    w2 = namelist.element_weights(nl, "weight_per_element_3ch")
    if nl.get("weighted_auto") and c.weighted:
        w1, w2 = (list(x) for x in elements.auto_channel_weights(els))
    for i, x in enumerate(w1[: _lib.MAX_ELEMENTS]):
        c.weight_per_element[i] = x
    for i, x in enumerate(w2[: _lib.MAX_ELEMENTS]):
        c.weight_per_element_3ch[i] = x
    c.desc_forces = int(bool(nl["desc_forces"])) or int(ml_type >= 0)
    c.lambda_krr = float(nl["lambda_krr"])
    c.svd_rcond = float(nl["svd_rcond"])
    c.sign_stress = float(nl["sign_stress"])
    c.sign_stress_big_box = float(nl["sign_stress_big_box"])
    c.kernel_type = int(nl["kernel_type"])
    c.kernel_power = float(nl["kernel_power"])
    c.length_kernel = float(nl["length_kernel"])
    c.sigma_kernel = float(nl["sigma_kernel"])
    c.precision = precision
    return c


def _load(cfgs: List[db_model.Config], root: str, els: List[str], iread_energy: int, want_forces: bool):
    ss = []
    for c in cfgs:
        s = poscar.read_poscar(os.path.join(root, c.filename), want_forces=want_forces)
        # map POSCAR species onto the namelist element list (itype_to_global)
        m = np.array([els.index(e) if e in els else 0 for e in s.elements], np.int32)
        s.types = m[s.types]
        ss.append(s)
    nat = np.array([s.nat for s in ss], np.int32)
    pos = np.concatenate([s.positions for s in ss])
    cell = np.stack([s.cell for s in ss])
    types = np.concatenate([s.types for s in ss])
    E = np.array([s.energies[iread_energy - 1] for s in ss])
    F = np.concatenate([s.forces if s.forces is not None else np.zeros((s.nat, 3)) for s in ss])
    S = np.stack([s.stress if s.stress is not None else np.zeros(6) for s in ss])
    has = np.array([[c.has_e and s.has_energy, c.has_f and s.has_force, c.has_s and s.has_stress]
                    for c, s in zip(cfgs, ss)], np.int32)
    w = np.array([[c.w_e, c.w_f, c.w_s] for c in cfgs])
    return ss, nat, pos, cell, types, E, F, S, has, w


def _write(path: str, rows: List[tuple]):
    with open(path, "w") as fh:
        for pred, ref, cls, name in rows:
            fh.write("%20.10E%20.10E %s %s\n" % (pred, ref, cls, name))


def _stem(c: db_model.Config) -> str:
    return os.path.splitext(os.path.basename(c.filename))[0]


def _atom_order(classes: List[str], cfg_class: List[str], nat: np.ndarray) -> np.ndarray:
    """Atoms of the configurations of the given classes, class by class, then in configuration
    order (the column order of compute_sca_phia, module_Sigma_matrix.F90:458-480)."""
    starts = np.concatenate([[0], np.cumsum(nat)])
    out = [np.arange(starts[i], starts[i + 1]) for cl in classes for i, c in enumerate(cfg_class) if c == cl]
    return np.concatenate(out) if out else np.zeros(0, np.int64)


def _kernel_points(cfg: _lib.MldGpuConfig, nl: dict, lines: List[db_model.DbLine], cfgs: List[db_model.Config],
                   DB: str, els: List[str], workdir: str, files: Dict[str, str]) -> np.ndarray:
    """Reference points from ``kernel_matrix.dat`` when it exists, else the two CUR picks of the
    reference's descriptor analysis (kernel_dump = 3): ``np_kernel_ref`` atoms from the classes of
    ``classes_for_mcd``, ``np_kernel_full`` from every class, over all selected configurations
    (main_descriptors_analysis.F90:316-372); the file is written and read back."""
    path = os.path.join(workdir, "kernel_matrix.dat")
    if os.path.exists(path):
        return potfile.read_kernel_matrix(path)
    with _lib.Handle(cfg) as h:
        _, nat, pos, cell, types, *_ = _load(cfgs, DB, els, int(nl["iread_energy"]), False)
        h.set_structures(nat, pos, cell, types)
        B, _ = h.descriptors()
    cfg_class = [lines[c.line].cls for c in cfgs]
    full_classes = list(dict.fromkeys(d.cls for d in lines))  # get_distinct_classes, build_subdata.F90:1636-1675
    inner = _atom_order(str(nl["classes_for_mcd"]).split(), cfg_class, nat)
    full = _atom_order(full_classes, cfg_class, nat)
    if inner.size == 0:
        raise ValueError("no configuration of the classes_for_mcd classes is selected")
    first, second = kernel_select.cur_kernel_points(
        B[inner], B[full], int(nl["np_kernel_ref"]), int(nl["np_kernel_full"]), seed=int(nl["seed"]),
        k=int(nl["cur_kval"]), r=int(nl["cur_rval"]), eps=float(nl["cur_eps"]), svd_rcond=float(nl["svd_rcond"]))
    idx = np.concatenate([inner[first.selected], full[second.selected]])
    starts = np.concatenate([[0], np.cumsum(nat)])
    conf = np.searchsorted(starts, idx, side="right") - 1
    potfile.write_kernel_matrix(path, B[idx], conf + 1, idx - starts[conf] + 1,
                                [f"{lines[cfgs[i].line].cls}_{lines[cfgs[i].line].klm}_{_stem(cfgs[i])}" for i in conf])
    files["kernel_matrix"] = path
    return potfile.read_kernel_matrix(path)  # the fit uses the points as written (10 digits), as the reference does


def _standardise(z: np.ndarray) -> np.ndarray:
    """(z - mean) / population std per component (compute_kernel.F90:1170-1199)."""
    d = z - z.mean(axis=0)
    return d / np.sqrt((d * d).mean(axis=0))


def milady_run(input: str, db_model_file: str = "db_model.in", DB: str = "DB/", workdir: str = ".",
               output: str = "out", check: bool = False, precision: int = _lib.MIXED) -> FitResult:
    nl = namelist.read_input_ml(input)
    lines = db_model.read_db_model(db_model_file, int(nl["selection_type"]))
    cfgs = db_model.select(lines, int(nl["selection_type"]), int(nl["seed"]), db_path="",
                           factors=(float(nl["factor_energy_error"]), float(nl["factor_force_error"]),
                                    float(nl["factor_stress_error"])))
    els = namelist.elements(nl)
    ml_type = int(nl["ml_type"])
    files: Dict[str, str] = {}
    cfg = _config(nl, precision)

    if ml_type == -1:
        out_dir = os.path.join(workdir, "desc" + str(nl["db_path"]).strip())
        os.makedirs(out_dir, exist_ok=True)
        with _lib.Handle(cfg) as h:
            ss, nat, pos, cell, types, *_ = _load(cfgs, DB, els, int(nl["iread_energy"]), False)
            h.set_structures(nat, pos, cell, types)
            B, _ = h.descriptors()
        a0 = 0
        for c, n in zip(cfgs, nat):
            p = os.path.join(out_dir, _stem(c) + ".eml")
            potfile.write_eml(p, B[a0:a0 + n])
            files[_stem(c)] = p
            a0 += int(n)
        return FitResult(None, None, None, 0, len(cfgs), files)

    train = [c for c in cfgs if c.train]
    test = [c for c in cfgs if not c.train]
    os.makedirs(os.path.join(workdir, output), exist_ok=True)
    with _lib.Handle(cfg) as h:
        ss, nat, pos, cell, types, E, F, S, has, w = _load(train, DB, els, int(nl["iread_energy"]), True)
        h.set_structures(nat, pos, cell, types)
        Z = None
        if ml_type == 1:
            Z = _kernel_points(cfg, nl, lines, cfgs, DB, els, workdir, files)
            h.set_kernel_points(Z)
        h.set_labels(E, F, S, has, w)
        coef, rmse = h.fit()

        order = potfile.MLD_KERNEL if ml_type == 1 else int(nl["mld_order"])
        extra = {}
        if ml_type == 1:
            extra = dict(kernel_points=_standardise(Z), kernel_type=cfg.kernel_type, sigma_kernel=cfg.sigma_kernel,
                         length_kernel=cfg.length_kernel, kernel_power=cfg.kernel_power)
        nch = 3 if cfg.weighted_3ch else (2 if cfg.weighted else 1)
        p_mld, p_lmp = potfile.write_potential(
            workdir, coef, els or ["X"], j_max=cfg.j_max, r_cut=cfg.r_cut, mld_order=order, nchannels=nch,
            weights=list(cfg.weight_per_element)[:len(els)] if cfg.weighted else None,
            weights_3ch=list(cfg.weight_per_element_3ch)[:len(els)] if cfg.weighted_3ch else None, **extra)
        files["pot"], files["lammps_pot"] = p_mld, p_lmp

        rmse_test = None
        for tag, group in (("train", train), ("test", test)):
            if not group or (tag == "test" and nl.get("train_only")):
                continue
            if tag == "test":
                ss, nat, pos, cell, types, E, F, S, has, w = _load(group, DB, els, int(nl["iread_energy"]), True)
                h.set_structures(nat, pos, cell, types)
            Ep, Fp, Sp = h.predict(coef)
            er, fr, sr = [], [], []
            a0 = 0
            for i, (c, s) in enumerate(zip(group, ss)):
                nm = os.path.basename(c.filename)
                cls = nm.split("_")[0]
                if has[i, 0]:
                    er.append((Ep[i], E[i], cls, nm))
                if has[i, 1]:
                    for a in range(s.nat):
                        for k in range(3):
                            fr.append((Fp[a0 + a, k], F[a0 + a, k], cls, nm))
                if has[i, 2]:
                    for k in range(6):
                        sr.append((Sp[i, k], S[i, k], cls, nm))
                a0 += s.nat
            for kind, rows in (("energy", er), ("force", fr), ("stress", sr)):
                p = os.path.join(workdir, output, f"{tag}_{kind}.out")
                _write(p, rows)
                files[f"{tag}_{kind}"] = p
            if tag == "test":
                rmse_test = np.array([np.sqrt(np.mean([(a - b) ** 2 for a, b, *_ in r])) if r else 0.0
                                      for r in (er, fr, sr)])
    return FitResult(coef, rmse, rmse_test, len(train), len(test), files)
