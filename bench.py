"""Benchmark of the batched bispectrum-SO(4) linear fit (MILADY descriptor-to-fit path).

Workload: 2,000 bcc Fe structures, atom counts log-uniform in 16..1024, supercells trimmed to size
with 0-3 extra vacancies, sigma = 0.08 A noise, +-2 % strain, Morse labels; bispectrum j_max = 4
(55 components), r_cut = 4.7 A, linear model (1 + 55 columns), energy + 3N force + 6 stress
rows per structure, ridge lambda = 1e-8, min-norm solve.  Seeded synthetic data (no dataset).

One step = one full fit of the whole set on the GPU: neighbour lists, fused descriptor +
design-row kernel, weighted Gram, ridge solve, train predictions/RMSE.

  value   design rows / s of the mixed method (FP32 descriptors and rows, FP64 Gram and solve),
          inputs resident in HBM, device time from CUDA events on the library's stream;
  e2e     the same through the C ABI with host buffers: each step stages positions, cells, types
          and labels from pinned host memory and reads back the coefficients and RMSE;
  plain   the all-FP64 method on the same data (the baseline named by the metric);
  roofline  for the dominant kernel (fused descriptor kernel) against the measured FMA peak of
          the pipe it runs on.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_STRUCT = 2000
RCUT = 4.7
J_MAX = 4.0
LAMBDA = 1e-8
# DRAM bytes (read + write) of one k_bso4<float> launch per atom, from an ncu capture of the
# 200-structure Fe case (45,702 atoms): 43.9 MB read (neighbour data, tables) + 1.017 GB written
# (w*dB of every pair, the input of the row gather); both grow with the atoms (and their pairs),
# so the figure is scaled by the atoms of the launch
BSO4_DRAM_BYTES_PER_ATOM = (43.937024e6 + 1.017037e9) / 45702


def _args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--structures", type=int, default=N_STRUCT)
    p.add_argument("--plain-steps", type=int, default=2)
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--workload", choices=["fe_linear", "hea_qnml", "hea_krr", "serve"], default="fe_linear",
                   help="fe_linear: batched linear Fe fit (default); hea_qnml: quadratic QNML fit of the "
                        "5-element alloy (4,000 x 250 atoms, weighted two-channel bispectrum); hea_krr: kernel "
                        "ridge regression of the same structures with 4,000 leverage-selected reference atoms")
    p.add_argument("--ref-points", type=int, default=4000, help="hea_krr: kernel reference points")
    p.add_argument("--requests", type=int, default=300, help="serve: number of requests")
    p.add_argument("--rate", type=float, default=100.0, help="serve: Poisson arrival rate [requests/s]")
    p.add_argument("--plain-structures", type=int, default=100,
                   help="hea_qnml / hea_krr: structures of the sample on which mixed and plain FP64 are compared")
    p.add_argument("--no-extra", action="store_true",
                   help="headline workload only (skip the alloy QNML, KRR and serving records)")
    return p.parse_args()


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    return rank, world


def max_over_ranks(ms_step: float, world: int) -> float:
    """The step time of the slowest replica (gloo all-reduce over the ranks; the process group
    is initialised by the caller when world > 1)."""
    if world <= 1:
        return ms_step
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms_step], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rows_per_s(rows_per_replica: int, ms_step: float, world: int) -> float:
    """Whole-job throughput of `world` replicas that each fit rows_per_replica rows in the
    slowest replica's step time."""
    return world * rows_per_replica / (ms_step * 1e-3)


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                      "-i", os.environ.get("LOCAL_RANK", "0")],
                                     capture_output=True, text=True, timeout=5).stdout.strip()
                if out:
                    self.rows.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if len(r) > 5 + i and r[5 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def make_dataset(n_struct):
    from mld_gb300 import synth
    return synth.fe_bcc_batched(n_struct=n_struct, rcut=RCUT, workers=min(16, os.cpu_count() or 1))


def flops_model(wc, n_pairs, n_atoms):
    """Algorithmic FLOPs of one launch of the fused descriptor kernel (per atom and per pair).

    Per neighbour pair: U recursion (8 flops for a one-term entry, 18 for a two-term entry),
    f_c*w*U accumulation (4 per entry per channel), U+dU recursion (U as above plus 54 per source
    term), vecall (12 per entry), dB contraction (3 components x 4 flops per merged Y slot per
    channel) and the row scatter (3*K adds per channel).  Per atom: the Z contraction (8 flops per
    CG term + 2 per row extent + 4 per output for the scale) and B (4 flops per ZA slot), per
    channel."""
    nch, NU, one, two = wc["nch"], wc["NU"], wc["u_one_term"], wc["u_two_term"]
    u_flops = 8 * one + 18 * two
    per_pair = (u_flops + 4 * NU * nch) + (u_flops + 54 * (one + 2 * two) + 12 * NU) + \
        nch * (12 * wc["y_slots"] + 3 * wc["K"])
    per_atom = nch * (8 * wc["cg_terms"] + 2 * wc["z_row_extents"] + 4 * wc["z_outputs"] + 4 * wc["y_slots_za"])
    return per_pair * n_pairs + per_atom * n_atoms, per_pair, per_atom


def run_ours(a, rank, world):
    from mld_gb300 import _lib
    ds = make_dataset(a.structures)
    nat, pos, cell, types = ds.arrays()
    E, F, S, has = ds.labels()
    wefs = np.ones((len(nat), 3))

    def handle(precision):
        c = _lib.default_config()
        c.j_max, c.r_cut, c.lambda_krr, c.precision = J_MAX, RCUT, LAMBDA, precision
        c.n_elements = 1
        h = _lib.Handle(c)
        h.set_structures(nat, pos, cell, types)
        h.set_labels(E, F, S, has, wefs)
        return h

    res = {}
    # ---------------- mixed method, inputs resident ---------------------------------------
    h = handle(_lib.MIXED)
    M = h.num_rows()
    A = int(nat.sum())
    for _ in range(a.warmup):
        w_mixed, rmse_mixed = h.fit()
    h.set_profiling(True)
    h.profile(reset=True)
    with Clocks() as clk:
        h.timer_start()
        for _ in range(a.steps):
            w_mixed, rmse_mixed = h.fit()
        ms_total = h.timer_stop()
    prof = h.profile(reset=True)
    h.set_profiling(False)
    ms_step = ms_total / a.steps
    wc = h.work_counts()
    flops, per_pair, per_atom = flops_model(wc, wc["pairs"], wc["atoms"])
    t_desc = prof["descriptors"][0] / max(prof["descriptors"][2], 1)
    peak32 = h.peak_flops(_lib.MIXED)
    launches = int(sum(v[1] for v in prof.values()))
    res["solve_info"] = h.solve_info()
    res["autotune"] = h.tuning(0)
    res.update(M=M, A=A, ms_step=ms_step, rmse_mixed=rmse_mixed.tolist(), prof=prof, wc=wc, flops=flops,
               t_desc=t_desc, peak32=peak32, launches=launches, clocks=clk.summary(),
               per_pair=per_pair, per_atom=per_atom)

    # ---------------- e2e through the C ABI with host buffers -----------------------------
    if not a.no_e2e:
        try:
            import torch
            def pinned(x):
                t = torch.from_numpy(np.ascontiguousarray(x)).pin_memory()
                return t, t.numpy()
        except Exception:  # pragma: no cover - torch absent: pageable host memory
            def pinned(x):
                y = np.ascontiguousarray(x)
                return None, y
        keep = [pinned(x) for x in (nat, pos, cell, types, E, F, S, has, wefs)]
        hn = [k[1] for k in keep]
        for _ in range(1):
            h.set_structures(hn[0], hn[1], hn[2], hn[3])
            h.set_labels(hn[4], hn[5], hn[6], hn[7], hn[8])
            h.fit()
        h.timer_start()
        t0 = time.perf_counter()
        for _ in range(a.steps):
            h.set_structures(hn[0], hn[1], hn[2], hn[3])
            h.set_labels(hn[4], hn[5], hn[6], hn[7], hn[8])
            w_e2e, _ = h.fit()
        ms_e2e = h.timer_stop() / a.steps
        wall_e2e = (time.perf_counter() - t0) * 1e3 / a.steps
        S_ = len(nat)
        h2d = (nat.nbytes + pos.nbytes + cell.nbytes + types.nbytes + E.nbytes + F.nbytes + S.nbytes +
               has.nbytes + wefs.nbytes + 4 * A + 4 * (S_ + 1) + 8 * 9 * S_ + 4 * S_ + 12 * S_ + 8 * S_ +
               3 * 8 * S_)
        d2h = 8 * h.dim_design_line + 8 * 6 + 8
        res.update(ms_e2e=ms_e2e, wall_e2e=wall_e2e, h2d=int(h2d), d2h=int(d2h))
    h.close()

    # ---------------- plain FP64 method on the same data ----------------------------------
    if a.plain_steps > 0:
        h64 = handle(_lib.PLAIN_FP64)
        w64, rmse64 = h64.fit()
        h64.set_profiling(True)
        h64.profile(reset=True)
        h64.timer_start()
        for _ in range(a.plain_steps):
            w64, rmse64 = h64.fit()
        ms64 = h64.timer_stop() / a.plain_steps
        prof64 = h64.profile(reset=True)
        peak64 = h64.peak_flops(_lib.PLAIN_FP64)
        h64.close()
        res.update(ms64=ms64, rmse64=rmse64.tolist(), prof64=prof64, peak64=peak64)
    else:
        res.update(ms64=None, rmse64=None, prof64=None, peak64=None)
    res["ds"] = ds
    return res


def run_hea(a):
    """QNML quadratic fit of the 5-element bcc alloy: one step = one full mixed-method fit of
    the whole set (neighbours, two-channel descriptors, quadratic rows, tensor-core Gram of the
    linear and quadratic blocks, Cholesky-preconditioned CG).  The plain FP64 method is timed on
    the first --plain-structures structures (its FP64 Gram grows as rows x D^2 and takes
    minutes on the whole set); both methods are fitted on that sample for the RMSE comparison."""
    from mld_gb300 import _lib, synth
    n_struct = a.structures if a.structures != N_STRUCT else 4000
    ds = synth.hea_bcc_batched(n_struct=n_struct, workers=min(16, os.cpu_count() or 1))
    lam = 1e-8

    def handle(precision, idx=None):
        c = _lib.default_config()
        c.j_max, c.r_cut, c.lambda_krr, c.precision, c.mld_order = 4.0, 5.0, lam, precision, 2
        c.weighted = 1
        c.n_elements = len(synth.HEA_ELEMENTS)
        for i, wv in enumerate(synth.HEA_WEIGHTS):
            c.weight_per_element[i] = wv
        h = _lib.Handle(c)
        sub = ds if idx is None else synth.Dataset([ds.structures[i] for i in idx], ds.rcut, ds.name)
        nat, pos, cell, types = sub.arrays()
        E, F, S, has = sub.labels()
        h.set_structures(nat, pos, cell, types)
        h.set_labels(E, F, S, has, np.ones((len(nat), 3)))
        return h, int(nat.sum())

    out = {}
    h, A = handle(_lib.MIXED)
    M = h.num_rows()
    for _ in range(a.warmup):
        h.fit()
    h.set_profiling(True)
    h.profile(reset=True)
    with Clocks() as clk:
        h.timer_start()
        for _ in range(a.steps):
            w, rmse = h.fit()
        ms = h.timer_stop() / a.steps
    prof = h.profile(reset=True)
    out.update(ms=ms, rmse=rmse.tolist(), prof={k: v[0] / a.steps for k, v in prof.items()},
               launches=int(sum(v[1] for v in prof.values())), solve=h.solve_info(), clocks=clk.summary(),
               D=h.dim_design_line)
    h.close()
    sample = {}
    if a.plain_structures > 0:
        # both methods fitted on the same structures: the same-workload speed ratio, and the mixed
        # fit's error against the FP64 fit per stage (linear block, quadratic block) in the
        # coefficients and in the energy / force / stress predictions
        idx = list(range(min(a.plain_structures, n_struct)))
        fits = {}
        for name, prec in (("mixed", _lib.MIXED), ("plain_fp64", _lib.PLAIN_FP64)):
            hs, As = handle(prec, idx)
            Ms = hs.num_rows()
            hs.fit()
            hs.timer_start()
            ws, rs = hs.fit()
            t = hs.timer_stop()
            fits[name] = (ws, hs.predict(ws))
            sample[name] = {"ms_per_fit": t, "design_rows": Ms, "rows_per_s": Ms / (t * 1e-3), "rmse_efs": rs.tolist()}
            if prec == _lib.MIXED:
                sample[name]["solve"] = hs.solve_info()
            hs.close()
        mx, pl = sample["mixed"], sample["plain_fp64"]
        sample["force_rmse_rel_diff"] = abs(mx["rmse_efs"][1] - pl["rmse_efs"][1]) / pl["rmse_efs"][1]
        sample["speedup_same_structures"] = mx["rows_per_s"] / pl["rows_per_s"]
        (wm, pm), (wp, pp) = fits["mixed"], fits["plain_fp64"]
        KK = int(round((-1 + np.sqrt(1 + 4 * (len(wp) - 1))) / 2))
        rel = lambda x, y: float(np.abs(np.asarray(x) - np.asarray(y)).max() / max(np.abs(y).max(), 1e-300))
        sample["mixed_vs_fp64"] = {
            "w_rel_linear_block": rel(wm[:1 + KK], wp[:1 + KK]),
            "w_rel_quadratic_block": rel(wm[1 + KK:], wp[1 + KK:]),
            "pred_rel_energy": rel(pm[0], pp[0]), "pred_rel_force": rel(pm[1], pp[1]),
            "pred_rel_stress": rel(pm[2], pp[2])}
    line = {
        "metric": "design rows/s (QNML quadratic fit, 5-element bcc alloy, weighted bispectrum j_max=4)",
        "value": M / (ms * 1e-3), "unit": "design rows/s", "n_gpus": 1, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32 descriptors/rows; linear block: bf16x3 tensor-core Gram (fp32 acc) + fp64 Cholesky; "
                 "quadratic block: sparse-sign sketch + double-fp32 Gram/Cholesky + fp32 inverse; double-fp32 CG",
        "data": "synthetic",
        "config": {"workload": "hea_bcc_MoNbTaVCr_4000x250_qnml_weighted_jmax4", "structures": n_struct,
                   "atoms": A, "design_rows": M, "dim_design_line_full": out["D"], "r_cut": 5.0, "lambda_krr": lam,
                   "l2": "working set above L2 every step", "parallelism": "single"},
        "atom_evals_per_s": A / (ms * 1e-3), "rmse_efs": out["rmse"], "phase_ms": out["prof"],
        "mixed_solve": out["solve"], "gpu_launches": out["launches"], "clocks": out["clocks"],
        "sample_comparison": sample or None,
    }
    return line


def run_hea_krr(a):
    """Kernel ridge regression (ml_type 1, polynomial kernel p = 2, length sqrt(1/2), sigma 0,
    lambda = 1e-6 with the lambda^2 penalty) of the 5-element alloy set: reference atoms chosen
    by seeded leverage-score selection over all atoms' descriptors.  One step = one full mixed
    fit (descriptors, kernel features and derivatives, design rows, tensor-core Gram, CG); the
    plain FP64 method is compared on the first --plain-structures structures with the same
    reference points."""
    from mld_gb300 import _lib, kernel_select, synth
    n_struct = a.structures if a.structures != N_STRUCT else 4000
    ds = synth.hea_bcc_batched(n_struct=n_struct, workers=min(16, os.cpu_count() or 1))
    lam = 1e-6

    def handle(precision, idx=None):
        c = _lib.default_config()
        c.j_max, c.r_cut, c.lambda_krr, c.precision, c.ml_type = 4.0, 5.0, lam, precision, 1
        c.weighted = 1
        c.n_elements = len(synth.HEA_ELEMENTS)
        for i, wv in enumerate(synth.HEA_WEIGHTS):
            c.weight_per_element[i] = wv
        h = _lib.Handle(c)
        sub = ds if idx is None else synth.Dataset([ds.structures[i] for i in idx], ds.rcut, ds.name)
        nat, pos, cell, types = sub.arrays()
        E, F, S, has = sub.labels()
        h.set_structures(nat, pos, cell, types)
        h.set_labels(E, F, S, has, np.ones((len(nat), 3)))
        return h, int(nat.sum())

    h, A = handle(_lib.MIXED)
    B, _ = h.descriptors()
    ref = kernel_select.select(B, a.ref_points)
    Zraw = B[ref].copy()
    del B
    h.set_kernel_points(Zraw)
    M = h.num_rows()
    for _ in range(a.warmup):
        h.fit()
    h.set_profiling(True)
    h.profile(reset=True)
    with Clocks() as clk:
        h.timer_start()
        for _ in range(a.steps):
            w, rmse = h.fit()
        ms = h.timer_stop() / a.steps
    prof = h.profile(reset=True)
    out = dict(ms=ms, rmse=rmse.tolist(), prof={k: v[0] / a.steps for k, v in prof.items()},
               launches=int(sum(v[1] for v in prof.values())), solve=h.solve_info(), clocks=clk.summary(),
               D=h.dim_design_line)
    h.close()
    sample = {}
    if a.plain_structures > 0:
        idx = list(range(min(a.plain_structures, n_struct)))
        for name, prec in (("mixed", _lib.MIXED), ("plain_fp64", _lib.PLAIN_FP64)):
            hs, As = handle(prec, idx)
            hs.set_kernel_points(Zraw)
            Ms = hs.num_rows()
            hs.fit()
            hs.timer_start()
            ws, rs = hs.fit()
            t = hs.timer_stop()
            sample[name] = {"ms_per_fit": t, "design_rows": Ms, "rows_per_s": Ms / (t * 1e-3), "rmse_efs": rs.tolist()}
            hs.close()
        mx, pl = sample["mixed"], sample["plain_fp64"]
        sample["force_rmse_rel_diff"] = abs(mx["rmse_efs"][1] - pl["rmse_efs"][1]) / pl["rmse_efs"][1]
        sample["speedup_same_structures"] = mx["rows_per_s"] / pl["rows_per_s"]
    line = {
        "metric": "design rows/s (kernel ridge regression, polynomial kernel, 5-element bcc alloy)",
        "value": M / (ms * 1e-3), "unit": "design rows/s", "n_gpus": 1, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32 descriptors, kernel rows (force rows: bf16x3 tensor cores, fp32 acc); sparse-sign sketch + "
                 "double-fp32 Gram/Cholesky + fp32 inverse as preconditioner; double-fp32 CG",
        "data": "synthetic",
        "config": {"workload": "hea_bcc_MoNbTaVCr_4000x250_krr_poly2_weighted_jmax4", "structures": n_struct,
                   "atoms": A, "design_rows": M, "reference_points": int(a.ref_points),
                   "dim_design_line": out["D"], "r_cut": 5.0, "lambda_krr": lam, "penalty": "lambda^2",
                   "l2": "working set above L2 every step", "parallelism": "single"},
        "atom_evals_per_s": A / (ms * 1e-3), "rmse_efs": out["rmse"], "phase_ms": out["prof"],
        "mixed_solve": out["solve"], "gpu_launches": out["launches"], "clocks": out["clocks"],
        "sample_comparison": sample or None,
    }
    return line


def run_serve(a):
    """Serving loop with the fitted quadratic alloy potential: requests are random 5-element bcc
    structures with atom counts log-uniform in 8..20,000 (sigma 0.1 A) arriving as a Poisson
    stream at --rate; the server admits them into free evaluation slots by HBM budget
    (continuous batching) and evaluates energy, forces and stress.  Reports p50/p99 latency
    (submit to result) and atoms/s for the mixed and the plain FP64 method on the same request
    stream, and the relative force difference between the two."""
    from mld_gb300 import _lib, synth
    rng = np.random.default_rng(20240607)
    # the potential: QNML fit on a training set of the alloy (mixed method)
    train = synth.hea_bcc_batched(n_struct=240, workers=min(16, os.cpu_count() or 1), seed=20240608)
    c = _lib.default_config()
    c.j_max, c.r_cut, c.lambda_krr, c.precision, c.mld_order = 4.0, 5.0, 1e-8, _lib.MIXED, 2
    c.weighted, c.n_elements = 1, len(synth.HEA_ELEMENTS)
    for i, wv in enumerate(synth.HEA_WEIGHTS):
        c.weight_per_element[i] = wv
    with _lib.Handle(c) as h:
        nat, pos, cell, types = train.arrays()
        E, F, S, has = train.labels()
        h.set_structures(nat, pos, cell, types)
        h.set_labels(E, F, S, has, np.ones((len(nat), 3)))
        w, _ = h.fit()
    n = a.requests
    sizes = np.exp(rng.uniform(np.log(8), np.log(20000), size=n)).round().astype(int)
    reqs = [synth.hea_request(rng, int(k)) for k in sizes]
    arrivals = np.cumsum(rng.exponential(1.0 / a.rate, size=n))
    total_atoms = int(sizes.sum())
    out = {}
    forces = {}
    for name, prec in (("mixed", _lib.MIXED), ("plain_fp64", _lib.PLAIN_FP64)):
        c.precision = prec
        srv = _lib.Server(c, w, n_slots=3, max_batch_atoms=150000, hbm_fraction=0.5)
        # warm-up: one request of each size class through every slot
        for k in (16, 2000, 20000):
            srv.wait(srv.submit(*(lambda r: (r.positions, r.cell, r.types))(synth.hea_request(rng, k))))
        lat = np.zeros(n)
        res = [None] * n
        pending = {}
        t0 = time.perf_counter()
        i = done = 0
        with Clocks() as clk:
            while done < n:
                now = time.perf_counter() - t0
                while i < n and arrivals[i] <= now:
                    r = reqs[i]
                    pending[srv.submit(r.positions, r.cell, r.types)] = i
                    i += 1
                srv.progress()
                for t in list(pending):
                    got = srv.result(t)
                    if got is not None:
                        j = pending.pop(t)
                        res[j] = got[1]
                        lat[j] = got[3]
                        done += 1
                if not pending and i < n:
                    time.sleep(max(0.0, min(0.002, arrivals[i] - (time.perf_counter() - t0))))
        wall = time.perf_counter() - t0
        st = srv.stats()
        srv.close()
        forces[name] = res
        out[name] = {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                     "mean_ms": float(lat.mean()), "atoms_per_s": total_atoms / wall, "wall_s": wall,
                     "batches": st["batches"], "clocks": clk.summary()}
    # per request: max |F_mixed - F_plain| / max |F_plain|; worst request reported
    ferr = max(float(np.abs(fm - fp).max() / max(np.abs(fp).max(), 1e-300))
               for fm, fp in zip(forces["mixed"], forces["plain_fp64"]))
    # over all atoms of all requests: ||F_mixed - F_plain|| / ||F_plain||
    fm_all = np.concatenate([np.asarray(f).reshape(-1) for f in forces["mixed"]])
    fp_all = np.concatenate([np.asarray(f).reshape(-1) for f in forces["plain_fp64"]])
    ferr_rms = float(np.linalg.norm(fm_all - fp_all) / max(np.linalg.norm(fp_all), 1e-300))
    mx = out["mixed"]
    line = {
        "metric": "serving atoms/s and p99 latency (continuous batching, fitted QNML alloy potential)",
        "value": mx["atoms_per_s"], "unit": "atoms/s", "n_gpus": 1, "steps": n, "warmup": 3,
        "ms_per_step": mx["mean_ms"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32 descriptors/rows (mixed) vs fp64 (plain)", "data": "synthetic",
        "config": {"workload": "hea_serve_poisson_8to20000_atoms_qnml_weighted_jmax4", "requests": n,
                   "rate_per_s": a.rate, "atoms": total_atoms, "slots": 3, "max_batch_atoms": 150000,
                   "hbm_fraction": 0.5, "parallelism": "single"},
        "p50_ms": mx["p50_ms"], "p99_ms": mx["p99_ms"], "mixed": mx, "plain_fp64": out["plain_fp64"],
        "force_rel_diff_mixed_vs_plain": ferr,
        "force_rel_diff_mixed_vs_plain_rms": ferr_rms,
    }
    return line


def cpu_sample(ds, target_s=15.0, threads=None):
    """Time the oracle (CPU restatement of the reference) on a bounded sample of the same set:
    neighbours + descriptors + rows in C (OpenMP over structures), Gram + gelsd in NumPy/LAPACK."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ctypes
    import oracle
    oracle.init(J_MAX)
    L = oracle.lib()
    L.orc_rows_batch.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 4 + [ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                                                         ctypes.c_double, ctypes.c_int, ctypes.c_double,
                                                                         ctypes.c_double, ctypes.c_void_p]
    if threads:
        os.environ["OMP_NUM_THREADS"] = str(threads)
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))

    def run(idx):
        ss = [ds.structures[i] for i in idx]
        nat = np.array([s.nat for s in ss], np.int32)
        pos = np.ascontiguousarray(np.concatenate([s.positions for s in ss]))
        cell = np.ascontiguousarray(np.stack([s.cell for s in ss]))
        types = np.ascontiguousarray(np.concatenate([s.types for s in ss]).astype(np.int32))
        rows = int(sum(1 + 3 * s.nat + 6 for s in ss))
        A = np.zeros((rows, 56))
        chw = np.ones(1)
        t0 = time.perf_counter()
        rc = L.orc_rows_batch(len(ss), nat.ctypes.data, pos.ctypes.data, cell.ctypes.data, types.ctypes.data, 1, 1,
                              chw.ctypes.data, RCUT, 300, 1.0, 1.0, A.ctypes.data)
        assert rc == 0
        y = np.concatenate([np.concatenate([[s.energies[1]], s.forces.reshape(-1), s.stress]) for s in ss])
        w = oracle.fit_linear(A, y, np.ones(rows), LAMBDA)
        dt = time.perf_counter() - t0
        return rows, int(nat.sum()), dt

    # calibrate on a few structures, then pick a sample of about target_s seconds
    order = np.random.default_rng(0).permutation(len(ds.structures))
    r0, a0, t0 = run(order[:8])
    per_atom = t0 / max(a0, 1)
    total_atoms = sum(s.nat for s in ds.structures)
    want_atoms = min(total_atoms, int(target_s / max(per_atom, 1e-9)))
    idx, acc = [], 0
    for i in order:
        if acc >= want_atoms:
            break
        idx.append(int(i))
        acc += ds.structures[i].nat
    rows, atoms, dt = run(idx)
    return {"value": rows / dt, "unit": "design rows/s", "cores": cores, "kind": "port",
            "sample": f"{len(idx)} of {len(ds.structures)} structures ({atoms} atoms, {rows} rows), "
                      f"full fit pipeline, {dt:.1f} s", "atoms_per_s": atoms / dt}


def main():
    a = _args()
    rank, world = _dist()
    if a.impl == "reference":
        if rank != 0:
            return
        ds = make_dataset(a.structures)
        vals = []
        for i in range(a.warmup + a.steps):
            r = cpu_sample(ds, target_s=8.0)
            if i >= a.warmup:
                vals.append(r["value"])
        v = float(np.mean(vals))
        line = {"metric": "design rows/s (batched linear fit, bispectrum j_max=4)", "value": v,
                "unit": "design rows/s", "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
                "higher_is_better": True, "impl": "reference", "dtype": "f64", "data": "synthetic",
                "config": {"workload": "fe_bcc_2000_struct_16to1024_atoms_linear_jmax4", "structures": a.structures},
                "cpu_baseline": dict(r, value=v),
                "e2e": {"value": v, "unit": "design rows/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "vs_baseline": None}
        print(json.dumps(line))
        return

    if a.workload in ("hea_qnml", "hea_krr", "serve"):
        if rank == 0:
            print(json.dumps({"hea_qnml": run_hea, "hea_krr": run_hea_krr, "serve": run_serve}[a.workload](a)))
        return
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    res = run_ours(a, rank, world)
    ms_step = max_over_ranks(res["ms_step"], world)
    if rank != 0:
        return
    M, A = res["M"], res["A"]
    value = aggregate_rows_per_s(M, ms_step, world)
    achieved = res["flops"] / (res["t_desc"] * 1e-3) / 1e12
    cpu = None if a.no_cpu else cpu_sample(res["ds"])
    line = {
        "metric": "design rows/s (batched linear fit, bispectrum j_max=4)",
        "value": value,
        "unit": "design rows/s",
        "n_gpus": world,
        "steps": a.steps,
        "warmup": a.warmup,
        "ms_per_step": ms_step,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "fp32 descriptors/rows + bf16x3 tensor-core Gram (fp32 acc) + fp64 Cholesky / double-fp32 CG",
        "data": "synthetic",
        "config": {"workload": "fe_bcc_2000_struct_16to1024_atoms_linear_jmax4", "structures": len(res["ds"].structures),
                   "atoms": A, "design_rows": M, "dim_design_line": 56, "r_cut": RCUT, "lambda_krr": LAMBDA,
                   "l2": "working set above L2 every step (design matrix %.2f GB)" % (M * 56 * 4 / 1e9),
                   "parallelism": "replicas" if world > 1 else "single"},
        "atom_evals_per_s": world * A / (ms_step * 1e-3),
        "rmse_efs": res["rmse_mixed"],
        "plain_fp64": None if res["ms64"] is None else {"value": M / (res["ms64"] * 1e-3), "ms_per_step": res["ms64"], "rmse_efs": res["rmse64"],
                       "steps": a.plain_steps,
                       "phase_ms": {k: v[0] / a.plain_steps for k, v in res["prof64"].items()},
                       "fp64_peak_tflops_measured": res["peak64"]},
        "speedup_vs_plain_fp64": None if res["ms64"] is None else res["ms64"] / ms_step,
        "phase_ms": {k: v[0] / a.steps for k, v in res["prof"].items()},
        "mixed_solve": res["solve_info"],
        "descriptor_autotune": res["autotune"],
        "roofline": {"kernel": "k_bso4<float> (fused descriptor + design rows)", "bound": "fp32",
                     "achieved": achieved, "peak": res["peak32"], "unit": "TFLOP/s", "frac": achieved / res["peak32"],
                     "peak_source": "measured in this run (FP32 FMA probe; not in MEASURED_PEAKS.json)",
                     "flops_per_launch": res["flops"], "flops_per_pair": res["per_pair"],
                     "flops_per_atom": res["per_atom"], "traffic": BSO4_DRAM_BYTES_PER_ATOM * A,
                     "traffic_unit": "bytes per launch",
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch on the "
                                       "200-structure case, scaled by atoms"},
        "gpu_launches": res["launches"],
        "clocks": res["clocks"],
    }
    if "ms_e2e" in res:
        line["e2e"] = {"value": world * M / (res["ms_e2e"] * 1e-3), "unit": "design rows/s",
                       "h2d_bytes_per_step": res["h2d"], "d2h_bytes_per_step": res["d2h"],
                       "ms_per_step": res["ms_e2e"], "host_wall_ms_per_step": res["wall_e2e"]}
    if cpu:
        line["cpu_baseline"] = cpu
    if world == 1 and not a.no_extra:
        line["extra_configs"] = run_extra(a)
    print(json.dumps(line))


def run_extra(a):
    """The alloy workloads of the other configurations at their full size, attached to the
    headline line (fewer timed steps each): the quadratic QNML fit with the same-structure
    comparison against the plain FP64 method, the kernel ridge fit, and the serving loop."""
    import copy
    out = {}
    b = copy.copy(a)
    b.structures, b.steps, b.warmup = N_STRUCT, min(a.steps, 3), 1
    for name, fn in (("hea_qnml", run_hea), ("hea_krr", run_hea_krr), ("serve", run_serve)):
        t0 = time.perf_counter()
        try:
            r = fn(b)
            r["wall_s"] = time.perf_counter() - t0
            out[name] = r
        except Exception as e:  # report, keep the headline line
            out[name] = {"error": f"{type(e).__name__}: {e}"}
    return out


if __name__ == "__main__":
    main()
