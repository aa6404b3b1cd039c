"""ctypes binding of libmld_gpu.so (include/mld_gpu.h).  No PyTorch on this path.

The library is built in-tree by ``mld_gb300.build`` (nvcc, sm_103a).  Loading fails loudly when
it is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional, Sequence, Tuple

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmld_gpu.so")

MLD_OK = 0
ERRORS = {1: "MLD_ERR_INVALID", 2: "MLD_ERR_CUDA", 3: "MLD_ERR_NEIGHBOUR_CAP", 4: "MLD_ERR_OOM",
          5: "MLD_ERR_SOLVE", 6: "MLD_ERR_STATE", 7: "MLD_ERR_UNSUPPORTED", 8: "MLD_ERR_NOALLOC_LIMIT",
          9: "MLD_ERR_TIMEOUT"}
PLAIN_FP64 = 0
MIXED = 1
MAX_ELEMENTS = 8

EXPORTED = ["mld_gpu_config_defaults", "mld_gpu_create", "mld_gpu_destroy", "mld_gpu_last_error", "mld_gpu_dims",
            "mld_gpu_set_structures", "mld_gpu_set_labels", "mld_gpu_descriptors",
            "mld_gpu_descriptor_derivatives", "mld_gpu_num_rows", "mld_gpu_design_matrix", "mld_gpu_gram",
            "mld_gpu_solve", "mld_gpu_fit", "mld_gpu_predict", "mld_gpu_evaluate", "mld_gpu_synchronize", "mld_gpu_set_profiling",
            "mld_gpu_profile", "mld_gpu_timer_start", "mld_gpu_timer_stop", "mld_gpu_work_counts",
            "mld_gpu_peak_flops", "mld_gpu_descriptors_noalloc", "mld_gpu_solve_info", "mld_gpu_gram_rows",
            "mld_gpu_set_kernel_points", "mld_gpu_server_create", "mld_gpu_server_destroy",
            "mld_gpu_server_last_error", "mld_gpu_server_submit", "mld_gpu_server_progress",
            "mld_gpu_server_result", "mld_gpu_server_wait", "mld_gpu_server_stats", "mld_gpu_server_admission",
            "mld_gpu_test_pipeline_timeout", "mld_gpu_tuning"]
NPHASE = 6
PHASES = ["neighbours", "rows", "descriptors", "gram", "solve", "predict"]


class MldGpuConfig(ctypes.Structure):
    _fields_ = [
        ("descriptor_type", ctypes.c_int),
        ("j_max", ctypes.c_double),
        ("r_cut", ctypes.c_double),
        ("inv_r0_input", ctypes.c_double),
        ("weighted", ctypes.c_int),
        ("weighted_3ch", ctypes.c_int),
        ("n_elements", ctypes.c_int),
        ("weight_per_element", ctypes.c_double * MAX_ELEMENTS),
        ("weight_per_element_3ch", ctypes.c_double * MAX_ELEMENTS),
        ("r_cut_pair_in", ctypes.c_double * (MAX_ELEMENTS * MAX_ELEMENTS)),
        ("r_cut_width_in", ctypes.c_double),
        ("desc_forces", ctypes.c_int),
        ("ml_type", ctypes.c_int),
        ("mld_order", ctypes.c_int),
        ("lambda_krr", ctypes.c_double),
        ("svd_rcond", ctypes.c_double),
        ("sign_stress", ctypes.c_double),
        ("sign_stress_big_box", ctypes.c_double),
        ("imm_neigh", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("kernel_type", ctypes.c_int),
        ("kernel_power", ctypes.c_double),
        ("length_kernel", ctypes.c_double),
        ("sigma_kernel", ctypes.c_double),
    ]


class MldError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


_lib: Optional[ctypes.CDLL] = None


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load the native library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it with `python -m mld_gb300.build` (needs nvcc)")
    L = ctypes.CDLL(path)
    P, I, D, LL = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_longlong
    L.mld_gpu_config_defaults.argtypes = [ctypes.POINTER(MldGpuConfig)]
    L.mld_gpu_config_defaults.restype = None
    L.mld_gpu_create.argtypes = [ctypes.POINTER(MldGpuConfig), ctypes.POINTER(P)]
    L.mld_gpu_destroy.argtypes = [P]
    L.mld_gpu_destroy.restype = None
    L.mld_gpu_last_error.argtypes = [P]
    L.mld_gpu_last_error.restype = ctypes.c_char_p
    L.mld_gpu_dims.argtypes = [P, ctypes.POINTER(I), ctypes.POINTER(I), ctypes.POINTER(I)]
    L.mld_gpu_set_structures.argtypes = [P, I, P, P, P, P]
    L.mld_gpu_set_labels.argtypes = [P, P, P, P, P, P]
    L.mld_gpu_descriptors.argtypes = [P, P, P]
    L.mld_gpu_descriptor_derivatives.argtypes = [P, ctypes.POINTER(LL), P, P, P]
    L.mld_gpu_num_rows.argtypes = [P, ctypes.POINTER(LL)]
    L.mld_gpu_design_matrix.argtypes = [P, P, P, P]
    L.mld_gpu_gram.argtypes = [P, P, P]
    L.mld_gpu_solve.argtypes = [P, P, P, I, P, ctypes.POINTER(I)]
    L.mld_gpu_fit.argtypes = [P, P, P]
    L.mld_gpu_predict.argtypes = [P, P, P, P, P]
    L.mld_gpu_evaluate.argtypes = [P, P, P, P, P]
    L.mld_gpu_synchronize.argtypes = [P]
    L.mld_gpu_set_profiling.argtypes = [P, I]
    L.mld_gpu_profile.argtypes = [P, P, P, P, I]
    L.mld_gpu_timer_start.argtypes = [P]
    L.mld_gpu_timer_stop.argtypes = [P, ctypes.POINTER(D)]
    L.mld_gpu_work_counts.argtypes = [P, P]
    L.mld_gpu_peak_flops.argtypes = [P, I, ctypes.POINTER(D)]
    L.mld_gpu_descriptors_noalloc.argtypes = [ctypes.POINTER(MldGpuConfig), I, P, P, P, P, P, ctypes.c_char_p, I]
    for n in EXPORTED:
        if n not in ("mld_gpu_config_defaults", "mld_gpu_destroy", "mld_gpu_last_error"):
            getattr(L, n).restype = I
    _lib = L
    return L


def _p(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def default_config() -> MldGpuConfig:
    c = MldGpuConfig()
    load().mld_gpu_config_defaults(ctypes.byref(c))
    return c


class Handle:
    """Thin owner of an ``mld_gpu_handle``; methods map 1:1 onto the C entry points."""

    def __init__(self, cfg: MldGpuConfig):
        self._L = load()
        self._h = ctypes.c_void_p()
        rc = self._L.mld_gpu_create(ctypes.byref(cfg), ctypes.byref(self._h))
        if rc != MLD_OK:
            raise MldError(rc, "mld_gpu_create failed")
        self.cfg = cfg
        self.nat = np.zeros(0, np.int32)
        self._dims()

    def _dims(self):
        K, dd, D = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self._L.mld_gpu_dims(self._h, ctypes.byref(K), ctypes.byref(dd), ctypes.byref(D))
        self.K, self.dim_desc, self.dim_design_line = K.value, dd.value, D.value

    def close(self):
        if self._h:
            self._L.mld_gpu_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc: int):
        if rc != MLD_OK:
            raise MldError(rc, self._L.mld_gpu_last_error(self._h).decode())

    def set_structures(self, nat: Sequence[int], pos: np.ndarray, cell: np.ndarray, types: np.ndarray):
        self.nat = np.ascontiguousarray(nat, dtype=np.int32)
        self._pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1)
        self._cell = np.ascontiguousarray(cell, dtype=np.float64).reshape(-1)
        self._types = np.ascontiguousarray(types, dtype=np.int32).reshape(-1)
        self._check(self._L.mld_gpu_set_structures(self._h, len(self.nat), _p(self.nat), _p(self._pos),
                                                   _p(self._cell), _p(self._types)))

    def set_labels(self, energy, force, stress, has_efs, w_efs):
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
                for a in (energy, force, stress)]
        has = np.ascontiguousarray(has_efs, dtype=np.int32).reshape(-1)
        w = np.ascontiguousarray(w_efs, dtype=np.float64).reshape(-1)
        self._check(self._L.mld_gpu_set_labels(self._h, _p(arrs[0]), _p(arrs[1]), _p(arrs[2]), _p(has), _p(w)))

    def descriptors(self) -> Tuple[np.ndarray, np.ndarray]:
        A = int(self.nat.sum())
        B = np.zeros((A, self.dim_desc))
        nn = np.zeros(A, np.int32)
        self._check(self._L.mld_gpu_descriptors(self._h, _p(B), _p(nn)))
        return B, nn

    def descriptor_derivatives(self, cap: int):
        P = ctypes.c_longlong(cap)
        nbr = np.zeros(cap, np.int32)
        u = np.zeros((cap, 3))
        dB = np.zeros((cap, 3, self.dim_desc))
        self._check(self._L.mld_gpu_descriptor_derivatives(self._h, ctypes.byref(P), _p(nbr), _p(u), _p(dB)))
        n = P.value
        return nbr[:n], u[:n], dB[:n]

    def num_rows(self) -> int:
        M = ctypes.c_longlong()
        self._check(self._L.mld_gpu_num_rows(self._h, ctypes.byref(M)))
        return M.value

    def design_matrix(self):
        M = self.num_rows()
        A = np.zeros((M, self.dim_design_line))
        y = np.zeros(M)
        w = np.zeros(M)
        self._check(self._L.mld_gpu_design_matrix(self._h, _p(A), _p(y), _p(w)))
        return A, y, w

    def gram(self):
        D = self.dim_design_line
        G = np.zeros((D, D))
        h = np.zeros(D)
        self._check(self._L.mld_gpu_gram(self._h, _p(G), _p(h)))
        return G, h

    def solve(self, G: np.ndarray, rhs: np.ndarray):
        D = G.shape[0]
        G = np.ascontiguousarray(G, dtype=np.float64)
        rhs = np.ascontiguousarray(rhs, dtype=np.float64)
        w = np.zeros(D)
        rank = ctypes.c_int()
        self._check(self._L.mld_gpu_solve(self._h, _p(G), _p(rhs), D, _p(w), ctypes.byref(rank)))
        return w, rank.value

    def fit(self):
        w = np.zeros(self.dim_design_line)
        rmse = np.zeros(3)
        self._check(self._L.mld_gpu_fit(self._h, _p(w), _p(rmse)))
        return w, rmse

    def predict(self, w: np.ndarray):
        A = int(self.nat.sum())
        S = len(self.nat)
        E = np.zeros(S)
        F = np.zeros((A, 3))
        St = np.zeros((S, 6))
        w = np.ascontiguousarray(w, dtype=np.float64)
        self._check(self._L.mld_gpu_predict(self._h, _p(w), _p(E), _p(F), _p(St)))
        return E, F, St

    def evaluate(self, w: np.ndarray):
        """E, F, S as predict() gives them, computed without design rows (mld_gpu_evaluate)."""
        A = int(self.nat.sum())
        S = len(self.nat)
        E = np.zeros(S)
        F = np.zeros((A, 3))
        St = np.zeros((S, 6))
        w = np.ascontiguousarray(w, dtype=np.float64)
        self._check(self._L.mld_gpu_evaluate(self._h, _p(w), _p(E), _p(F), _p(St)))
        return E, F, St

    def synchronize(self):
        self._check(self._L.mld_gpu_synchronize(self._h))

    def set_profiling(self, on: bool = True):
        self._check(self._L.mld_gpu_set_profiling(self._h, int(on)))

    def profile(self, reset: bool = False):
        ms = np.zeros(NPHASE)
        la = np.zeros(NPHASE, np.int64)
        ca = np.zeros(NPHASE, np.int64)
        self._check(self._L.mld_gpu_profile(self._h, _p(ms), _p(la), _p(ca), int(reset)))
        return {k: (ms[i], int(la[i]), int(ca[i])) for i, k in enumerate(PHASES)}

    def timer_start(self):
        self._check(self._L.mld_gpu_timer_start(self._h))

    def timer_stop(self) -> float:
        t = ctypes.c_double()
        self._check(self._L.mld_gpu_timer_stop(self._h, ctypes.byref(t)))
        return t.value

    def peak_flops(self, precision: int) -> float:
        t = ctypes.c_double()
        self._check(self._L.mld_gpu_peak_flops(self._h, int(precision), ctypes.byref(t)))
        return t.value

    def work_counts(self):
        out = np.zeros(12, np.int64)
        self._check(self._L.mld_gpu_work_counts(self._h, _p(out)))
        keys = ["NU", "u_one_term", "u_two_term", "cg_terms", "z_row_extents", "z_outputs", "y_slots",
                "y_slots_za", "K", "nch", "pairs", "atoms"]
        return dict(zip(keys, (int(v) for v in out)))

    def set_kernel_points(self, z_raw: np.ndarray) -> None:
        Z = np.ascontiguousarray(z_raw, dtype=np.float64)
        self._check(self._L.mld_gpu_set_kernel_points(self._h, int(Z.shape[0]), _p(Z)))
        self._dims()

    def tuning(self, mode: int = 0):
        """Launch shape the autotuner chose for the descriptor kernel and the candidates' times."""
        shape = np.zeros(4, np.int32)
        n = ctypes.c_int(16)
        ms = np.zeros(16)
        self._check(self._L.mld_gpu_tuning(self._h, int(mode), _p(shape), ctypes.byref(n), _p(ms)))
        return {"col_tile": int(shape[0]), "ctas_per_sm": int(shape[1]), "sorted_queue": int(shape[2]),
                "tuned": bool(shape[3]), "candidate_ms": [float(v) for v in ms[:n.value]]}

    def solve_info(self):
        it = np.zeros(2, np.int32)
        res = np.zeros(2)
        sh = np.zeros(2)
        rt = ctypes.c_int()
        self._check(self._L.mld_gpu_solve_info(self._h, _p(it), _p(res), _p(sh), ctypes.byref(rt)))
        return {"pcg_iterations": [int(v) for v in it], "pcg_residual": [float(v) for v in res],
                "precond_shift": [float(v) for v in sh], "chol_retries": int(rt.value)}


def gram_rows(method: int, X_ptr: int, x_is_fp32: bool, M: int, D: int, ldx: int, w_ptr: int, y_ptr: int,
              G_ptr: int, rhs_ptr: int = 0, stream: int = 0) -> None:
    """G = X^T W X (and rhs = X^T W y) of device rows given as raw device addresses."""
    L = load()
    err = ctypes.create_string_buffer(512)
    vp = ctypes.c_void_p
    rc = L.mld_gpu_gram_rows(int(method), vp(X_ptr), int(bool(x_is_fp32)), ctypes.c_longlong(M), int(D), int(ldx),
                             vp(w_ptr), vp(y_ptr or None), vp(G_ptr), vp(rhs_ptr or None), vp(stream or None), err,
                             512)
    if rc != 0:
        raise MldError(rc, err.value.decode(errors="replace"))


class Server:
    """Serving loop over the C ABI: submit structures, progress(), collect results."""

    def __init__(self, cfg: MldGpuConfig, w_params: np.ndarray, n_slots: int = 2, max_batch_atoms: int = 200000,
                 hbm_fraction: float = 0.5):
        L = load()
        L.mld_gpu_server_last_error.restype = ctypes.c_char_p
        L.mld_gpu_server_last_error.argtypes = [ctypes.c_void_p]
        L.mld_gpu_server_destroy.restype = None
        L.mld_gpu_server_wait.argtypes = [ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double]
        L.mld_gpu_server_result.argtypes = [ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p, ctypes.c_void_p,
                                            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.mld_gpu_server_create.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong,
                                            ctypes.c_double, ctypes.c_void_p]
        self._L = L
        self._s = ctypes.c_void_p()
        w = np.ascontiguousarray(w_params, dtype=np.float64)
        rc = L.mld_gpu_server_create(ctypes.byref(cfg), _p(w), int(n_slots), int(max_batch_atoms), float(hbm_fraction),
                                     ctypes.byref(self._s))
        if rc != MLD_OK:
            raise MldError(rc, "mld_gpu_server_create failed")
        self._nat = {}

    def _check(self, rc):
        if rc != MLD_OK:
            raise MldError(rc, (self._L.mld_gpu_server_last_error(self._s) or b"").decode())

    def submit(self, pos, cell, types) -> int:
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1)
        cell = np.ascontiguousarray(cell, dtype=np.float64).reshape(-1)
        types = np.ascontiguousarray(types, dtype=np.int32).reshape(-1)
        t = ctypes.c_longlong()
        self._check(self._L.mld_gpu_server_submit(self._s, int(types.shape[0]), _p(pos), _p(cell), _p(types),
                                                  ctypes.byref(t)))
        self._nat[t.value] = int(types.shape[0])
        return t.value

    def progress(self):
        b, q = ctypes.c_int(), ctypes.c_int()
        self._check(self._L.mld_gpu_server_progress(self._s, ctypes.byref(b), ctypes.byref(q)))
        return b.value, q.value

    def result(self, ticket: int):
        nat = self._nat[ticket]
        E, F, S = ctypes.c_double(), np.zeros((nat, 3)), np.zeros(6)
        lat, ready = ctypes.c_double(), ctypes.c_int()
        self._check(self._L.mld_gpu_server_result(self._s, ctypes.c_longlong(ticket), ctypes.byref(E), _p(F), _p(S),
                                                  ctypes.byref(lat), ctypes.byref(ready)))
        if not ready.value:
            return None
        del self._nat[ticket]
        return E.value, F, S, lat.value

    def wait(self, ticket: int, timeout_ms: float = 600000.0):
        nat = self._nat[ticket]
        E, F, S, lat = ctypes.c_double(), np.zeros((nat, 3)), np.zeros(6), ctypes.c_double()
        self._check(self._L.mld_gpu_server_wait(self._s, ctypes.c_longlong(ticket), ctypes.byref(E), _p(F), _p(S),
                                                ctypes.byref(lat), float(timeout_ms)))
        del self._nat[ticket]
        return E.value, F, S, lat.value

    def stats(self):
        b, a, bud = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_double()
        self._check(self._L.mld_gpu_server_stats(self._s, ctypes.byref(b), ctypes.byref(a), ctypes.byref(bud)))
        return {"batches": b.value, "atoms_done": a.value, "budget_bytes": bud.value}

    def admission(self):
        """Admission record: peak estimated bytes on the GPU, per-slot share, largest batch."""
        pk, sh, lg = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        self._check(self._L.mld_gpu_server_admission(self._s, ctypes.byref(pk), ctypes.byref(sh), ctypes.byref(lg)))
        return {"peak_bytes_in_flight": pk.value, "share_bytes": sh.value, "largest_batch_bytes": lg.value}

    def close(self):
        if self._s:
            self._L.mld_gpu_server_destroy(self._s)
            self._s = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
