"""mld_gpu_descriptors_noalloc: descriptors of one structure without device allocation.

This entry point is for callers that cannot call cudaMalloc: MD steps, serving loops, and
hosts whose device memory belongs to another runtime's pool.  They hand over device pointers
they already own, and the library's scratch comes from a static device array.  The test calls
the entry point through the C ABI on two structures in a row, so the shared array is reused.
It checks each result against the regular entry point (mld_gpu_descriptors) with the
tolerances used by the other parity tests.  Device buffers for the test inputs come from
PyTorch: the test owns them, the entry point does not allocate.  The file sorts last, so a run
that stops at the first failure has already run the other tests.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {0: 1e-10, 1: 2e-5}


def _reference(cfg, pos, cell, types):
    from mld_gb300 import _lib
    with _lib.Handle(cfg) as h:
        h.set_structures([pos.shape[0]], pos, cell[None], types)
        B, _ = h.descriptors()
    return B


@pytest.mark.parametrize("precision", [0, 1])
def test_noalloc_matches_regular_entry_point(fit17, precision):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from mld_gb300 import _lib
    L = _lib.load()
    cfg = _lib.default_config()
    cfg.j_max, cfg.r_cut, cfg.precision = 4.0, 4.7, precision
    err = ctypes.create_string_buffer(256)
    # two structures in a row: a small box (periodic images) then a large box (minimum image)
    for idx in (0, 9):
        pos = np.ascontiguousarray(fit17[f"pos_{idx}"], dtype=np.float64)
        cell = np.ascontiguousarray(fit17[f"cell_{idx}"], dtype=np.float64)
        types = np.ascontiguousarray(fit17[f"types_{idx}"], dtype=np.int32)
        nat = pos.shape[0]
        want = _reference(cfg, pos, cell, types)
        d_pos = torch.from_numpy(pos.reshape(-1)).cuda()
        d_types = torch.from_numpy(types).cuda()
        d_B = torch.full((nat * want.shape[1],), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        rc = L.mld_gpu_descriptors_noalloc(ctypes.byref(cfg), nat, ctypes.c_void_p(d_pos.data_ptr()),
                                           cell.ctypes.data_as(ctypes.c_void_p), ctypes.c_void_p(d_types.data_ptr()),
                                           ctypes.c_void_p(d_B.data_ptr()), None, err, len(err))
        assert rc == 0, err.value.decode()
        torch.cuda.synchronize()
        got = d_B.cpu().numpy().reshape(nat, -1)
        rel = np.abs(got - want).max() / np.abs(want).max()
        assert rel <= TOL[precision], (idx, rel)
        # golden descriptors of MILADY's fit17 test as well
        ref = fit17[f"B_{idx}"]
        assert np.abs(got - ref).max() / np.abs(ref).max() <= TOL[precision]


@pytest.mark.parametrize("precision", [0, 1])
def test_noalloc_alternating_j_max_on_a_side_stream(fit17, precision):
    """Calls that change j_max (3, 4, 3) re-upload the tables into the shared array.  They are
    queued on a non-blocking side stream, with no host synchronisation between them, and every
    output buffer is read only at the end: each result must still equal the regular entry
    point's."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from mld_gb300 import _lib
    L = _lib.load()
    err = ctypes.create_string_buffer(256)
    idx = 9
    pos = np.ascontiguousarray(fit17[f"pos_{idx}"], dtype=np.float64)
    cell = np.ascontiguousarray(fit17[f"cell_{idx}"], dtype=np.float64)
    types = np.ascontiguousarray(fit17[f"types_{idx}"], dtype=np.int32)
    nat = pos.shape[0]
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        d_pos = torch.from_numpy(pos.reshape(-1)).cuda()
        d_types = torch.from_numpy(types).cuda()
    cfgs, wants, outs = [], [], []
    for j_max in (3.0, 4.0, 3.0):
        cfg = _lib.default_config()
        cfg.j_max, cfg.r_cut, cfg.precision = j_max, 4.7, precision
        cfgs.append(cfg)
        wants.append(_reference(cfg, pos, cell, types))
        with torch.cuda.stream(side):
            outs.append(torch.full((nat * wants[-1].shape[1],), float("nan"), dtype=torch.float64,
                                   device="cuda"))
    torch.cuda.synchronize()
    for cfg, d_B in zip(cfgs, outs):
        rc = L.mld_gpu_descriptors_noalloc(ctypes.byref(cfg), nat, ctypes.c_void_p(d_pos.data_ptr()),
                                           cell.ctypes.data_as(ctypes.c_void_p), ctypes.c_void_p(d_types.data_ptr()),
                                           ctypes.c_void_p(d_B.data_ptr()), ctypes.c_void_p(side.cuda_stream), err,
                                           len(err))
        assert rc == 0, err.value.decode()
    side.synchronize()
    for d_B, want in zip(outs, wants):
        got = d_B.cpu().numpy().reshape(nat, -1)
        rel = np.abs(got - want).max() / np.abs(want).max()
        assert rel <= TOL[precision], rel


def test_noalloc_rejects_oversized_input():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from mld_gb300 import _lib
    L = _lib.load()
    cfg = _lib.default_config()
    cfg.j_max, cfg.r_cut = 4.0, 4.7
    err = ctypes.create_string_buffer(256)
    cell = np.eye(3) * 100.0
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")  # the size check rejects before any access
    ptr = ctypes.c_void_p(buf.data_ptr())
    rc = L.mld_gpu_descriptors_noalloc(ctypes.byref(cfg), 16384 + 1, ptr, cell.ctypes.data_as(ctypes.c_void_p),
                                       ptr, ptr, None, err, len(err))
    assert rc == 8 and b"MLD_NOALLOC_MAX_ATOMS" in err.value
