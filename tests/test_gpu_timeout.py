"""The bounded-wait error path of the tensor-core pipelines.

A test hook makes the tensor-core Gram's producer warp issue no loads, so the MMA and epilogue
warps wait on barriers that nothing completes.  Every such wait is bounded (here shortened to
about a millisecond): the kernel records the expiry, frees its tensor memory and returns, and
the fit fails with MLD_ERR_TIMEOUT.  No fault, trap or hang is involved, and the same handle
must fit normally afterwards.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHORT_WAIT = 2_000_000  # SM clocks, about 1 ms


def _mixed_handle():
    from mld_gb300 import _lib, synth
    ds = synth.fe_bcc_batched(n_struct=4, nmin=16, nmax=120, seed=13)
    c = _lib.default_config()
    c.j_max, c.r_cut, c.lambda_krr, c.precision = 4.0, 4.7, 1e-8, _lib.MIXED
    h = _lib.Handle(c)
    nat, pos, cell, types = ds.arrays()
    h.set_structures(nat, pos, cell, types)
    E, F, S, has = ds.labels()
    h.set_labels(E, F, S, has, np.ones((len(nat), 3)))
    return h


def test_pipeline_wait_expiry_reports_timeout_and_handle_recovers(lib):
    from mld_gb300 import _lib
    L = _lib.load()
    L.mld_gpu_test_pipeline_timeout.argtypes = [ctypes.c_int, ctypes.c_longlong]
    h = _mixed_handle()
    try:
        w_ref, r_ref = h.fit()
        assert L.mld_gpu_test_pipeline_timeout(1, SHORT_WAIT) == 0
        try:
            with pytest.raises(_lib.MldError) as ei:
                h.fit()
            assert ei.value.code == 9  # MLD_ERR_TIMEOUT
        finally:
            assert L.mld_gpu_test_pipeline_timeout(0, 0) == 0
        # the context and the handle stay usable: the next fit is the normal one (the mixed
        # method's tensor-core Gram adds its row splits in arrival order, so not bitwise)
        w, r = h.fit()
        assert np.abs(r - r_ref).max() <= 1e-6 * np.abs(r_ref).max()
        assert np.abs(w - w_ref).max() <= 1e-5 * np.abs(w_ref).max()
    finally:
        h.close()
