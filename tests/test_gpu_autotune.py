"""Launch-shape autotuner of the descriptor kernel and the CUDA graph of the row-assembly stage.

The first fit of a large enough batch times every candidate shape once (column tile 4 or 2,
persistent CTAs per SM, longest-first or index-order atom queue) and keeps the fastest; the
second fit captures the stage (descriptor kernel, reverse pairs, row gathers) as a CUDA graph
and later fits replay it.  Every shape and the graph give bitwise the same rows and fit.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [0, 1])
def test_tuner_and_graph_keep_results_bitwise(lib, precision):
    from mld_gb300 import _lib, synth
    ds = synth.fe_bcc_batched(n_struct=70, nmin=100, nmax=300, seed=51)
    nat, pos, cell, types = ds.arrays()
    assert nat.sum() >= 64 * 152  # enough atoms per SM to tune
    E, F, S, has = ds.labels()
    c = _lib.default_config()
    c.j_max, c.r_cut, c.lambda_krr, c.precision = 4.0, 4.7, 1e-8, precision
    with _lib.Handle(c) as h:
        h.set_structures(nat, pos, cell, types)
        h.set_labels(E, F, S, has, np.ones((len(nat), 3)))
        fits = [h.fit() for _ in range(3)]  # tuning run, graph capture, graph replay
        A, _, _ = h.design_matrix()
        t = h.tuning(0)
    assert t["tuned"] and len(t["candidate_ms"]) == 8
    assert t["col_tile"] in (2, 4) and t["sorted_queue"] in (0, 1)
    assert min(t["candidate_ms"]) > 0
    for w, r in fits[1:]:
        if precision == 0:
            assert np.array_equal(w, fits[0][0]) and np.array_equal(r, fits[0][1])
        else:  # the tensor-core Gram adds its row splits in arrival order
            assert np.abs(w - fits[0][0]).max() <= 1e-6 * np.abs(fits[0][0]).max()
    # rows of a fresh handle (its first call tunes again) are the same
    with _lib.Handle(c) as h2:
        h2.set_structures(nat, pos, cell, types)
        h2.set_labels(E, F, S, has, np.ones((len(nat), 3)))
        A2, _, _ = h2.design_matrix()
    assert np.array_equal(A, A2)
