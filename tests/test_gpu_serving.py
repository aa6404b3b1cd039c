"""Serving loop: continuous batching over several evaluation slots.  Each structure's energy,
forces and stress must be the same whether it is evaluated alone or in a mixed batch (within
1e-5 relative for the mixed method, whose FP32 rows are assembled with atomics whose order
depends on the batch partners; 1e-12 for the plain method), and must agree with the handle's
prediction entry point."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _fit(precision, order=1):
    from mld_gb300 import _lib, synth
    ds = synth.fe_bcc_batched(n_struct=6, nmin=16, nmax=150, seed=31)
    c = _lib.default_config()
    c.j_max, c.r_cut, c.lambda_krr, c.precision, c.mld_order = (4.0 if order == 1 else 1.5), 4.7, 1e-6, precision, order
    with _lib.Handle(c) as h:
        nat, pos, cell, types = ds.arrays()
        h.set_structures(nat, pos, cell, types)
        E, F, S, has = ds.labels()
        h.set_labels(E, F, S, has, np.ones((len(nat), 3)))
        w, _ = h.fit()
    return c, w


def _requests(n=10, seed=5):
    from mld_gb300 import synth
    ds = synth.fe_bcc_batched(n_struct=n, nmin=16, nmax=400, seed=seed)
    return ds.structures


def _rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("precision,order,tol", [(1, 1, 1e-5), (0, 1, 1e-12), (1, 2, 1e-5)])
def test_alone_equals_mixed_batch(lib, precision, order, tol):
    from mld_gb300 import _lib
    c, w = _fit(precision, order)
    reqs = _requests()
    with _lib.Server(c, w, n_slots=2, max_batch_atoms=100000, hbm_fraction=0.2) as srv:
        alone = []
        for s in reqs:
            t = srv.submit(s.positions, s.cell, s.types)
            alone.append(srv.wait(t))
        tickets = [srv.submit(s.positions, s.cell, s.types) for s in reqs]
        mixed = [srv.wait(t) for t in tickets]
        st = srv.stats()
    assert st["batches"] < 2 * len(reqs)  # the second round was batched
    for (Ea, Fa, Sa, _), (Em, Fm, Sm, _) in zip(alone, mixed):
        assert abs(Ea - Em) <= tol * max(abs(Ea), 1.0)
        assert _rel(Fm, Fa) <= tol
        assert _rel(Sm, Sa) <= max(tol, 1e-12)
    # the handle's prediction entry point gives the same results
    with _lib.Handle(c) as h:
        nat = np.array([s.nat for s in reqs], np.int32)
        h.set_structures(nat, np.concatenate([s.positions for s in reqs]), np.stack([s.cell for s in reqs]),
                         np.concatenate([s.types for s in reqs]))
        E, F, S = h.predict(w)
    off = np.cumsum([0] + [s.nat for s in reqs])
    for i, (Ea, Fa, Sa, _) in enumerate(alone):
        assert abs(E[i] - Ea) <= tol * max(abs(Ea), 1.0)
        assert _rel(Fa, F[off[i]:off[i + 1]]) <= tol


def test_server_rejects_bad_requests(lib):
    from mld_gb300 import _lib
    c, w = _fit(1)
    with _lib.Server(c, w, n_slots=1) as srv:
        with pytest.raises(_lib.MldError):
            srv.submit(np.zeros((0, 3)), np.eye(3), np.zeros(0, np.int32))
