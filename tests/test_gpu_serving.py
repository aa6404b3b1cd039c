"""Serving loop: continuous batching over several evaluation slots.  Each structure's energy,
forces and stress must be the same, bitwise, whether it is evaluated alone or in a mixed batch
(every sum runs over the structure's own atoms and pairs in a fixed order), and must agree with
the handle's prediction entry point within the method's tolerance (1e-5 mixed, 1e-12 plain).
Admission keeps the estimated bytes on the GPU within the server's HBM budget."""
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
        assert Ea == Em
        assert np.array_equal(Fm, Fa)
        assert np.array_equal(Sm, Sa)
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


def test_admission_keeps_a_large_request_alone(lib):
    """A request larger than the per-slot share but within the budget waits until every slot is
    idle and runs alone, so the estimated bytes in flight never exceed the budget."""
    from mld_gb300 import _lib, synth
    torch = pytest.importorskip("torch")
    c, w = _fit(1)
    big = synth.fe_bcc_batched(n_struct=1, nmin=900, nmax=1000, seed=41).structures[0]
    small = synth.fe_bcc_batched(n_struct=24, nmin=60, nmax=120, seed=43).structures
    # size of the big request on its own, from a first server with a generous budget
    with _lib.Server(c, w, n_slots=3, hbm_fraction=0.5) as srv:
        srv.wait(srv.submit(big.positions, big.cell, big.types))
        big_bytes = srv.admission()["largest_batch_bytes"]
        free = srv.stats()["budget_bytes"] / 0.5
    # budget 1.5x the big request: share = 0.5x, so the big one exceeds a slot's share
    frac = 1.5 * big_bytes / free
    with _lib.Server(c, w, n_slots=3, max_batch_atoms=100000, hbm_fraction=frac) as srv:
        st = srv.stats()
        adm = srv.admission()
        assert adm["share_bytes"] < big_bytes < st["budget_bytes"]
        t_small1 = [srv.submit(s.positions, s.cell, s.types) for s in small[:12]]
        t_big = srv.submit(big.positions, big.cell, big.types)
        t_small2 = [srv.submit(s.positions, s.cell, s.types) for s in small[12:]]
        res = [srv.wait(t) for t in t_small1 + [t_big] + t_small2]
        adm = srv.admission()
        st = srv.stats()
    assert adm["peak_bytes_in_flight"] <= st["budget_bytes"]
    assert adm["largest_batch_bytes"] >= big_bytes
    # the big request's result equals its evaluation alone
    with _lib.Server(c, w, n_slots=1, hbm_fraction=0.5) as srv:
        Eb, Fb, Sb, _ = srv.wait(srv.submit(big.positions, big.cell, big.types))
    E, F, S, _ = res[12]
    assert E == Eb and np.array_equal(F, Fb) and np.array_equal(S, Sb)
