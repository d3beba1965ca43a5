"""Solve engine: batched si_eig (many small dense symmetric problems, the C4 shape scaled down) and
the serving queue (concurrent requests, admission by an HBM budget, results independent of the mix)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def api(built_lib):
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from mixedprecisionofrr_gb300 import api as a

    return a


def sym_problem(n, seed, ratio=0.9):
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    lam = ratio ** np.arange(n)
    return (Q * lam) @ Q.T, lam


def test_batch_si_eig(api):
    probs = [sym_problem(n, 100 + i) for i, n in enumerate([64, 96, 128, 160, 200, 256, 300, 72] * 3)]
    srv = api.Server(workers=4)
    try:
        Vs, vals, sts = api.batch_si_eig(srv, [A for A, _ in probs], 16, mode="mixed", tol=1e-8, nev=8, maxiter=300,
                                         step_size=4, p_output="bfloat16")
        assert list(sts) == [0] * len(probs)
        for (A, lam), V, d in zip(probs, Vs, vals):
            assert np.allclose(d[:8], lam[:8], rtol=1e-9)
            X = api.to_numpy(V)[:, :8]
            r = np.linalg.norm(A @ X - X * d[:8], axis=0) / np.linalg.norm(X, axis=0)
            assert np.max(r) <= 1e-8
        s = srv.stats()
        assert s["completed"] == len(probs) and s["failed"] == 0
    finally:
        srv.close()


def test_serve_results_do_not_depend_on_the_mix(api):
    A, lam = sym_problem(256, 7)
    B = np.random.default_rng(3).standard_normal((600, 150))
    srv = api.Server(workers=4)
    try:
        t = srv.submit_si_eig(A, 16, mode="mixed", tol=1e-8, nev=8, maxiter=300)
        st, lat, alone = srv.wait(t)
        assert st == 0
        tickets = []
        for i in range(6):
            tickets.append(srv.submit_si_svd(B, 16, mode="mixed", tol=1e-8, nev=8, maxiter=300))
            if i == 3:
                mine = srv.submit_si_eig(A, 16, mode="mixed", tol=1e-8, nev=8, maxiter=300)
        st, lat, mixed = srv.wait(mine)
        for tk in tickets:
            s2, _, _ = srv.wait(tk)
            assert s2 == 0
        assert st == 0
        # bit-identical eigenvalues and vectors, alone and among other requests
        assert np.array_equal(alone[2], mixed[2])
        assert np.array_equal(api.to_numpy(alone[1]), api.to_numpy(mixed[1]))
        assert np.allclose(alone[2][:8], lam[:8], rtol=1e-9)
    finally:
        srv.close()


def test_serve_budget_admission_and_poll(api):
    A, lam = sym_problem(128, 9)
    srv = api.Server(workers=3, hbm_budget_bytes=1)  # every request exceeds the budget: one at a time
    try:
        ts = [srv.submit_si_eig(A, 8, mode="fp64", tol=1e-9, nev=4, maxiter=300) for _ in range(5)]
        for t in ts:
            done, st = srv.poll(t)
            assert done in (False, True)
        outs = [srv.wait(t) for t in ts]
        assert all(o[0] == 0 for o in outs)
        for o in outs:  # outputs: (operator, V, values, resid, info)
            assert np.allclose(o[2][2][:4], lam[:4], rtol=1e-9)
        s = srv.stats()
        assert s["completed"] == 5 and s["queued"] == 0 and s["charged_bytes"] == 0
    finally:
        srv.close()
