"""Per-solve tracing: one JSON line per solve with the phase breakdown (CUDA events on the context's
stream); tracing does not change results."""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def api(built_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from mixedprecisionofrr_gb300 import api as a

    return a


def _problem(m=600, n=200, seed=5):
    rng = np.random.default_rng(seed)
    U, _ = np.linalg.qr(rng.standard_normal((m, n)))
    V, _ = np.linalg.qr(rng.standard_normal((n, n)))
    s = 1e-3 ** (np.arange(n) / (n - 1))
    return (U * s) @ V.T


@pytest.mark.parametrize("mode", ["mixed", "fp64"])
def test_trace_records_phases_and_keeps_results(api, tmp_path, mode):
    A = _problem()
    Ad = api.to_device_cm(A, api.PREC["double"])
    kw = dict(maxiter=40, step_size=4, mode=mode, tol=1e-8, nev=8, check_every=1, generalized_tol=0.0)
    _, s0, _, info0 = api.subspace_iter_svd(Ad, 600, 200, 24, "single", "half", **kw)
    ctx = api.context()
    path = tmp_path / "trace.jsonl"
    ctx.set_trace(path)
    try:
        _, s1, _, info1 = api.subspace_iter_svd(Ad, 600, 200, 24, "single", "half", **kw)
    finally:
        ctx.set_trace(None)
    assert np.array_equal(s0, s1) and info0.iterations == info1.iterations
    recs = [json.loads(line) for line in path.read_text().splitlines()]
    assert len(recs) == 1
    r = recs[0]
    assert r["solver"] == "si_svd" and r["m"] == 600 and r["n"] == 200 and r["status"] == 0
    assert r["iterations"] == info1.iterations and r["launches"] > 0 and r["total_ms"] > 0
    names = set(r["phases"])
    assert {"power.f64", "basis.f64", "rr.f64", "check.f64"} <= names
    if mode == "mixed":
        assert {"power.16bit", "basis.16bit", "rr.16bit", "prepare.f64"} <= names
    assert sum(p["ms"] for p in r["phases"].values()) <= r["total_ms"] * 1.01 + 0.05
    # nothing is recorded once tracing is off
    api.subspace_iter_svd(Ad, 600, 200, 24, "single", "half", **kw)
    assert len(path.read_text().splitlines()) == 1
