"""GPU tests of the batched dense symmetric eigensolver (one persistent launch for the first pass, one for
the FP64 refinement): ragged sizes, the leading 8 eigenpairs of each matrix against the known spectrum,
true FP64 residuals recomputed with NumPy (tol 1e-7 of the largest eigenvalue), and the solo mixed-mode
si_eig result of a few of the same matrices (eigenvalues within 1e-7 relative)."""
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


@pytest.fixture(scope="module")
def orc():
    from oracle import ofrr_oracle as o

    return o


def _pack(api, mats):
    import torch

    ns = np.array([m.shape[0] for m in mats], dtype=np.int64)
    offs = np.concatenate([[0], np.cumsum(ns * ns)[:-1]]).astype(np.int64)
    buf = np.concatenate([np.asfortranarray(m).ravel(order="F") for m in mats])
    return torch.as_tensor(buf, device="cuda"), ns, offs


@pytest.mark.parametrize("p16", ["bfloat16", "half"])
def test_batch_sym_eig_ragged(api, orc, p16):
    rng = np.random.default_rng(1)
    sizes = [16, 17, 64, 1024] + list(rng.integers(64, 400, 40))
    mats, lams = [], []
    for i, n in enumerate(sizes):
        A, lam = orc.dense_sym_problem(int(n), seed=100 + i)
        mats.append(A)
        lams.append(lam)
    Ad, ns, offs = _pack(api, mats)
    Xs, ev, res, its, sts = api.batch_sym_eig(Ad, ns, offs, nev=8, block=16, tol=1e-7, p_output=p16)
    assert np.all(sts == 0), (sts, res.max(axis=1))
    for i, A in enumerate(mats):
        lam = lams[i][:8]
        assert np.allclose(ev[i], lam, rtol=1e-7, atol=0), (i, ev[i], lam)
        X = api.to_numpy(Xs[i])
        r = np.linalg.norm(A @ X - X * ev[i][None, :], axis=0) / (np.max(np.abs(ev[i])) * np.linalg.norm(X, axis=0))
        assert np.max(r) <= 1e-7 * 1.01, (i, r)
        assert np.all(r <= res[i] * (1 + 1e-6) + 1e-15)


def test_batch_matches_solo_si_eig(api, orc):
    mats = [orc.dense_sym_problem(n, seed=7 + n)[0] for n in (96, 200, 333)]
    Ad, ns, offs = _pack(api, mats)
    Xs, ev, res, its, sts = api.batch_sym_eig(Ad, ns, offs, nev=8, block=16, tol=1e-7)
    assert np.all(sts == 0)
    for i, A in enumerate(mats):
        V, d, info = api.subspace_iter_eig(A, A.shape[0], 16, "single", "bfloat16", maxiter=400, step_size=2,
                                           mode="mixed", tol=1e-7, nev=8, symmetric=True)
        assert info.status == 0
        assert np.allclose(ev[i], d[:8], rtol=1e-7, atol=0)


def test_batch_rejects_bad_sizes(api, orc):
    import torch

    A = torch.zeros(2000 * 2000, dtype=torch.float64, device="cuda")
    with pytest.raises(Exception):
        api.batch_sym_eig(A, [2000], [0], nev=8)  # above the 1024 held in shared memory
    with pytest.raises(Exception):
        api.batch_sym_eig(A, [8], [0], nev=8)  # below the block width
