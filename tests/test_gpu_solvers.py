"""GPU parity tests of the solvers against the CPU oracle (same start blocks, same precisions),
plus convergence to the analytic spectra at full benchmark sizes."""
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden"


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


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD / "golden.npz")


def test_si_eig_reference_double_golden(api, orc, gold):
    L = orc.laplacian_2d(20)
    V, d, info = api.subspace_iter_eig(api.CsrMatrix(L), L.shape[0], 16, "double", maxiter=8, step_size=2,
                                      V0=gold["si_V0"])
    assert np.allclose(d, gold["si_d_double"], rtol=1e-11, atol=1e-11)
    assert info.iterations == 8


def test_si_eig_reference_half_golden(api, orc, gold):
    """half storage / single compute (the reference's 'half' experiment, +tests/+test2/test.m:55-60)."""
    L = orc.laplacian_2d(20)
    V, d, info = api.subspace_iter_eig(api.CsrMatrix(L), L.shape[0], 16, "single", "half", maxiter=8, step_size=2,
                                      V0=gold["si_V0"])
    # element-wise steps are bit-exact; FP32 sums differ in order -> agreement at the half-precision level
    assert np.allclose(d[:8], gold["si_d_half"][:8], rtol=5e-3)


def test_si_eig_dense_single_vs_oracle(api, orc):
    A, lam = orc.dense_sym_problem(300, seed=3)
    V0 = orc.randn_block(1, 300, 12)
    V, d, _ = api.subspace_iter_eig(A, 300, 12, "single", maxiter=6, step_size=2, V0=V0)
    Vo, do = orc.subspace_iter_eig(A, 300, 12, "single", maxiter=6, step_size=2, V0=V0)
    assert np.allclose(d[:6], do[:6], rtol=2e-5)


def test_rr_eig_vs_oracle(api, orc):
    A, lam = orc.dense_sym_problem(200, seed=4)
    V = orc.randn_block(3, 200, 10)
    for gen in (False, True):
        Vg, d = api.eig_rr(A, V, "double", use_generalized=gen, generalized_tol=1e-10)
        Vo, do = orc.eig_rr(A, V, "double", use_generalized=gen, generalized_tol=1e-10)
        assert np.allclose(d, do, rtol=1e-10, atol=1e-12)
        # Ritz vectors agree up to sign
        X, Xo = api.to_numpy(Vg), Vo
        cos = np.abs(np.sum(X * Xo, 0)) / (np.linalg.norm(X, axis=0) * np.linalg.norm(Xo, axis=0))
        assert np.min(cos) > 1 - 1e-9


def test_rr_svd_vs_oracle(api, orc):
    A, U, s, V = orc.dense_svd_problem(400, 80, seed=6, smin=1e-3)
    P = orc.randn_block(1, 400, 12)
    Q = orc.randn_block(2, 80, 12)
    Ug, sg, Vg = api.svd_rr(A, P, Q, "double", generalized_tol=1e-12)
    Uo, so, Vo = orc.svd_rr(A, P, Q, "double", use_generalized=True, generalized_tol=1e-12)
    assert np.allclose(sg, so, rtol=1e-9, atol=1e-12)


def test_si_svd_double_vs_oracle(api, orc):
    A, U, s, V = orc.dense_svd_problem(500, 100, seed=8, smin=1e-3)
    V0 = orc.randn_block(42, 100, 16)
    Ug, sg, Vg, info = api.subspace_iter_svd(A, 500, 100, 16, "double", maxiter=6, step_size=2, V0=V0)
    Uo, so, Vo = orc.subspace_iter_svd(A, 500, 100, 16, "double", maxiter=6, step_size=2, V0=V0)
    assert np.allclose(sg, so, rtol=1e-10, atol=1e-13)


def test_arnoldi_hess_golden_and_pivots(api, orc, gold):
    L = orc.laplacian_2d(20)
    X, d, info = api.arnoldi_hess_eig(api.CsrMatrix(L), L.shape[0], 6, "double", maxiter=61, kdim=30, v0=gold["kr_v0"])
    assert np.allclose(d, gold["kr_d_double"], rtol=1e-10)


def test_arnoldi_hess_half_vs_oracle(api, orc):
    L = orc.laplacian_2d(12, 9)
    Ac = orc.sparse2csr(L)
    v0 = orc.randn_block(9, L.shape[0], 1)[:, 0]
    X, d, info = api.arnoldi_hess_eig(api.CsrMatrix(L), L.shape[0], 3, "single", "half", maxiter=21, kdim=20, v0=v0)
    Xo, do, inf = orc.arnoldi_hess_eig(Ac, L.shape[0], 3, "single", "half", maxiter=21, kdim=20, v0=v0, symmetric=True)
    assert np.allclose(d, do, rtol=5e-3)


def test_si_eig_laplacian_converges_fp64(api, orc):
    """32x32 Dirichlet Laplacian, 8 largest pairs, block 16, tol 1e-10 (the C1 shape scaled down)."""
    L = orc.laplacian_2d(32)
    V, d, info = api.subspace_iter_eig(api.CsrMatrix(L), L.shape[0], 16, "double", maxiter=400, step_size=8,
                                      mode="fp64", tol=1e-10, nev=8, check_every=5)
    assert info.status == 0, info
    assert np.allclose(d[:8], orc.laplacian_2d_eigs(32)[:8], rtol=1e-9)
    assert np.max(info.residuals[:8]) <= 1e-10


def test_si_svd_geometric_converges_fp64(api, orc):
    A, U, s, V = orc.dense_svd_problem(2048, 512, seed=42, smin=1e-6)
    Ug, sg, Vg, info = api.subspace_iter_svd(A, 2048, 512, 48, "double", maxiter=60, step_size=2, mode="fp64",
                                             tol=1e-8, nev=16, check_every=2)
    assert info.status == 0
    assert np.allclose(sg[:16], s[:16], rtol=1e-9)
    r = orc.svd_residual_norms(A, api.to_numpy(Ug)[:, :16], sg[:16], api.to_numpy(Vg)[:, :16])
    assert np.max(r) < 1e-8
