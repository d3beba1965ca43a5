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


@pytest.mark.parametrize("gen", [False, True])
def test_rr_eig_nonsymmetric_vs_oracle(api, orc, gen):
    """Nonsymmetric projected pencils (convection-diffusion operator) on an FP64 basis: the Hessenberg-QR
    eigensolver runs in FP64 after the FP64 Cholesky reduction; Ritz values (real parts) within 1e-10 of
    ||C||, real Ritz pairs satisfy the projected equation to 1e-9."""
    A = orc.convdiff_3d(6).toarray()  # n = 216, real spectrum
    V = orc.randn_block(5, 216, 24)
    Vg, d = api.eig_rr(A, V, "double", use_generalized=gen, generalized_tol=1e-10, symmetric=False)
    Vo, do = orc.eig_rr(A, V, "double", use_generalized=gen, generalized_tol=1e-10, symmetric=False)
    scale = np.max(np.abs(do))
    assert np.max(np.abs(d - do)) <= 1e-10 * scale
    # every real Ritz pair satisfies the projected equation to FP64 accuracy: G u = d M u with x = V u
    X = api.to_numpy(Vg)
    Uc = np.linalg.lstsq(V, X, rcond=None)[0]
    G = V.T @ A @ V
    M = V.T @ V + 1e-10 * np.eye(V.shape[1]) if gen else np.eye(V.shape[1])
    R = G @ Uc - (M @ Uc) * d[None, :]
    import scipy.linalg as sla

    w = sla.eig(G, M, right=False)
    w = w[np.argsort(-w.real, kind="stable")]
    real = np.abs(w.imag) <= 1e-9 * scale  # real parts of complex pairs satisfy no real equation
    assert real.sum() >= 4
    assert np.max(np.abs(R[:, real])) <= 1e-9 * scale * np.max(np.abs(M @ Uc))


def test_rr_eig_nonsymmetric_complex_pairs(api, orc):
    """A rotation-dominated operator with complex Ritz values: real parts match the oracle."""
    rng = np.random.default_rng(11)
    n = 120
    B = rng.standard_normal((n, n))
    A = B - B.T + np.diag(np.linspace(0.0, 1.0, n))  # skew part gives complex pairs
    V = orc.randn_block(8, n, 40)
    Vg, d = api.eig_rr(A, V, "double", use_generalized=False, symmetric=False)
    Vo, do = orc.eig_rr(A, V, "double", use_generalized=False, symmetric=False)
    assert np.max(np.abs(np.sort(d) - np.sort(do))) <= 1e-10 * np.max(np.abs(np.linalg.eigvals(V.T @ A @ V)))


@pytest.mark.parametrize("n,p", [(31, 12), (65, 24), (90, 40)])
def test_invariant_subspace_sign_function(api, orc, n, p):
    """The restart block of the nonsymmetric thick-restart Krylov path: the invariant subspace of the pencil
    (G, M) for its eigenvalues with real part above sigma, from the matrix sign function, equals the
    sorted real Schur subspace computed by SciPy (largest principal-angle sine below 1e-9)."""
    import scipy.linalg as sla

    rng = np.random.default_rng(n)
    lam = np.sort(rng.uniform(1.0, 100.0, n))[::-1]
    lam[p:] *= 0.9  # a gap after the p-th eigenvalue
    X = rng.standard_normal((n, n))
    G0 = X @ np.diag(lam) @ np.linalg.inv(X)  # non-normal, real spectrum
    B = rng.standard_normal((n, n))
    M = B @ B.T / n + np.eye(n)
    Lc = np.linalg.cholesky(M)
    G = Lc @ G0 @ Lc.T  # so that L^-1 G L^-T = G0
    sigma = 0.5 * (lam[p - 1] + lam[p])
    Y = api.debug_invariant_subspace(G, M, sigma, p)
    T, S, sdim = sla.schur(G0, output="real", sort=lambda x, y: x > sigma)
    assert sdim == p
    Yref = sla.solve_triangular(Lc.T, S[:, :p], lower=False)
    Q1, _ = np.linalg.qr(Y)
    Q2, _ = np.linalg.qr(Yref)
    sin_max = np.linalg.norm(Q1 - Q2 @ (Q2.T @ Q1), 2)  # the largest principal-angle sine
    assert sin_max <= 1e-9


def test_arnoldi_hess_nonsymmetric_vs_oracle(api, orc):
    """Hessenberg-process Krylov with restarts on the (nonsymmetric) convection-diffusion operator."""
    A = orc.convdiff_3d(8)
    Ac = orc.sparse2csr(A)
    v0 = orc.randn_block(13, A.shape[0], 1)[:, 0]
    X, d, info = api.arnoldi_hess_eig(api.CsrMatrix(A), A.shape[0], 4, "double", maxiter=61, kdim=30, v0=v0,
                                      symmetric=False)
    Xo, do, inf = orc.arnoldi_hess_eig(Ac, A.shape[0], 4, "double", maxiter=61, kdim=30, v0=v0, symmetric=False)
    assert np.max(np.abs(d - do)) <= 1e-5 * np.max(np.abs(do))


@pytest.mark.parametrize("symmetric", [True, False])
def test_arnoldi_mgs_vs_oracle(api, orc, symmetric):
    """Orthogonal MGS Arnoldi with re-orthogonalisation (the FP64 comparison path) on the GPU."""
    A = orc.laplacian_2d(14) if symmetric else orc.convdiff_3d(7)
    Ac = orc.sparse2csr(A)
    v0 = orc.randn_block(17, A.shape[0], 1)[:, 0]
    X, d, info = api.arnoldi_mgs_eig(api.CsrMatrix(A), A.shape[0], 4, "double", maxiter=41, kdim=20, v0=v0,
                                     symmetric=symmetric)
    Xo, do = orc.arnoldi_mgs_eig(Ac, A.shape[0], 4, "double", maxiter=41, kdim=20, v0=v0, symmetric=symmetric)
    tol = 1e-10 if symmetric else 1e-5
    assert np.max(np.abs(d - do)) <= tol * np.max(np.abs(do))


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


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_si_eig_laplacian_c1_full(api, orc, mode):
    """The C1 workload at full size: 64x64 Dirichlet Laplacian (n = 4096, CSR FP64), block 16, top 8,
    tol 1e-10, against the analytic spectrum (the top 8 close a multiplet)."""
    L = orc.laplacian_2d(64)
    V, d, info = api.subspace_iter_eig(api.CsrMatrix(L), L.shape[0], 16, "double", maxiter=2000, step_size=8,
                                      mode=mode, tol=1e-10, nev=8, check_every=10)
    assert info.status == 0, info
    assert np.allclose(d[:8], orc.laplacian_2d_eigs(64)[:8], rtol=1e-10)
    assert np.max(info.residuals[:8]) <= 1e-10
    X = api.to_numpy(V)[:, :8]
    r = np.linalg.norm(L @ X - X * d[:8], axis=0) / np.linalg.norm(X, axis=0) / 8.0  # ||L|| < 8
    assert np.max(r) <= 1e-10


def test_si_svd_geometric_converges_fp64(api, orc):
    A, U, s, V = orc.dense_svd_problem(2048, 512, seed=42, smin=1e-6)
    Ug, sg, Vg, info = api.subspace_iter_svd(A, 2048, 512, 48, "double", maxiter=60, step_size=2, mode="fp64",
                                             tol=1e-8, nev=16, check_every=2)
    assert info.status == 0
    assert np.allclose(sg[:16], s[:16], rtol=1e-9)
    r = orc.svd_residual_norms(A, api.to_numpy(Ug)[:, :16], sg[:16], api.to_numpy(Vg)[:, :16])
    assert np.max(r) < 1e-8


def test_si_svd_mixed_dense_certified(api, orc):
    """The benchmark path at a quarter of its size: dense 4096 x 1024 geometric-spectrum SVD, mixed
    mode (16-bit bases, then FP64 emulated on the tensor cores with certified checks), tol 1e-8.
    The singular values match the truth, the true FP64 residuals (NumPy) meet tol, and every reported
    residual bounds the true one (the certification is an upper bound, never an estimate below)."""
    A, U, s, V = orc.dense_svd_problem(4096, 1024, seed=7, smin=1e-6)
    Ug, sg, Vg, info = api.subspace_iter_svd(A, 4096, 1024, 64, "single", "half", maxiter=80, step_size=6,
                                             mode="mixed", tol=1e-8, nev=16, check_every=1, generalized_tol=0.0)
    assert info.status == 0, info
    assert np.allclose(sg[:16], s[:16], rtol=1e-9)
    r = orc.svd_residual_norms(A, api.to_numpy(Ug)[:, :16], sg[:16], api.to_numpy(Vg)[:, :16])
    assert np.max(r) <= 1e-8
    assert np.all(r <= info.residuals[:16] * (1 + 1e-6) + 1e-15)


@pytest.mark.parametrize("block,step,step64", [(64, 6, 0), (128, 8, 0), (64, 6, 9)])
def test_si_svd_mixed_benchmark_size(api, orc, block, step, step64):
    """The benchmark configuration itself: dense 8192 x 2048 geometric-spectrum SVD (seed 42, the bench's
    problem), top 32 triplets, mixed mode, tol 1e-8, at three of the autotuner's block / power-step
    choices (the last with its own FP64-phase power steps).  The true FP64 residuals computed here with
    NumPy meet tol and are bounded by the reported (certified) residuals; the singular values match the
    construction to 1e-9 relative."""
    A, U, s, V = orc.dense_svd_problem(8192, 2048, seed=42, smin=1e-6)
    Ug, sg, Vg, info = api.subspace_iter_svd(A, 8192, 2048, block, "single", "half", maxiter=80, step_size=step,
                                             mode="mixed", tol=1e-8, nev=32, check_every=1, generalized_tol=0.0,
                                             step_size_f64=step64)
    assert info.status == 0, info
    assert np.allclose(sg[:32], s[:32], rtol=1e-9)
    r = orc.svd_residual_norms(A, api.to_numpy(Ug)[:, :32], sg[:32], api.to_numpy(Vg)[:, :32])
    assert np.max(r) <= 1e-8
    assert np.all(r <= info.residuals[:32] * (1 + 1e-6) + 1e-15)


def test_si_svd_fp8_variant_certified(api, orc):
    """The FP8 variant of the mixed SVD (E4M3 products in the 16-bit power steps, then the FP64 phase):
    the same certified tolerance and singular values as the 16-bit path on a quarter of the benchmark."""
    A, U, s, V = orc.dense_svd_problem(4096, 1024, seed=7, smin=1e-6)
    Ug, sg, Vg, info = api.subspace_iter_svd(A, 4096, 1024, 64, "single", "half", maxiter=80, step_size=6,
                                             mode="mixed", tol=1e-8, nev=16, check_every=1, generalized_tol=0.0,
                                             power_fp8=True)
    assert info.status == 0, info
    assert np.allclose(sg[:16], s[:16], rtol=1e-9)
    r = orc.svd_residual_norms(A, api.to_numpy(Ug)[:, :16], sg[:16], api.to_numpy(Vg)[:, :16])
    assert np.max(r) <= 1e-8


@pytest.mark.parametrize("step64", [0, 9])
def test_si_eig_mixed_dense_certified(api, orc, step64):
    """Dense symmetric 2048 x 2048 (Haar Q, log-uniform spectrum), mixed mode, tol 1e-8: eigenvalues,
    true FP64 residuals and the certified residuals as an upper bound (FP64-phase power steps as the
    16-bit phase's, and 9)."""
    A, lam = orc.dense_sym_problem(2048, seed=11)
    Vg, d, info = api.subspace_iter_eig(A, 2048, 48, "single", "half", maxiter=200, step_size=6, mode="mixed",
                                       tol=1e-8, nev=8, check_every=1, symmetric=True, step_size_f64=step64)
    assert info.status == 0, info
    assert np.allclose(d[:8], lam[:8], rtol=1e-9)
    X = api.to_numpy(Vg)[:, :8]
    r = orc.residual_norms(A, X, d[:8], normA=float(np.max(np.abs(d[:8]))))
    assert np.max(r) <= 1e-8
    assert np.all(r <= info.residuals[:8] * (1 + 1e-6) + 1e-15)
