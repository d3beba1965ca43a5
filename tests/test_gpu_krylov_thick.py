"""GPU parity tests of the thick-restart Hessenberg-process Krylov eigensolver (the production modes of
ofrr_arnoldi_eig with a CSR operator): FP64 mode against the FP64 oracle restatement on the same start
vector, mixed mode (16-bit phase, then FP64) against the analytic spectra and true FP64 residuals
recomputed here, the fused Krylov step's profiling entry, and the 128^3 convection-diffusion operator
at full size.

Tolerances: converged Ritz values agree with the analytic eigenvalues to 1e-9 relative to the largest
(residual tol 1e-10) or 1e-7 (tol 1e-8; the operator is non-normal, so eigenvalue errors can exceed
the residual); residuals are recomputed in FP64 with SciPy and must meet the tolerance."""
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


def _true_residuals(A, X, lam):
    X = np.asarray(X)
    R = A @ X - X * lam[None, :]
    return np.linalg.norm(R, axis=0) / (np.max(np.abs(lam)) * np.linalg.norm(X, axis=0))


@pytest.mark.parametrize("N", [8, 10])
def test_thick_fp64_matches_oracle(api, orc, N):
    A = orc.convdiff_3d(N)
    n = A.shape[0]
    ex = orc.convdiff_3d_eigs(N)
    v0 = orc.randn_block(5, n, 1)[:, 0]
    X, d, info = api.arnoldi_hess_eig(api.CsrMatrix(A), n, 6, "double", maxiter=3000, kdim=30, v0=v0, mode="fp64",
                                      tol=1e-10)
    assert info.status == 0, info
    Xo, do, io = orc.arnoldi_thick_eig(orc.sparse2csr(A), n, 6, 30, 1e-10, v0=v0)
    assert np.max(np.abs(d - ex[:6])) <= 1e-9 * ex[0]
    assert np.max(np.abs(d - do)) <= 1e-9 * ex[0]
    assert abs(info.iterations - io["cycles"]) <= 2
    assert np.max(_true_residuals(A, api.to_numpy(X), d)) <= 1e-10 * 1.01


@pytest.mark.parametrize("p16", ["half", "bfloat16"])
def test_thick_mixed_convdiff(api, orc, p16):
    N = 12
    A = orc.convdiff_3d(N)
    n = A.shape[0]
    ex = orc.convdiff_3d_eigs(N)
    X, d, info = api.arnoldi_hess_eig(api.CsrMatrix(A), n, 10, "single", p16, maxiter=6000, kdim=40, mode="mixed",
                                      tol=1e-8)
    assert info.status == 0, info
    assert info.escalations == 1  # the 16-bit phase cannot reach 1e-8 alone
    assert np.max(np.abs(d - ex[:10])) <= 1e-7 * ex[0]
    assert np.max(_true_residuals(A, api.to_numpy(X), d)) <= 1e-8 * 1.01


def test_thick_mixed_symmetric_laplacian(api, orc):
    # a 40 x 41 grid: a square grid has exactly repeated eigenvalues, and a Krylov space of one start
    # vector holds one vector of each eigenspace (in exact arithmetic, and FP64 is close to it)
    from mixedprecisionofrr_gb300 import serve_stream as ss

    L = ss.laplacian_grid((40, 41))
    n = L.shape[0]
    i = np.arange(1, 41)[:, None]
    j = np.arange(1, 42)[None, :]
    ex = np.sort((4.0 - 2.0 * np.cos(i * np.pi / 41) - 2.0 * np.cos(j * np.pi / 42)).ravel())[::-1]
    X, d, info = api.arnoldi_hess_eig(api.CsrMatrix(L), n, 8, "single", "half", maxiter=8000, kdim=40, mode="mixed",
                                      tol=1e-9)
    assert info.status == 0, info
    assert np.max(np.abs(d - ex[:8])) <= 1e-8 * ex[0]
    assert np.max(_true_residuals(L, api.to_numpy(X), d)) <= 1e-9 * 1.01


def test_thick_reference_restart_still_available(api, orc):
    """restart_keep = 1 keeps arnoldi_hess_eig.m's single-vector restart in the production modes."""
    L = orc.laplacian_2d(12)
    n = L.shape[0]
    X, d, info = api.arnoldi_hess_eig(api.CsrMatrix(L), n, 3, "double", maxiter=61, kdim=20, mode="fp64",
                                      restart_keep=1)
    assert info.status == 0
    assert np.all(np.isfinite(d))


def test_krylov_step_profile_entry(api, orc):
    A = orc.convdiff_3d(24)
    us, by = api.profile_krylov_step(api.CsrMatrix(A, symmetric=False), "half", 10, reps=3)
    n, nnz = A.shape[0], A.nnz
    assert us > 0
    assert by == nnz * 8 + 4 * (n + 1) + n * (8 + 2 * 10 + 1)


def test_c3_convdiff_128_full_size(api, orc):
    """The 3D convection-diffusion operator on the 128^3 grid (n = 2,097,152, 14.6 M nonzeros): 20
    eigenvalues of largest real part, Krylov dimension 64 with thick restarts, FP32 matvec and FP16
    basis in the first phase, FP64 after it.  Checked against the analytic spectrum and true FP64
    residuals."""
    N = 128
    A = orc.convdiff_3d(N)
    n = A.shape[0]
    ex = orc.convdiff_3d_eigs(N)
    X, d, info = api.arnoldi_hess_eig(api.CsrMatrix(A, symmetric=False), n, 20, "single", "half", maxiter=40000,
                                      kdim=64, mode="mixed", tol=1e-8)
    assert info.status == 0, info
    res = _true_residuals(A, api.to_numpy(X), d)
    assert np.max(res) <= 1e-8 * 1.01
    assert np.max(np.abs(d - ex[:20])) <= 1e-7 * ex[0]
