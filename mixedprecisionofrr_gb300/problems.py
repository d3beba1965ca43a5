"""Host-side synthetic operators with known spectra, the inputs of the benchmark and serving workloads.

* convdiff_3d: -Lap u + Pe w.grad u on the unit cube with Dirichlet boundaries, N^3 interior points,
  central differences (7-point stencil; h = 1/(N+1)), as CSR.  The operator is a Kronecker sum of three
  tridiagonal Toeplitz matrices T_d = tridiag(-1/h^2 - c_d, 2/h^2, -1/h^2 + c_d), c_d = Pe w_d / (2h), so
  its eigenvalues are the sums of 2/h^2 + 2 sqrt((1/h^2)^2 - c_d^2) cos(k pi / (N+1)) over the three
  dimensions (all real while Pe w_d h / 2 < 1).  "Largest real part" are the largest of these.
* laplacian: the Dirichlet Laplacian in 2 or 3 dimensions with the integer stencil (symmetric).
* dense_svd: A = U diag(s) V' with Haar U, V (QR of seeded Gaussians from the library's counter-based
  generator) and a geometric spectrum.
* dense_sym: Q diag(lambda) Q' with Haar Q and lambda log-uniform.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp


def _toeplitz_1d(N: int, c: float) -> sp.csr_matrix:
    h = 1.0 / (N + 1)
    lo = (-1.0 / h ** 2 - c) * np.ones(N - 1)
    up = (-1.0 / h ** 2 + c) * np.ones(N - 1)
    return sp.diags([lo, (2.0 / h ** 2) * np.ones(N), up], [-1, 0, 1], format="csr")


def convdiff_3d(N: int, Pe: float = 10.0, w=(1.0, 0.5, 0.25)) -> sp.csr_matrix:
    """7-point convection-diffusion operator on an N^3 grid (x fastest), CSR with sorted indices."""
    h = 1.0 / (N + 1)
    T = [_toeplitz_1d(N, Pe * wd / (2 * h)) for wd in w]
    I = sp.identity(N, format="csr")
    A = sp.kron(sp.kron(I, I), T[0]) + sp.kron(sp.kron(I, T[1]), I) + sp.kron(sp.kron(T[2], I), I)
    A = sp.csr_matrix(A)
    A.sort_indices()
    return A


def convdiff_3d_eigs(N: int, Pe: float = 10.0, w=(1.0, 0.5, 0.25), count: int | None = None) -> np.ndarray:
    """The eigenvalues of convdiff_3d, descending (the first `count`)."""
    h = 1.0 / (N + 1)
    k = np.arange(1, N + 1)
    parts = []
    for wd in w:
        c = Pe * wd / (2 * h)
        parts.append(2.0 / h ** 2 - 2.0 * np.sqrt((1.0 / h ** 2) ** 2 - c ** 2) * np.cos(k * np.pi / (N + 1)))
    lam = np.sort((parts[0][:, None, None] + parts[1][None, :, None] + parts[2][None, None, :]).ravel())[::-1]
    return lam if count is None else lam[:count]


def laplacian(N: int, dim: int = 2) -> sp.csr_matrix:
    """Dirichlet Laplacian on an N^dim grid with the integer stencil (2 dim, -1 per neighbour; the 2D
    form is the 5-point matrix with stencil 4, -1 x 4), symmetric positive definite."""
    T = sp.diags([-np.ones(N - 1), 2.0 * np.ones(N), -np.ones(N - 1)], [-1, 0, 1], format="csr")
    I = sp.identity(N, format="csr")
    if dim == 2:
        A = sp.kron(I, T) + sp.kron(T, I)
    else:
        A = sp.kron(sp.kron(I, I), T) + sp.kron(sp.kron(I, T), I) + sp.kron(sp.kron(T, I), I)
    A = sp.csr_matrix(A)
    A.sort_indices()
    return A


def laplacian_eigs(N: int, dim: int = 2, count: int | None = None) -> np.ndarray:
    """Eigenvalues of laplacian(N, dim), descending: sums of 2 - 2 cos(k pi / (N + 1))."""
    e = 2.0 - 2.0 * np.cos(np.arange(1, N + 1) * np.pi / (N + 1))
    if dim == 2:
        lam = (e[:, None] + e[None, :]).ravel()
    else:
        lam = (e[:, None, None] + e[None, :, None] + e[None, None, :]).ravel()
    lam = np.sort(lam)[::-1]
    return lam if count is None else lam[:count]


def _haar(n: int, k: int, seed: int) -> np.ndarray:
    from .api import randn_host

    Q, R = np.linalg.qr(randn_host(seed, n, k))
    return Q * np.sign(np.diag(R))[None, :]


def dense_svd(m: int, n: int, seed: int = 42, smin: float = 1e-6):
    """(A, s): A = U diag(s) V' (m x n, m >= n), s geometric from 1 to smin."""
    U = _haar(m, n, seed)
    V = _haar(n, n, seed + 1)
    s = smin ** (np.arange(n) / max(n - 1, 1))
    return (U * s[None, :]) @ V.T, s


def dense_sym(n: int, seed: int, lam_lo: float = 1e-4, lam_hi: float = 1.0):
    """(A, lambda descending): Q diag(lambda) Q' with lambda log-uniform in [lam_lo, lam_hi]."""
    Q = _haar(n, n, seed)
    u = np.random.default_rng(seed + 7).random(n)
    lam = np.exp(np.log(lam_lo) + (np.log(lam_hi) - np.log(lam_lo)) * u)
    A = (Q * lam[None, :]) @ Q.T
    return 0.5 * (A + A.T), np.sort(lam)[::-1]
