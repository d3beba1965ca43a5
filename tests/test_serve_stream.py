"""The serving stream's request generator and operators, on the CPU: the seeded stream is deterministic
and independent of its length, follows the workload's mix, ranges and arrival rate, and its Laplacians
are the Dirichlet stencils on rectangular grids whose spectra have no exactly repeated eigenvalue."""
import numpy as np
import pytest

ss = pytest.importorskip("mixedprecisionofrr_gb300.serve_stream")


def test_stream_deterministic_and_prefix_stable():
    a = ss.make_stream(seed=2024, count=300)
    b = ss.make_stream(seed=2024, count=300)
    assert a == b
    assert ss.make_stream(seed=2024, count=120) == a[:120]  # request i does not depend on count
    assert ss.make_stream(seed=2025, count=50) != a[:50]


def test_stream_mix_ranges_and_rate():
    reqs = ss.make_stream(seed=7, count=4000)
    svd = [r for r in reqs if r.kind == "svd"]
    lap = [r for r in reqs if r.kind == "lap"]
    assert len(svd) + len(lap) == len(reqs)
    assert abs(len(svd) / len(reqs) - 0.6) < 0.03  # 60 % dense SVD, 40 % Laplacian
    assert {r.tol for r in reqs} == {1e-6, 1e-8, 1e-10}
    for r in svd:
        assert 512 <= r.m <= 16384 and r.n <= r.m and r.n >= min(r.m // 8, r.m)
        assert 4 <= r.k <= 64 and r.k <= r.n // 2
    for r in lap:
        assert 4 <= r.k <= 64 and r.dim in (2, 3)
        N = r.grid[0]
        assert r.grid == tuple(N + d for d in range(r.dim))  # sides N, N+1 (, N+2)
        assert r.n == int(np.prod(r.grid)) and 5_000 <= r.n <= 1_100_000
    t = np.array([r.arrival for r in reqs])
    assert np.all(np.diff(t) > 0)
    gaps = np.diff(np.concatenate([[0.0], t]))
    assert abs(gaps.mean() * 2000.0 - 1.0) < 0.05  # Poisson at 2000 requests/s
    assert abs(gaps.std() / gaps.mean() - 1.0) < 0.1  # exponential gaps: coefficient of variation 1


@pytest.mark.parametrize("grid", [(6, 7), (4, 5, 6)])
def test_laplacian_grid_is_the_dirichlet_stencil(grid):
    A = ss.laplacian_grid(grid)
    n = int(np.prod(grid))
    assert A.shape == (n, n)
    assert (A != A.T).nnz == 0
    d = len(grid)
    assert np.all(A.diagonal() == 2.0 * d)
    # nonzeros: the diagonal plus two per interior edge of the grid
    edges = sum((grid[a] - 1) * int(np.prod(grid)) // grid[a] for a in range(d))
    assert A.nnz == n + 2 * edges
    lam = np.sort(np.linalg.eigvalsh(A.toarray()))[::-1]
    axes = [2.0 - 2.0 * np.cos(np.pi * np.arange(1, N + 1) / (N + 1)) for N in grid]
    ref = axes[0]
    for ax in axes[1:]:
        ref = np.add.outer(ref, ax).ravel()
    assert np.allclose(lam, np.sort(ref)[::-1], atol=1e-12)


@pytest.mark.parametrize("grid", [(39, 40, 41), (330, 331), (485, 486)])
def test_rectangular_grids_have_no_repeated_top_eigenvalue(grid):
    """Sides N, N+1 (, N+2): the largest eigenvalues (the ones the stream asks for) are all distinct, so a
    single-vector Krylov space can hold each eigenvector."""
    axes = [2.0 - 2.0 * np.cos(np.pi * np.arange(1, N + 1) / (N + 1)) for N in grid]
    lam = axes[0]
    for ax in axes[1:]:
        lam = np.add.outer(lam, ax).ravel()
    top = np.sort(lam)[::-1][:80]
    assert np.min(-np.diff(top)) > 1e-9
