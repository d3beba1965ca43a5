"""CPU tests: the oracle against the reference's own known answers and analytic spectra."""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import ofrr_oracle as orc

GOLD = Path(__file__).resolve().parent / "golden"
KA = json.loads((GOLD / "known_answers.json").read_text())


def tridiag(n):
    return np.diag(2 * np.ones(n)) - np.diag(np.ones(n - 1), 1) - np.diag(np.ones(n - 1), -1)


def test_syev_known_answer():
    # CPP/tests/mvops_test.cpp:2292-2370 (tol 1e-10)
    w, V = orc.syev(tridiag(10))
    assert np.max(np.abs(w - KA["syev_true_eigenvalues"])) < KA["syev_tol"]
    assert np.max(np.abs(tridiag(10) @ V - V * w)) < 1e-10


def test_sygv_known_answer():
    # CPP/tests/mvops_test.cpp:2450-2530
    B = np.diag(np.arange(1, 11.0))
    w, V = orc.sygv(tridiag(10), B)
    assert np.max(np.abs(w - KA["sygv_true_eigenvalues"])) < 1e-10
    assert np.max(np.abs(tridiag(10) @ V - B @ V * w)) < 1e-10


def test_iamax_planted():
    # CPP/tests/mvops_test.cpp:774-796: 1-based index of the planted maximum
    n = KA["iamax_n"]
    x = (np.arange(n) - 65536) / 131072.0
    x[KA["iamax_planted_index0"]] = KA["iamax_planted_value"]
    idx, val = orc.iamax(x)
    assert idx == KA["iamax_planted_index0"] + 1 and val == KA["iamax_planted_value"]


def test_iamax_tie_lowest_index():
    x = np.array([0.5, -2.0, 1.0, 2.0, -2.0])
    assert orc.iamax(x) == (2, -2.0)


def test_dot_55():
    v = np.arange(1, 11.0)
    assert float(orc.dot(v, v)) == KA["dot_1_to_10"] + 330.0  # 1^2+..+10^2 = 385
    assert float(orc.dot(v, np.ones(10))) == KA["dot_1_to_10"]


@pytest.mark.parametrize("prec,pc", [("double", "double"), ("single", "single"), ("half", "single")])
def test_hessenberg_qr_and_skip(prec, pc):
    # CPP/tests/hessenberg_test.cpp:30-92 at 2000 x 200 (100 for half)
    rng = np.random.default_rng(11)
    n = 100 if prec == "half" else 200
    A = rng.uniform(-1, 1, (2000, n)).astype(orc._dt(prec))
    Q, R, sel, perm = orc.hessenberg(A, pc, prec)
    assert np.all(sel)
    err = np.max(np.abs(A.astype(np.float64) - Q.astype(np.float64) @ R.astype(np.float64)))
    assert err < KA["hessenberg_tols"][prec]
    assert np.max(np.abs(Q)) <= 1.0
    # unit entries at the pivot rows, zeros above in the pivot order
    for i in range(n):
        assert Q[perm[i], i] == 1.0
        assert np.all(Q[perm[:i], i] == 0.0)
    A[:, 3:6] = A[:, 0:3]
    _, _, sel, _ = orc.hessenberg(A, pc, prec, select_tol=KA["hessenberg_select_tols"][prec])
    assert list(np.where(~sel)[0]) == KA["hessenberg_skip_columns"]


def test_scalecols_semantics():
    U = np.array([[1.0, -4.0, 0.0], [-3.0, 2.0, 0.0], [3.0, 4.0, 0.0]])
    out, piv = orc.scalecols(U, "double", "double", return_pivots=True)
    assert list(piv) == [1, 0, 0]  # first occurrence of the max |.|
    assert np.allclose(out[:, 0], [-1 / 3, 1.0, -1.0]) and np.allclose(out[:, 1], [1.0, -0.5, -1.0])
    assert np.all(out[:, 2] == 0.0)  # zero column left untouched


def test_laplacian_analytic_spectrum():
    L = orc.laplacian_2d(64)
    assert L.shape == (4096, 4096) and L.nnz == 20224
    lam = orc.laplacian_2d_eigs(64)
    assert np.allclose(lam[:8], [7.99533, 7.98833, 7.98833, 7.98133, 7.97668, 7.97668, 7.96968, 7.96968], atol=1e-5)
    small = orc.laplacian_2d(7, 5)
    assert np.allclose(np.sort(np.linalg.eigvalsh(small.toarray()))[::-1], orc.laplacian_2d_eigs(7, 5))


def test_convdiff_analytic_spectrum():
    A = orc.convdiff_3d(6, Pe=10.0)
    ev = np.linalg.eigvals(A.toarray())
    assert np.max(np.abs(ev.imag)) < 1e-8
    assert np.allclose(np.sort(ev.real)[::-1], orc.convdiff_3d_eigs(6, Pe=10.0), rtol=1e-10)
    big = orc.convdiff_3d(128)
    assert big.shape[0] == 2097152 and big.nnz == 14581760


def test_subspace_iter_eig_converges_to_laplacian():
    L = orc.laplacian_2d(10)
    Ac = orc.sparse2csr(L)
    V, d = orc.subspace_iter_eig(Ac, 100, 16, "double", maxiter=60, step_size=3)
    assert np.allclose(d[:4], orc.laplacian_2d_eigs(10)[:4], rtol=1e-10)
    r = orc.residual_norms(Ac, V[:, :4], d[:4])
    assert np.max(r) < 1e-9


def test_subspace_iter_svd_dense():
    A, U, s, Vt = orc.dense_svd_problem(300, 60, seed=5, smin=1e-3)
    Uo, so, Vo = orc.subspace_iter_svd(A, 300, 60, 20, "double", maxiter=30, step_size=2)
    assert np.allclose(so[:6], s[:6], rtol=1e-9)
    assert np.max(orc.svd_residual_norms(A, Uo[:, :6], so[:6], Vo[:, :6])) < 1e-8


def test_arnoldi_hess_eig_symmetric():
    # 12 x 9 grid: simple eigenvalues (a one-vector restart cannot resolve multiplicities)
    L = orc.laplacian_2d(12, 9)
    Ac = orc.sparse2csr(L)
    V, d, info = orc.arnoldi_hess_eig(Ac, L.shape[0], 4, "double", maxiter=200, kdim=40, symmetric=True)
    assert np.allclose(d[:3], orc.laplacian_2d_eigs(12, 9)[:3], rtol=1e-9)
    assert orc.residual_norms(Ac, V[:, :1], d[:1])[0] < 1e-12


def test_arnoldi_mgs_eig_symmetric():
    L = orc.laplacian_2d(12, 9)
    Ac = orc.sparse2csr(L)
    V, d = orc.arnoldi_mgs_eig(Ac, L.shape[0], 4, "double", maxiter=200, kdim=40, symmetric=True)
    assert np.allclose(d[:3], orc.laplacian_2d_eigs(12, 9)[:3], rtol=1e-8)


def test_svd_rr_matches_svd_on_orthonormal_bases():
    A, U, s, V = orc.dense_svd_problem(200, 50, seed=9, smin=1e-2)
    Un, sn, Vn = orc.svd_rr(A, U[:, :10], V[:, :10], use_generalized=True, generalized_tol=0.0)
    assert np.allclose(sn, s[:10], rtol=1e-10)


def test_rng_block_deterministic_and_normal():
    a = orc.randn_block(42, 1000, 30)
    assert np.array_equal(a, orc.randn_block(42, 1000, 30))
    assert abs(a.mean()) < 0.02 and abs(a.std() - 1) < 0.02
    assert not np.array_equal(a, orc.randn_block(43, 1000, 30))


def test_golden_regression():
    """The oracle still reproduces the committed fixtures bit for bit."""
    g = np.load(GOLD / "golden.npz")
    for tag, pc, po in (("half", "single", "half"), ("single", "single", "single"), ("double", "double", "double")):
        Q, R, sel, perm = orc.hessenberg(g[f"hess_{tag}_A"], pc, po)
        assert np.array_equal(Q, g[f"hess_{tag}_Q"]) and np.array_equal(perm, g[f"hess_{tag}_perm"])
    _, _, sel, _ = orc.hessenberg(g["hess_dup_A"], "single", "half", select_tol=1e-2)
    assert np.array_equal(sel, g["hess_dup_sel"])
    assert np.array_equal(orc.scalecols(g["scal_U"], "single", "half"), g["scal_out"])


@pytest.mark.parametrize("classical", [False, True])
@pytest.mark.parametrize("p,tol,stol", [("double", 1e-10, 1e-12), ("single", 2e-6, 1e-6)])
def test_oracle_gram_schmidt_reference_contract(classical, p, tol, stol):
    """mgs.m / cgs.m restated: the checks of CPP/tests/qr_test.cpp:30-118 (uniform random 2000 x 200:
    Q'Q = I and A = QR within tol; columns 3..5 duplicating 0..2 are skipped, and the skipped
    columns' projections kept in R still give A = QR)."""
    from oracle import ofrr_oracle as o

    rng = np.random.default_rng(7)
    A = rng.uniform(0, 1, (2000, 200)).astype(o._dt(p))
    f = o.cgs if classical else o.mgs
    Q, R, sel = f(A, p, p, full=True)
    Qd, Rd = Q.astype(np.float64), R.astype(np.float64)
    assert sel.all()
    assert np.max(np.abs(Qd.T @ Qd - np.eye(200))) < tol
    assert np.max(np.abs(A - Qd @ Rd)) < tol
    A[:, 3:6] = A[:, 0:3]
    Q, R, sel = f(A, p, p, select_tol=stol, full=True)
    assert [i for i in range(200) if not sel[i]] == [3, 4, 5]
    assert np.max(np.abs(A - Q.astype(np.float64) @ R.astype(np.float64))) < tol


@pytest.mark.parametrize("p,stol", [("double", 1e-12), ("single", 1e-5)])
def test_oracle_lu_basis(p, stol):
    """lu.m restated: A_work = L U with rows permuted (A(perm, :) = L U up to rounding), |L| <= 1 with a
    unit diagonal, duplicated columns dropped with their rows consumed."""
    from oracle import ofrr_oracle as o

    rng = np.random.default_rng(3)
    A = rng.standard_normal((300, 40)).astype(o._dt(p))
    L, U, perm, sel = o.lu(A, p, p, full=True)
    assert sel.all()
    Ld, Ud = L.astype(np.float64), U.astype(np.float64)
    tol = 1e-12 if p == "double" else 1e-4
    assert np.max(np.abs(A.astype(np.float64)[perm] - Ld @ Ud)) < tol * np.max(np.abs(A))
    assert np.all(np.abs(Ld) <= 1.0) and np.all(np.diag(Ld[:40]) == 1.0)
    A[:, 7] = A[:, 2]
    A[:, 20] = A[:, 11]
    Q, R = o.lu(A, p, p, select_tol=stol)
    _, _, _, sel = o.lu(A, p, p, select_tol=stol, full=True)
    assert [i for i in range(40) if not sel[i]] == [7, 20] and Q.shape == (300, 38)


def test_oracle_hessenberg_keeps_all_nan_column():
    """hessenberg.m:62-70: max of an all-NaN column gives index 1 and abs(NaN) < select_tol is false,
    so the column stays selected with pivot row 0."""
    A = np.random.default_rng(0).uniform(-1, 1, (50, 4))
    A[:, 1] = np.nan
    Q, R, sel, perm = orc.hessenberg(A, "double")
    assert sel[1] and perm[1] == 0 and np.all(np.isnan(Q[:, 1]))


def test_oracle_thick_restart_convdiff_analytic():
    """The thick-restart restatement (the production Krylov path) converges to the analytic spectrum of the
    nonsymmetric 3D convection-diffusion operator."""
    A = orc.convdiff_3d(8)
    ex = orc.convdiff_3d_eigs(8)
    X, d, info = orc.arnoldi_thick_eig(orc.sparse2csr(A), A.shape[0], 12, 40, 1e-10)
    assert np.max(info["residuals"]) <= 1e-10
    assert np.max(np.abs(d - ex[:12])) <= 1e-9 * ex[0]
    R = A @ X - X * d[None, :]
    assert np.max(np.linalg.norm(R, axis=0)) <= 1e-10 * np.max(np.abs(d)) * 1.01


def test_oracle_thick_restart_symmetric():
    L = orc.laplacian_2d(16)
    ex = orc.laplacian_2d_eigs(16)
    X, d, info = orc.arnoldi_thick_eig(orc.sparse2csr(L), L.shape[0], 6, 30, 1e-11, symmetric=True)
    assert np.max(np.abs(d - ex[:6])) <= 1e-10 * ex[0]


def test_problem_generators_match_oracle():
    """The package's host-side generators (the bench inputs) equal the oracle's operators."""
    from mixedprecisionofrr_gb300 import problems

    A = problems.convdiff_3d(6)
    B = orc.convdiff_3d(6)
    assert abs(A - B).max() == 0
    assert np.allclose(problems.convdiff_3d_eigs(6), orc.convdiff_3d_eigs(6), rtol=0, atol=1e-9)
    assert abs(problems.laplacian(7, 2) - orc.laplacian_2d(7)).max() == 0
    assert np.allclose(problems.laplacian_eigs(7, 2), orc.laplacian_2d_eigs(7), rtol=0, atol=1e-9)
