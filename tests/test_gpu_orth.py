"""Orthogonal comparison bases on the GPU (MATLAB/+src/+qr/mgs.m, cgs.m; C++ msvd::mgs / cgs2 of
CPP/linalg/factorization/qr.hpp): the reference's own QR test contract (CPP/tests/qr_test.cpp:
Q'Q = I and A = QR within 1e-10 / 2e-6 / 2e-2 in double / single / half, duplicated columns skipped),
parity with the oracle's restatement (same skip flags; Q and R to rounding, since only the dots'
summation order differs), and subspace iteration with these bases against the oracle's."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# (Q'Q / A = QR tolerance, select_tol of the dependent-column case); in half precision the residual
# of a duplicated 2000-row column is ~2e-2 of rounding noise, so the skip test uses 5e-2 (cgs2's
# value in qr_test.cpp:539)
TOL = {"double": (1e-10, 1e-12), "single": (2e-6, 1e-6), "half": (2e-2, 5e-2)}


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


@pytest.mark.parametrize("classical", [False, True])
@pytest.mark.parametrize("p,pc", [("double", "double"), ("single", "single"), ("half", "single")])
def test_gs_reference_contract(api, orc, classical, p, pc):
    tol, stol = TOL[p]
    m, n = (2000, 200) if p != "half" else (2000, 40)
    rng = np.random.default_rng(11)
    A = rng.uniform(0, 1, (m, n)).astype(orc._dt(p))
    Q, R, skip = api.gs_basis(A, classical, pc, p)
    Qd = api.to_numpy(Q).astype(np.float64)
    assert not skip.any()
    assert np.max(np.abs(Qd.T @ Qd - np.eye(n))) < tol
    assert np.max(np.abs(A.astype(np.float64) - Qd @ R)) < tol
    A[:, 3:6] = A[:, 0:3]
    Q, R, skip = api.gs_basis(A, classical, pc, p, select_tol=stol)
    assert list(np.flatnonzero(skip)) == [3, 4, 5]
    Qd = api.to_numpy(Q).astype(np.float64)
    assert np.all(Qd[:, 3:6] == 0)
    assert np.max(np.abs(A.astype(np.float64) - Qd @ R)) < tol


@pytest.mark.parametrize("classical", [False, True])
@pytest.mark.parametrize("p,pc,tol,stol", [("double", "double", 1e-12, 1e-10), ("single", "double", 2e-6, 1e-3),
                                           ("single", "single", 2e-5, 1e-3)])
def test_gs_matches_oracle(api, orc, classical, p, pc, tol, stol):
    """a dependent column leaves rounding noise after its projections; select_tol above that noise
    drops it in both (below it, both would keep normalised noise, which no two summation orders share)"""
    rng = np.random.default_rng(5)
    A = rng.standard_normal((700, 24))
    A[:, 10] = A[:, 2] * 3.0  # dependent: dropped after the projections
    A[:, 17] = 0.0            # zero: dropped before any projection
    A = A.astype(orc._dt(p))
    f = orc.cgs if classical else orc.mgs
    Qo, Ro, selo = f(A, pc, p, select_tol=stol, full=True)
    Q, R, skip = api.gs_basis(A, classical, pc, p, select_tol=stol)
    assert np.array_equal(skip == 0, selo)
    assert np.max(np.abs(api.to_numpy(Q).astype(np.float64) - Qo.astype(np.float64))) < tol
    assert np.max(np.abs(R - Ro.astype(np.float64))) < tol * np.max(np.abs(Ro.astype(np.float64)))


def test_gs_no_reorth_and_aliasing(api, orc):
    """reorth_tol < 0 (mgs_v2's single pass) follows the oracle with the loop off; an input that is
    also the output is read before it is overwritten."""
    import torch

    rng = np.random.default_rng(2)
    A = rng.uniform(0, 1, (500, 30))
    Qo, Ro, _ = orc.mgs(A, "double", "double", reorth_tol=-1.0, full=True)
    Q, R, skip = api.gs_basis(A, False, "double", "double", reorth_tol=-1.0)
    assert not skip.any()
    assert np.max(np.abs(api.to_numpy(Q) - Qo)) < 1e-12
    from mixedprecisionofrr_gb300 import _lib as L

    ctx = api.context()
    X = api.to_device_cm(A, L.F64)
    Rh = np.zeros(30 * 30)
    sk = np.zeros(30, np.int32)
    assert ctx.lib.ofrr_gs_basis(ctx.h, 0, L.F64, L.F64, L.F64, 500, 30, X.data_ptr(), 500, X.data_ptr(), 500, -1.0,
                                 float("nan"), float("nan"), Rh.ctypes.data_as(L.C.POINTER(L.C.c_double)),
                                 sk.ctypes.data_as(L.C.POINTER(L.C.c_int))) == L.SUCCESS
    Qf, _, _ = orc.mgs(A, "double", "double", full=True)
    assert np.max(np.abs(api.to_numpy(X) - Qf)) < 1e-12
    torch.cuda.synchronize()


@pytest.mark.parametrize("orth", ["mgs", "cgs"])
def test_si_eig_with_orthogonal_basis_matches_oracle(api, orc, orth):
    """subspace_iter_eig.m with function_orth = mgs (its default) or cgs, reference mode, FP64"""
    A = orc.laplacian_2d(20).toarray()
    n = A.shape[0]
    V0 = orc.randn_block(42, n, 12)
    Vo, do = orc.subspace_iter_eig(A, n, 12, "double", "double", maxiter=30, step_size=2, orth=orth, V0=V0)
    V, d, info = api.subspace_iter_eig(A, n, 12, "double", "double", maxiter=30, step_size=2, V0=V0, orth=orth)
    assert np.max(np.abs(np.asarray(d)[:8] - np.asarray(do)[:8])) < 1e-10 * np.max(np.abs(do))


@pytest.mark.parametrize("orth", ["mgs", "cgs"])
def test_si_svd_with_orthogonal_basis_matches_oracle(api, orc, orth):
    rng = np.random.default_rng(3)
    U0, _ = np.linalg.qr(rng.standard_normal((600, 150)))
    W0, _ = np.linalg.qr(rng.standard_normal((150, 150)))
    s_true = 0.8 ** np.arange(150)
    A = (U0 * s_true) @ W0.T
    V0 = orc.randn_block(7, 150, 16)
    _, so, _ = orc.subspace_iter_svd(A, 600, 150, 16, "double", "double", maxiter=12, orth=orth, V0=V0)
    U, s, V, info = api.subspace_iter_svd(A, 600, 150, 16, "double", "double", maxiter=12, V0=V0, orth=orth)
    assert np.max(np.abs(np.asarray(s)[:8] - np.asarray(so)[:8])) < 1e-10
    assert np.max(np.abs(np.asarray(s)[:6] - s_true[:6])) < 1e-9


def test_fp64_mode_orthogonal_vs_hessenberg(api, orc):
    """the paper's comparison at small scale: the FP64 solver with an MGS basis and with the
    Hessenberg basis reach the same eigenvalues to the tolerance"""
    A = api.CsrMatrix(orc.laplacian_2d(16), symmetric=True)
    n = A.shape[0]
    lam = orc.laplacian_2d_eigs(16)
    V0 = orc.randn_block(42, n, 16)
    out = {}
    for orth in ("hessenberg", "mgs"):
        V, d, info = api.subspace_iter_eig(A, n, 16, V0=V0, nev=4, tol=1e-10, maxiter=3000, mode="fp64", orth=orth)
        assert info.status == 0
        out[orth] = np.asarray(d)[:4]
    assert np.allclose(out["mgs"], lam[:4], rtol=1e-9)
    assert np.allclose(out["hessenberg"], lam[:4], rtol=1e-9)


@pytest.mark.parametrize("p,pc,stol", [("double", "double", 1e-12), ("single", "single", 1e-5),
                                       ("half", "single", 1e-2), ("single", "double", 1e-5)])
def test_lu_basis_bit_exact_vs_oracle(api, orc, p, pc, stol):
    """lu.m on the GPU: element-wise arithmetic and an exact argmax with MATLAB's tie rule, so Q (the
    un-permuted L), U and the skip flags equal the oracle's bit for bit"""
    rng = np.random.default_rng(4)
    A = rng.standard_normal((1500, 48))
    A[:, 9] = A[:, 3]    # duplicated: dropped, its row consumed
    A[:, 30] = 0.0       # zero: dropped at once
    A[[5, 6], 12] = [4.0, -4.0]  # a tie in |value|: the first row in the current order wins
    A = A.astype(orc._dt(p))
    L, U, perm, sel = orc.lu(A, pc, p, select_tol=stol, full=True)
    rperm = np.empty_like(perm)
    rperm[perm] = np.arange(len(perm))
    Lu = L[rperm]
    Lu[:, ~sel] = 0
    Q, R, skip = api.lu_basis(A, pc, p, select_tol=stol)
    assert np.array_equal(skip == 0, sel)
    Qh = api.to_numpy(Q)
    assert np.array_equal(Qh.astype(np.float64), Lu.astype(np.float64))
    assert np.array_equal(R, U.astype(np.float64))


def test_si_eig_with_lu_basis_matches_oracle(api, orc):
    A = orc.laplacian_2d(20).toarray()
    n = A.shape[0]
    V0 = orc.randn_block(42, n, 12)
    _, do = orc.subspace_iter_eig(A, n, 12, "double", "double", maxiter=30, step_size=2, orth="lu", V0=V0)
    V, d, info = api.subspace_iter_eig(A, n, 12, "double", "double", maxiter=30, step_size=2, V0=V0, orth="lu")
    assert np.max(np.abs(np.asarray(d)[:8] - np.asarray(do)[:8])) < 1e-10 * np.max(np.abs(do))
