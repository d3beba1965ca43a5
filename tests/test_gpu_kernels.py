"""GPU parity tests of the building-block kernels against the CPU oracle and the reference's
known answers.  Integer/index work and the element-wise Hessenberg arithmetic are bit-exact;
contractions are checked with the stated tolerances."""
import json
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden"
KA = json.loads((GOLD / "known_answers.json").read_text())


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


def test_device_rng_matches_oracle(api, orc):
    x = api.to_numpy(api.randn(42, 1000, 9))
    assert np.max(np.abs(x - orc.randn_block(42, 1000, 9))) < 1e-13
    assert np.array_equal(api.randn_host(5, 10, 3), api.randn_host(5, 10, 3))


def test_iamax_planted(api):
    n = KA["iamax_n"]
    x = (np.arange(n) - 65536) / 131072.0
    x[KA["iamax_planted_index0"]] = KA["iamax_planted_value"]
    for dt in (np.float64, np.float32, np.float16):
        idx, val = api.iamax(x.astype(dt))
        assert idx == KA["iamax_planted_index0"] + 1 and val == KA["iamax_planted_value"]


def test_iamax_ties_empty_and_nan(api):
    assert api.iamax(np.array([0.5, -2.0, 1.0, 2.0, -2.0])) == (2, -2.0)
    big = np.zeros(300001)
    big[[7, 250000, 299999]] = 3.0
    assert api.iamax(big)[0] == 8
    assert api.iamax(np.array([np.nan, 1.0, -4.0, np.nan]))[0] == 3


@pytest.mark.parametrize("pc,po", [("single", "half"), ("single", "single"), ("double", "double"),
                                   ("double", "half")])
def test_scalecols_bit_exact(api, orc, pc, po):
    rng = np.random.default_rng(1)
    U = (rng.standard_normal((3001, 17)) * 5).astype(orc._dt(po))
    U[:, 4] = 0
    U[10, 5] = -U[:, 5].max() * 2  # planted negative max
    out, piv = api.scalecols(U, pc, po, return_pivots=True)
    ref, rpiv = orc.scalecols(U, pc, po, return_pivots=True)
    assert np.array_equal(api.to_numpy(piv), rpiv)
    assert np.array_equal(api.to_numpy(out), ref)


@pytest.mark.parametrize("m", [2048, 2049, 6000, 8192, 9000])
def test_scalecols_chunked_ties(api, orc, m):
    """Columns over 2048 rows (one 1024-thread CTA up to 8192 rows, chunked beyond): equal maxima in
    different chunks pick the lowest row."""
    rng = np.random.default_rng(m)
    U = rng.uniform(-1, 1, (m, 5))
    U[[2047, m - 1], 0] = [-3.0, 3.0]   # tie across the chunk boundary: row 2047 wins
    U[[m - 1, 5], 1] = [4.0, -4.0]      # tie, lower row first in the column
    U[:, 2] = 0.0
    U[m // 2, 3] = np.nan               # NaN is never the pivot
    for pc, po in (("double", "double"), ("single", "half")):
        Ui = U.astype(orc._dt(po))
        out, piv = api.scalecols(Ui, pc, po, return_pivots=True)
        ref, rpiv = orc.scalecols(Ui, pc, po, return_pivots=True)
        piv = api.to_numpy(piv)
        assert piv[0] == 2047 and piv[1] == 5 and piv[2] == 0
        assert np.array_equal(piv[[0, 1, 2, 4]], rpiv[[0, 1, 2, 4]])
        got = api.to_numpy(out)
        assert np.array_equal(got[:, [0, 1, 2, 4]], ref[:, [0, 1, 2, 4]])


def test_scalecols_golden(api, gold):
    out = api.scalecols(gold["scal_U"], "single", "half")
    assert np.array_equal(api.to_numpy(out), gold["scal_out"])


@pytest.mark.parametrize("tag,pc,po", [("half", "single", "half"), ("single", "single", "single"),
                                       ("double", "double", "double")])
def test_hessenberg_golden_bit_exact(api, gold, tag, pc, po):
    Q, R, sel, perm = api.hessenberg(gold[f"hess_{tag}_A"], pc, po)
    assert np.array_equal(perm, gold[f"hess_{tag}_perm"])
    assert np.array_equal(api.to_numpy(Q), gold[f"hess_{tag}_Q"])
    assert np.array_equal(R, gold[f"hess_{tag}_R"].astype(np.float64))


@pytest.mark.parametrize("prec,pc", [("double", "double"), ("single", "single"), ("half", "single")])
def test_hessenberg_reference_contract(api, prec, pc):
    """hessenberg_test.cpp:30-92: no NaN/Inf, max|A - QR| bounds, skip pattern {3,4,5}."""
    rng = np.random.default_rng(12)
    n = 100 if prec == "half" else 200
    dt = {"double": np.float64, "single": np.float32, "half": np.float16}[prec]
    A = rng.uniform(-1, 1, (2000, n)).astype(dt)
    Q, R, sel, perm = api.hessenberg(A, pc, prec)
    assert api.check_special_values(Q) == 0
    Qn = api.to_numpy(Q).astype(np.float64)
    assert np.max(np.abs(A.astype(np.float64) - Qn @ R)) < KA["hessenberg_tols"][prec]
    A[:, 3:6] = A[:, 0:3]
    Q, R, sel, perm = api.hessenberg(A, pc, prec, select_tol=KA["hessenberg_select_tols"][prec])
    assert list(np.where(~sel)[0]) == KA["hessenberg_skip_columns"]
    assert np.all(api.to_numpy(Q)[:, 3:6] == 0)  # deselected columns are zero (hessenberg.m:262-268)


def test_hessenberg_live_oracle_large(api, orc):
    rng = np.random.default_rng(99)
    A = rng.standard_normal((20000, 40)).astype(np.float16)
    Q, R, sel, perm = api.hessenberg(A, "single", "half")
    Qo, Ro, selo, permo = orc.hessenberg(A, "single", "half")
    assert np.array_equal(perm, permo)
    assert np.array_equal(api.to_numpy(Q), Qo)


def test_hessenberg_edge_shapes(api, orc):
    for shape in ((1, 1), (5, 1), (7, 7), (33, 32)):
        A = np.random.default_rng(sum(shape)).uniform(-1, 1, shape)
        Q, R, sel, perm = api.hessenberg(A, "double")
        Qo, Ro, selo, permo = orc.hessenberg(A, "double")
        assert np.array_equal(api.to_numpy(Q), Qo) and np.array_equal(perm, permo)
    with pytest.raises(Exception):
        api.hessenberg(np.ones((3, 5)), "double")  # hessenberg.m:52 tall-thin assertion


@pytest.mark.parametrize("m", [300, 20000])  # the clustered block kernel and the per-column kernel
def test_hessenberg_all_nan_column_kept(api, orc, m):
    """hessenberg.m keeps a column whose values are all NaN (abs(NaN) < select_tol is false): pivot row
    0, the column scaled by NaN.  Later columns eliminate against it, so they turn NaN too."""
    rng = np.random.default_rng(m)
    A = rng.uniform(-1, 1, (m, 6))
    A[:, 2] = np.nan
    Q, R, sel, perm = api.hessenberg(A, "double")
    Qo, Ro, selo, permo = orc.hessenberg(A, "double")
    assert list(sel) == list(selo) and sel[2]
    assert list(perm) == list(permo) and perm[2] == 0
    Qn = api.to_numpy(Q)
    assert np.array_equal(np.isnan(Qn), np.isnan(Qo))
    assert np.array_equal(Qn[:, :2], Qo[:, :2])


@pytest.mark.parametrize("pc,pin,po,tol", [("double", "double", "double", 1e-13), ("single", "single", "single", 1e-5),
                                           ("single", "half", "half", 2e-3), ("single", "half", "single", 1e-5),
                                           ("single", "bfloat16", "single", 1e-5)])
@pytest.mark.parametrize("trans", ["N", "T"])
def test_gemm_semantics(api, pc, pin, po, tol, trans):
    import torch

    rng = np.random.default_rng(4)
    for (M, N, K) in ((300, 24, 500), (256, 64, 1024), (1000, 16, 37)):
        A = rng.standard_normal((K, M) if trans == "T" else (M, K))
        B = rng.standard_normal((K, N))
        pid = api.PREC[pin]
        Ad = api.to_device_cm(A, pid)
        Bd = api.to_device_cm(B, pid)
        Cd = api.gemm(Ad, trans, Bd, pc, po)
        # exact products of the rounded inputs, FP64 reference
        Ar = Ad.double().cpu().numpy()
        Br = Bd.double().cpu().numpy()
        ref = (Ar.T if trans == "T" else Ar) @ Br
        got = Cd.double().cpu().numpy()
        err = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
        assert err < tol, (M, N, K, err)
        assert Cd.dtype == api.TORCH_DT[api.PREC[po]]


@pytest.mark.parametrize("pc,tol", [("double", 1e-14), ("single", 1e-6)])
def test_csrmm_vs_scipy(api, orc, pc, tol):
    L = orc.laplacian_2d(30, 17)
    Ac = api.CsrMatrix(L)
    X = np.random.default_rng(2).standard_normal((L.shape[0], 11))
    for nr in (1, 3, 11):
        Y = api.to_numpy(api.csrmv(Ac, "N", X[:, :nr], pc, "double")).astype(np.float64)
        ref = L @ X[:, :nr].astype(orc._dt(pc)).astype(np.float64)
        assert np.max(np.abs(Y - ref)) < tol * np.max(np.abs(ref))
    C = orc.convdiff_3d(5)
    Cc = api.CsrMatrix(C)
    Y = api.to_numpy(api.csrmv(Cc, "T", X[:125, :3], pc, "double"))
    assert np.allclose(Y, C.T @ X[:125, :3], rtol=tol * 10, atol=tol * 1e3)


def test_csrmm_transposed_deterministic_and_wide(api, orc):
    """The transposed product runs on a transpose built by a deterministic counting sort (no floating-point
    atomics): two calls give bit-identical results, equal to the 'N' product of the explicit transpose.
    Rectangular operator with rows of 0 .. 40 nonzeros (some CTAs exceed the staging capacity), 65
    right-hand sides (several column chunks over one staging of the nonzeros)."""
    import scipy.sparse as sp

    rng = np.random.default_rng(4)
    m, n = 3000, 1700
    lens = rng.integers(0, 41, m)
    lens[:300] = 40  # the first CTAs hold more nonzeros than the shared-memory staging holds
    rows = np.repeat(np.arange(m), lens)
    cols = rng.integers(0, n, rows.size)
    A = sp.csr_matrix((rng.standard_normal(rows.size), (rows, cols)), shape=(m, n))
    A.sum_duplicates()
    A.sort_indices()
    Ac = api.CsrMatrix(A)
    X = rng.standard_normal((m, 65))
    Y1 = api.to_numpy(api.csrmv(Ac, "T", X, "double", "double"))
    Y2 = api.to_numpy(api.csrmv(Ac, "T", X, "double", "double"))
    assert np.array_equal(Y1, Y2)
    At = sp.csr_matrix(A.T)
    At.sort_indices()
    Y3 = api.to_numpy(api.csrmv(api.CsrMatrix(At), "N", X, "double", "double"))
    assert np.array_equal(Y1, Y3)
    assert np.allclose(Y1, A.T @ X, rtol=1e-13, atol=1e-12)
    Z = rng.standard_normal((n, 65))
    YN = api.to_numpy(api.csrmv(Ac, "N", Z, "double", "double"))
    assert np.allclose(YN, A @ Z, rtol=1e-13, atol=1e-12)


def test_syev_sygv_known_answers(api):
    n = 10
    A = np.diag(2 * np.ones(n)) - np.diag(np.ones(n - 1), 1) - np.diag(np.ones(n - 1), -1)
    w, V = api.syev(A)
    assert np.max(np.abs(w - KA["syev_true_eigenvalues"])) < 1e-10
    assert np.max(np.abs(A @ V - V * w)) < 1e-10
    B = np.diag(np.arange(1, 11.0))
    w, V = api.sygv(A, B)
    assert np.max(np.abs(w - KA["sygv_true_eigenvalues"])) < 1e-10
    assert np.max(np.abs(A @ V - B @ V * w)) < 1e-10
    assert np.max(np.abs(V.T @ B @ V - np.eye(n))) < 1e-12


@pytest.mark.parametrize("n", [1, 2, 7, 64, 97, 130])
def test_syev_random(api, n):
    rng = np.random.default_rng(n)
    A = rng.standard_normal((n, n))
    A = A + A.T
    w, V = api.syev(A)
    assert np.allclose(w, np.linalg.eigvalsh(A), atol=1e-11 * max(1, np.abs(w).max()))
    assert np.max(np.abs(A @ V - V * w)) < 1e-10 * max(1, np.abs(w).max())


def test_check_special_values(api):
    X = np.ones((100, 3))
    assert api.check_special_values(X) == 0
    X[5, 1] = np.nan
    assert api.check_special_values(X) == 1005
    X[5, 1] = np.inf
    assert api.check_special_values(X) == 1006


@pytest.mark.parametrize("pc,po,shape", [("single", "half", (3000, 64)), ("double", "double", (8192, 64)),
                                         ("single", "single", (1500, 37)), ("single", "half", (20000, 96)),
                                         ("double", "double", (2047, 80)), ("single", "half", (8192, 64))])
def test_hessenberg_blocked_equals_per_column(api, orc, pc, po, shape):
    """The cluster-blocked schedule and the per-column schedule give bit-identical bases."""
    import os

    rng = np.random.default_rng(shape[0] + shape[1])
    A = rng.uniform(-1, 1, shape).astype(orc._dt(po))
    A[:, 20] = A[:, 3]  # a dependent column inside the second block
    Qb, Rb, selb, permb = api.hessenberg(A, pc, po)
    os.environ["OFRR_HESS_PER_COLUMN"] = "1"
    try:
        Qc, Rc, selc, permc = api.hessenberg(A, pc, po)
    finally:
        del os.environ["OFRR_HESS_PER_COLUMN"]
    os.environ["OFRR_HESS_CLUSTER"] = "8"  # portable cluster size (the default may be 16 CTAs)
    try:
        Q8, R8, sel8, perm8 = api.hessenberg(A, pc, po)
    finally:
        del os.environ["OFRR_HESS_CLUSTER"]
    assert np.array_equal(permb, permc) and np.array_equal(selb, selc)
    assert np.array_equal(api.to_numpy(Qb), api.to_numpy(Qc))
    assert np.array_equal(Rb, Rc)
    assert np.array_equal(perm8, permc) and np.array_equal(api.to_numpy(Q8), api.to_numpy(Qc))
    assert np.array_equal(R8, Rc)
    if po != "double":  # in FP64 the duplicate's rounding residual can exceed the default eps threshold
        assert not selb[20]
    if shape[0] <= 3000:
        Qo, Ro, selo, permo = orc.hessenberg(A, pc, po)
        assert np.array_equal(api.to_numpy(Qb), Qo) and np.array_equal(permb, permo)
