"""Fused scale-and-split kernels of the emulated FP64 power iteration (subspace_iter_svd.m:63-69: a
product, then scalecols.m).  In the refinement phase every scaled block is also split into BF16 digit
planes for the next exact-slice product, and inside the power loop the product's split-K partial sums
are combined by the scaling kernel itself.  Checked bit for bit:
  * the scaled columns against scalecols' FP64 rule with a reciprocal multiply (pivot row exactly 1),
    restated in numpy (IEEE round-to-nearest, as the kernel);
  * the fused product + scaling against the plain emulated product followed by that rule;
  * the digit planes against the stand-alone slicer on the same columns, and against the values
    (the digits are round(x 2^(35 - e)) in base 2^7, so they reconstruct x within 2^(e - 36)).
Columns over 2048 rows are split over a 2-CTA cluster: ties across the CTA boundary must pick the
lower row."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

S, BETA = 5, 7


@pytest.fixture(scope="module")
def api(built_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from mixedprecisionofrr_gb300 import api as a

    return a


def scale_fast(X):
    """scalecols (FP64) with y = 1/t rounded once and x y rounded once; the pivot row becomes 1."""
    X = X.copy()
    for j in range(X.shape[1]):
        a = np.abs(X[:, j])
        a = np.where(np.isnan(a), -1.0, a)
        k = int(np.argmax(a))  # first index of the maximum: lowest row on ties
        t = X[k, j]
        if t != 0.0:
            X[:, j] = X[:, j] * (1.0 / t)
            X[k, j] = 1.0
    return X


def run(api, mode, X, A=None, B=None):
    import torch
    from mixedprecisionofrr_gb300 import _lib as L

    ctx = api.context()
    M, N = X.shape
    Kp = (M + 63) // 64 * 64
    Xd = torch.as_tensor(np.asfortranarray(X).T.copy(), device="cuda")  # N x M rows = columns of X
    dig = torch.zeros(N * S * Kp, dtype=torch.int16, device="cuda")
    expo = torch.zeros(N, dtype=torch.int32, device="cuda")
    if mode == 1:
        K = A.shape[0]
        Ad = torch.as_tensor(np.ascontiguousarray(A.T), device="cuda")
        Bd = torch.as_tensor(np.ascontiguousarray(B.T), device="cuda")
        st = ctx.lib.ofrr_debug_scale_slice(ctx.h, 1, M, N, K, Ad.data_ptr(), K, Bd.data_ptr(), K, Xd.data_ptr(), M,
                                            dig.data_ptr(), expo.data_ptr())
    else:
        st = ctx.lib.ofrr_debug_scale_slice(ctx.h, mode, M, N, 0, None, 1, None, 1, Xd.data_ptr(), M,
                                            dig.data_ptr(), expo.data_ptr())
    assert st == L.SUCCESS
    assert ctx.lib.ofrr_ctx_synchronize(ctx.h) == L.SUCCESS
    d = dig.view(torch.bfloat16).float().cpu().numpy().reshape(N, S, Kp)
    return Xd.cpu().numpy().T.copy(), d, expo.cpu().numpy()


def check_digits(X, d, e):
    M = X.shape[0]
    assert np.all(np.abs(d[:, 0, :]) <= 2 ** BETA) and np.all(np.abs(d[:, 1:, :]) <= 2 ** (BETA - 1))
    assert np.all(d[:, :, M:] == 0)
    w = 2.0 ** (-BETA * np.arange(1, S + 1))
    rec = np.einsum("nsk,s->kn", d[:, :, :M].astype(np.float64), w) * 2.0 ** e[None, :].astype(np.float64)
    assert np.all(np.abs(rec - X) <= 2.0 ** (e[None, :].astype(np.float64) - BETA * S - 1))


def plant(X, M):
    """ties and maxima on both sides of the split rows of a clustered column"""
    h = 2048 if M <= 4096 else 4096
    if M > h and X.shape[1] >= 4:
        X[:, :3] = 0.9 * np.sin(np.arange(M))[:, None]  # |x| < 1 outside the planted rows
        X[[h - 1, h], 0] = [-3.0, 3.0]  # tie across the boundary: row h - 1 (first CTA) wins
        X[[h, M - 1], 1] = [-5.0, 5.0]  # maximum only in the second CTA, tie inside it
        X[[3, h + 1], 2] = [7.0, -7.0]  # tie, first CTA first
        X[:, 3] = 0.0  # zero column: left unscaled, digits zero
    return X


@pytest.mark.parametrize("M,N", [(700, 5), (1500, 6), (2048, 64), (3000, 7), (4096, 9), (6000, 4), (8192, 64)])
def test_scale_slice_matches_scalecols_and_slicer(api, M, N):
    rng = np.random.default_rng(M + N)
    X = plant(rng.standard_normal((M, N)) * np.exp(rng.uniform(-20, 20, N))[None, :], M)
    got, d, e = run(api, 0, X)
    assert np.array_equal(got.view(np.int64), scale_fast(X).view(np.int64))
    _, d2, e2 = run(api, 2, got)
    assert np.array_equal(e, e2) and np.array_equal(d, d2)
    check_digits(got, d, e)


@pytest.mark.parametrize("M,N,K", [(700, 5, 512), (2048, 64, 2048), (3000, 7, 300), (8192, 64, 2048),
                                   (8192, 3, 64), (4096, 33, 1000)])
def test_fused_product_scale_slice(api, M, N, K):
    rng = np.random.default_rng(K + M)
    A = rng.standard_normal((K, M))
    B = rng.standard_normal((K, N))
    got, d, e = run(api, 1, np.zeros((M, N)), A, B)
    C = api.gemm_f64_emulated(A, B).cpu().numpy()  # finished by the separate kernel
    assert np.array_equal(got.view(np.int64), scale_fast(C).view(np.int64))
    _, d2, e2 = run(api, 2, got)
    assert np.array_equal(e, e2) and np.array_equal(d, d2)
    check_digits(got, d, e)
