"""Test-problem generators: point sets (MATLAB/+src/+kernel/generate_pts.m) and Gaussian kernel
matrices (CPP/testproblems/gaussian_kernel.hpp:14-77, MATLAB gaussian.m).  CPU: the oracle against the
reference's own test contract (CPP/tests/gaussian_kernel_test.cpp: symmetry, diagonal f^2 (1 + s^2)
exactly, off-diagonal formula within 1e-10, entries in [0, f^2], float 1e-5 / half 1e-2 of the FP64
kernel) and the argument checks of the C ABI.  GPU: points and kernels against the oracle."""
import numpy as np
import pytest


def test_oracle_gaussian_kernel_reference_contract():
    from oracle import ofrr_oracle as o

    f, l, s, n, d = 1.5, 2.0, 0.1, 10, 3
    X = o.rand_points(42, n, d, 0)
    K = o.generate_gaussian_kernel(f, l, s, X)
    assert np.array_equal(K, K.T)
    assert np.all(np.diag(K) == f * f * (1.0 + s * s))
    off = ~np.eye(n, dtype=bool)
    for i in range(n):
        for j in range(n):
            if i != j:
                dist = 0.0
                for k in range(d):
                    dist += (X[i, k] - X[j, k]) ** 2
                arg = -dist / (2 * l * l)
                assert abs(K[i, j] - (0.0 if arg < -700 else f * f * np.exp(arg))) < 1e-10
    assert np.all(K[off] >= 0) and np.all(K[off] <= f * f)
    assert np.all((X >= 0) & (X < n ** (1 / d)))
    with pytest.raises(ValueError):
        o.generate_gaussian_kernel(1.0, 0.0, 0.1, X)
    # gaussian.m on the same points equals the C++ form off the diagonal when f = 1 (up to rounding)
    G = o.gaussian(X, X, l, 1.0, s)
    K1 = o.generate_gaussian_kernel(1.0, l, s, X)
    assert np.allclose(G[off], K1[off], rtol=0, atol=1e-12)


def test_capi_argument_checks(built_lib):
    from mixedprecisionofrr_gb300 import _lib as L

    lib = L.load()
    for args in ((0.0, 1.0, 0.1, 10, 3), (-1.0, 1.0, 0.1, 10, 3), (1.0, 1.0, -0.1, 10, 3), (1.0, 1.0, 0.1, 0, 3),
                 (1.0, 1.0, 0.1, 10, 0), (1.0, 1.0, 0.1, -1, 3)):
        l, f, s, n, d = args
        assert lib.ofrr_gaussian_kernel(None, 0, n, n, d, None, 1, None, 1, l, f, s, L.F64, None, 1) == 1000
    assert lib.ofrr_rand_points(None, 1, 10, 3, 0, None, 10) == 1000      # no context
    assert lib.ofrr_rand_points(None, 1, 10, 3, 21, None, 10) == 1000     # disk needs d = 2
    assert lib.ofrr_rand_points(None, 1, 10, 2, 23, None, 10) == 1000     # grid needs a square n


@pytest.fixture(scope="module")
def api(built_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from mixedprecisionofrr_gb300 import api as a

    return a


@pytest.mark.gpu
@pytest.mark.parametrize("type,d", [(0, 1), (0, 3), (0, 5), (20, 2), (30, 3), (21, 2), (22, 2), (23, 2), (31, 3),
                                    (32, 3)])
def test_points_match_oracle(api, type, d):
    from oracle import ofrr_oracle as o

    n = 1024
    X = api.to_numpy(api.rand_points(9, n, d, type))
    Xo = o.rand_points(9, n, d, type)
    if type in (0, 20, 30, 23):
        assert np.array_equal(X, Xo)  # products of exact draws and one host-computed scale
    else:
        assert np.allclose(X, Xo, rtol=0, atol=1e-12 * n)  # sin / cos / asin / cbrt to an ulp or two


@pytest.mark.gpu
@pytest.mark.parametrize("n,d,f,l,s", [(10, 3, 1.5, 2.0, 0.1), (5, 2, 1.0, 1.0, 0.05), (700, 3, 2.0, 0.3, 0.0),
                                       (300, 2, 1.0, 0.05, 1.0)])
def test_gaussian_kernel_matches_oracle(api, n, d, f, l, s):
    """includes the exp(-700) cutoff (l = 0.05 on points ~17 apart)"""
    from oracle import ofrr_oracle as o

    K, X = api.generate_gaussian_kernel(f, l, s, 42, n, d)
    K = api.to_numpy(K)
    Ko = o.generate_gaussian_kernel(f, l, s, api.to_numpy(X))
    assert np.array_equal(K, K.T)
    assert np.all(np.diag(K) == f * f * (1.0 + s * s))
    assert np.array_equal(K == 0, Ko == 0)
    assert np.allclose(K, Ko, rtol=1e-15, atol=0)
    for prec, tol in (("single", 1e-5), ("half", 1e-2)):  # gaussian_kernel_test.cpp:181, :196
        Kp, _ = api.generate_gaussian_kernel(f, l, s, 42, n, d, precision=prec)
        assert np.max(np.abs(api.to_numpy(Kp).astype(np.float64) - Ko)) < tol * max(1.0, f * f)


@pytest.mark.gpu
def test_gaussian_matlab_form(api):
    from oracle import ofrr_oracle as o

    X = o.rand_points(3, 400, 2, 21)
    Y = o.rand_points(4, 250, 2, 21)
    K = api.to_numpy(api.gaussian(X, Y, 1.7, 1.3, 0.2))
    assert np.allclose(K, o.gaussian(X, Y, 1.7, 1.3, 0.2), rtol=0, atol=1e-12)
