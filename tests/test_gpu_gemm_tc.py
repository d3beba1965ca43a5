"""tcgen05 TN GEMM (16-bit operands, FP32 accumulation): shapes with tails in M, N and K, split-K,
every output type, against an FP64 product of the same rounded inputs and against cuBLAS."""
import os

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


SHAPES = [(128, 64, 64), (8192, 64, 2048), (2048, 64, 8192), (64, 64, 8192), (300, 40, 1000), (129, 33, 77),
          (1000, 128, 256), (4096, 96, 640), (50, 16, 16)]


@pytest.mark.parametrize("M,N,K", SHAPES)
@pytest.mark.parametrize("pin", ["half", "bfloat16"])
def test_tc_gemm_vs_fp64(api, M, N, K, pin):
    from mixedprecisionofrr_gb300 import _lib as L

    rng = np.random.default_rng(M * 7 + N * 3 + K)
    A = rng.standard_normal((K, M))  # stored K x M: the TN operand layout
    B = rng.standard_normal((K, N))
    p = api.PREC[pin]
    Ad = api.to_device_cm(A, p)
    Bd = api.to_device_cm(B, p)
    ref = Ad.double().cpu().numpy().T @ Bd.double().cpu().numpy()
    scale = np.max(np.abs(ref))
    for po, tol in (("single", 2e-6 * np.sqrt(K)), ("half", 1e-3), (pin, 1e-2)):
        Cd = api.gemm(Ad, "T", Bd, "single", po)
        got = Cd.double().cpu().numpy()
        assert np.max(np.abs(got - ref)) / scale < tol, (po, np.max(np.abs(got - ref)) / scale)
    launches = api.context().launch_count
    assert launches > 0


def test_tc_matches_cublas(api):
    """The same product through cuBLAS GemmEx (tensor path disabled) agrees to FP32 rounding."""
    rng = np.random.default_rng(5)
    A = rng.standard_normal((2048, 512))
    B = rng.standard_normal((2048, 64))
    Ad = api.to_device_cm(A, api.PREC["half"])
    Bd = api.to_device_cm(B, api.PREC["half"])
    c_tc = api.gemm(Ad, "T", Bd, "single", "single").double().cpu().numpy()
    os.environ["OFRR_DISABLE_TC"] = "1"
    try:
        c_lib = api.gemm(Ad, "T", Bd, "single", "single").double().cpu().numpy()
    finally:
        del os.environ["OFRR_DISABLE_TC"]
    assert np.max(np.abs(c_tc - c_lib)) / np.max(np.abs(c_lib)) < 1e-5


def test_tc_exact_small_integers(api):
    """Integer-valued operands with |a|,|b| <= 63 and K = 2048: every partial sum is exact in FP32,
    so the tensor-core result must equal the exact integer product bit for bit."""
    rng = np.random.default_rng(9)
    A = rng.integers(-63, 64, (2048, 256)).astype(np.float64)
    B = rng.integers(-63, 64, (2048, 64)).astype(np.float64)
    Ad = api.to_device_cm(A, api.PREC["bfloat16"])
    Bd = api.to_device_cm(B, api.PREC["bfloat16"])
    got = api.gemm(Ad, "T", Bd, "single", "single").double().cpu().numpy()
    assert np.array_equal(got, A.T @ B)


@pytest.mark.parametrize("M,N,K", [(2048, 64, 8192), (8192, 64, 2048), (64, 64, 8192), (300, 17, 1000), (77, 5, 64),
                                   (20000, 64, 512), (1000, 130, 3000), (128, 64, 1), (96, 16, 9000)])
def test_f64_emulated_gemm(api, M, N, K):
    """Exact-slice FP64 emulation: element error within 2^-33 |A'| |B| (two bits of margin over the
    2^-35 design bound), on operands with widely varying column scales."""
    rng = np.random.default_rng(M + N + K)
    A = rng.standard_normal((K, M)) * np.exp(rng.uniform(-20, 20, M))[None, :]
    B = rng.standard_normal((K, N)) * np.exp(rng.uniform(-20, 20, N))[None, :]
    C = api.gemm_f64_emulated(A, B).cpu().numpy()
    ref = A.T @ B
    bound = np.abs(A).T @ np.abs(B)
    assert np.all(np.abs(C - ref) <= 2.0 ** -33 * bound + 1e-300)
    # integer accumulation: the result does not depend on the schedule (bit-identical on repeat)
    assert np.array_equal(api.gemm_f64_emulated(A, B).cpu().numpy(), C)


def test_f64_emulated_gemm_extreme_scales(api):
    """Columns with subnormal, huge, unit and zero scales (the digit split works on the bit patterns)."""
    rng = np.random.default_rng(7)
    K = 700
    A = rng.standard_normal((K, 6))
    A[:, 0] *= 1e-310
    A[:, 1] *= 1e300
    A[:, 3] = 0.0
    A[5, 4] = 5e-324  # one denormal entry in an otherwise normal column
    B = rng.standard_normal((K, 3))
    C = api.gemm_f64_emulated(A, B).cpu().numpy()
    ref = A.T @ B
    bound = np.abs(A).T @ np.abs(B)
    assert np.all(np.abs(C - ref) <= 2.0 ** -33 * bound + 1e-320)
    assert np.array_equal(C[3], np.zeros(3))


def test_f64_emulated_gemm_zero_columns(api):
    A = np.zeros((256, 40))
    B = np.random.default_rng(1).standard_normal((256, 8))
    A[:, 3] = 1.0
    C = api.gemm_f64_emulated(A, B).cpu().numpy()
    assert np.array_equal(C[[0, 1, 2, 4]], np.zeros((4, 8)))
    assert np.allclose(C[3], B.sum(0), rtol=1e-12)


@pytest.mark.parametrize("M,N,K", [(8192, 64, 2048), (2048, 64, 8192), (1500, 9, 3000), (3000, 7, 5000), (700, 33, 4096),
                                   (4096, 64, 64), (6000, 5, 1000)])
@pytest.mark.parametrize("pin", ["half", "bfloat16"])
def test_tc_gemm_scalecols_fused(api, M, N, K, pin):
    """The 16-bit power step: product with the split-K reduction fused into scalecols equals the
    product (ofrr_gemm) followed by ofrr_scalecols, bit for bit (both FP32 scaling forms)."""
    import torch
    from mixedprecisionofrr_gb300 import _lib as L

    rng = np.random.default_rng(M + N + K)
    A = rng.standard_normal((K, M))
    B = rng.standard_normal((K, N))
    B[:, 0] = 0.0  # zero column of C: left unscaled
    p = api.PREC[pin]
    Ad = api.to_device_cm(A, p)
    Bd = api.to_device_cm(B, p)
    ref = api.scalecols(api.gemm(Ad, "T", Bd, "single", pin), "single", pin)
    ctx = api.context()
    for fast in (1, 0):
        Cd = api.empty_cm(M, N, p)
        assert ctx.lib.ofrr_debug_gemm16_scalecols(ctx.h, p, M, N, K, Ad.data_ptr(), api.ld_of(Ad), Bd.data_ptr(),
                                                   api.ld_of(Bd), Cd.data_ptr(), api.ld_of(Cd), fast) == L.SUCCESS
        assert ctx.lib.ofrr_ctx_synchronize(ctx.h) == L.SUCCESS
        assert torch.equal(Cd.view(torch.int16), ref.view(torch.int16))


@pytest.mark.parametrize("M,N,K", [(8192, 64, 2048), (2048, 64, 8192), (64, 64, 8192), (300, 40, 1000)])
def test_tile_autotuner_plan_is_used_and_correct(api, M, N, K):
    """The autotuner times every tile width and K split of a shape and keeps the fastest; the product of
    that shape then runs with the tuned plan and stays within the FP32-accumulation tolerance."""
    t = api.autotune_gemm16(M, N, K, "half", reps=3)
    assert t["BN"] in (32, 64, 128) and t["splits"] >= 1 and t["us"] > 0
    plan = api.gemm16_plan(M, N, K, "half")
    assert plan["tuned"] and plan["BN"] == t["BN"] and plan["splits"] == t["splits"]
    rng = np.random.default_rng(M + N + K)
    p = api.PREC["half"]
    Ad = api.to_device_cm(rng.standard_normal((K, M)), p)
    Bd = api.to_device_cm(rng.standard_normal((K, N)), p)
    ref = Ad.double().cpu().numpy().T @ Bd.double().cpu().numpy()
    Cd = api.gemm(Ad, "T", Bd, "single", "single")
    got = Cd.double().cpu().numpy()
    assert np.max(np.abs(got - ref)) <= 2e-6 * np.sqrt(K) * np.max(np.abs(ref))


@pytest.mark.parametrize("M,N,K", [(128, 64, 128), (8192, 64, 2048), (300, 40, 1000), (64, 16, 8192)])
def test_e4m3_gemm_exact_on_representable_inputs(api, M, N, K):
    """The E4M3 tensor-core product: inputs that E4M3 holds exactly (small integers times powers of two,
    so the per-column scales reproduce them) give the exact product (FP32 sums of integers below 2^24)."""
    rng = np.random.default_rng(M + N + K)
    A = rng.integers(-7, 8, (K, M)).astype(np.float32) * 2.0 ** rng.integers(-3, 4, (1, M))
    B = rng.integers(-7, 8, (K, N)).astype(np.float32) * 2.0 ** rng.integers(-3, 4, (1, N))
    A[:, 0] = 0.0  # an all-zero column (scale 1, product zero)
    C = api.to_numpy(api.gemm_e4m3(A, B)).astype(np.float64)
    ref = A.astype(np.float64).T @ B.astype(np.float64)
    assert np.array_equal(C, ref)


def test_e4m3_gemm_quantisation_error(api):
    """Gaussian inputs: the product of the E4M3 copies is within the format's rounding (2^-4 relative per
    entry) of the exact product, in the Cauchy-Schwarz scale."""
    rng = np.random.default_rng(9)
    K, M, N = 2048, 512, 64
    A = rng.standard_normal((K, M)).astype(np.float32)
    B = rng.standard_normal((K, N)).astype(np.float32)
    C = api.to_numpy(api.gemm_e4m3(A, B)).astype(np.float64)
    ref = A.astype(np.float64).T @ B.astype(np.float64)
    bound = 2.0 ** -3 * np.sqrt(np.sum(A.astype(np.float64) ** 2, 0))[:, None] * np.sqrt(np.sum(B.astype(np.float64) ** 2, 0))[None, :]
    assert np.all(np.abs(C - ref) <= bound)
