"""The allocation-free Hessenberg entry point (ofrr_hessenberg_noalloc), called through the C ABI.

It exists for callers that cannot allocate GPU memory (a pool that already owns all of HBM, or a
request path that must not pay cudaMalloc's device-wide synchronisation).  Its scratch is one fixed
1 MiB device array shared by every call, so this test checks, on two different inputs in a row,
that its outputs equal those of ofrr_hessenberg (same arithmetic: bit for bit), and that a width
beyond the array's capacity is refused.  The file sorts last so a failure here leaves every other
test already run; it also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env(built_lib):
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from mixedprecisionofrr_gb300 import _lib as L
    from mixedprecisionofrr_gb300 import api

    return api, L, api.context()


def _noalloc(api, L, ctx, A, tin, tout, tc):
    import torch

    m, n = A.shape
    Ad = api.to_device_cm(A, tin)
    Q = api.empty_cm(m, n, tout)
    R = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    sel = torch.zeros(n, dtype=torch.int32, device="cuda")
    perm = torch.zeros(n, dtype=torch.int32, device="cuda")
    st = ctx.lib.ofrr_hessenberg_noalloc(C.c_void_p(ctx.stream.cuda_stream), tin, tout, tc, m, n, Ad.data_ptr(),
                                         api.ld_of(Ad), Q.data_ptr(), api.ld_of(Q), -1.0, R.data_ptr(),
                                         sel.data_ptr(), perm.data_ptr())
    assert st == 0, st
    ctx.stream.synchronize()
    # R was written column-major (n x n): element (i, j) at i + j n -> transpose of the row-major view
    return api.to_numpy(Q), R.cpu().numpy().T.copy(), sel.cpu().numpy() == 1, perm.cpu().numpy().astype(np.int64)


@pytest.mark.parametrize("tin,tout,tc", [("half", "half", "single"), ("double", "double", "double")])
def test_noalloc_matches_hessenberg_twice(env, tin, tout, tc):
    api, L, ctx = env
    pi, po, pc = api.PREC[tin], api.PREC[tout], api.PREC[tc]
    rng = np.random.default_rng(2)
    for call in range(2):  # two calls in a row: the shared scratch must not carry state over
        m, n = (3000, 48) if call == 0 else (1700, 33)
        A = rng.uniform(-1, 1, (m, n)).astype(np.float16 if tin == "half" else np.float64)
        if call == 1:
            A[:, 7] = A[:, 2]  # a dependent column: exercises the deselection path
        Qn, Rn, seln, permn = _noalloc(api, L, ctx, A, pi, po, pc)
        Q, R, sel, perm = api.hessenberg(A, tc, tout)
        assert np.array_equal(permn, perm)
        assert np.array_equal(seln, sel)
        assert np.array_equal(Qn, api.to_numpy(Q))
        assert np.array_equal(Rn, R)


def test_noalloc_at_the_fp64_width_limit(env):
    """n = 360 FP64 columns is the widest basis the 1 MiB array holds: it runs and matches."""
    api, L, ctx = env
    rng = np.random.default_rng(5)
    A = rng.uniform(-1, 1, (2000, 360))
    Qn, Rn, seln, permn = _noalloc(api, L, ctx, A, L.F64, L.F64, L.F64)
    Q, R, sel, perm = api.hessenberg(A, "double", "double")
    assert np.array_equal(permn, perm)
    assert np.array_equal(seln, sel)
    assert np.array_equal(Qn, api.to_numpy(Q))
    assert np.array_equal(Rn, R)


def test_noalloc_rejects_one_column_beyond_the_limit(env):
    api, L, ctx = env
    m, n = 2000, 361
    A = api.empty_cm(m, n, L.F64)
    Q = api.empty_cm(m, n, L.F64)
    st = ctx.lib.ofrr_hessenberg_noalloc(C.c_void_p(ctx.stream.cuda_stream), L.F64, L.F64, L.F64, m, n,
                                         A.data_ptr(), m, Q.data_ptr(), m, -1.0, Q.data_ptr(), Q.data_ptr(),
                                         Q.data_ptr())
    assert st == 2005  # OFRR_ERR_BLAS_INVALID_SIZE


def test_noalloc_rejects_in_place_type_change(env):
    api, L, ctx = env
    m, n = 256, 8
    A = api.empty_cm(m, n, L.F64)
    st = ctx.lib.ofrr_hessenberg_noalloc(C.c_void_p(ctx.stream.cuda_stream), L.F64, L.F32, L.F64, m, n,
                                         A.data_ptr(), m, A.data_ptr(), m, -1.0, A.data_ptr(), A.data_ptr(),
                                         A.data_ptr())
    assert st == 1000  # OFRR_ERR_INVALID_ARGUMENT


def test_noalloc_rejects_width_beyond_scratch(env):
    api, L, ctx = env
    assert ctx.lib.ofrr_hessenberg_noalloc_scratch_bytes() == 1 << 20
    m, n = 4000, 400  # 400 * 400 * 8 bytes of FP64 pivot rows exceed the 1 MiB array
    A = api.empty_cm(m, n, L.F64)
    Q = api.empty_cm(m, n, L.F64)
    st = ctx.lib.ofrr_hessenberg_noalloc(C.c_void_p(ctx.stream.cuda_stream), L.F64, L.F64, L.F64, m, n,
                                         A.data_ptr(), m, Q.data_ptr(), m, -1.0, Q.data_ptr(), Q.data_ptr(),
                                         Q.data_ptr())
    assert st == 2005  # OFRR_ERR_BLAS_INVALID_SIZE
