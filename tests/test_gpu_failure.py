"""Failure detection on the GPU without a fault: every wait in the library's kernels is bounded; when
one gives up, the kernel records the timeout in the context's status words and returns, and the next
synchronisation reports OFRR_ERR_DEVICE_TIMEOUT.  The test makes a wait run out on purpose (an
mbarrier that nothing arrives on, 1 ms limit) and checks the status and that the context still works."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def api(built_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from mixedprecisionofrr_gb300 import api as a

    return a


def test_bounded_wait_timeout_is_reported_and_context_stays_usable(api):
    from mixedprecisionofrr_gb300 import _lib as L

    ctx = api.context()
    lib = ctx.lib
    assert lib.ofrr_ctx_synchronize(ctx.h) == L.SUCCESS
    assert lib.ofrr_debug_bounded_wait(ctx.h, 1_000_000) == L.SUCCESS
    assert lib.ofrr_ctx_synchronize(ctx.h) == 6004  # OFRR_ERR_DEVICE_TIMEOUT
    assert lib.ofrr_ctx_synchronize(ctx.h) == L.SUCCESS  # the status words were cleared
    # the context still computes: an emulated FP64 product within its error bound 2^-33 |A|'|B|
    rng = np.random.default_rng(3)
    A = rng.standard_normal((300, 40))
    B = rng.standard_normal((300, 8))
    got = api.gemm_f64_emulated(A, B).cpu().numpy()
    assert np.all(np.abs(got - A.T @ B) <= 2.0 ** -33 * (np.abs(A).T @ np.abs(B)))
