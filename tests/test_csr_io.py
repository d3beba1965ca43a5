"""On-disk CSR format of CPP/io/matrix_reader.cpp:8-50 (<prefix>_row_ptr.bin, _col_ind.bin,
_values.bin, _singular_values.bin).  The CPU tests read through the C ABI's host mode (no GPU call)
and compare with the oracle's restatement of MatrixReader, including the error cases; the GPU tests
stream the files into HBM, validate there, and run the sparse product and a solve on the result."""
import ctypes as C

import numpy as np
import pytest
import scipy.sparse as sp


def write_csr(prefix, indptr, indices, values, sv=None):
    np.asarray(indptr, np.int32).tofile(str(prefix) + "_row_ptr.bin")
    np.asarray(indices, np.int32).tofile(str(prefix) + "_col_ind.bin")
    np.asarray(values, np.float64).tofile(str(prefix) + "_values.bin")
    if sv is not None:
        np.asarray(sv, np.float64).tofile(str(prefix) + "_singular_values.bin")


def random_csr(m, n, density, seed):
    A = sp.random(m, n, density=density, random_state=seed, format="csr", dtype=np.float64)
    A.sort_indices()
    return A


@pytest.fixture(scope="module")
def lib(built_lib):
    from mixedprecisionofrr_gb300 import _lib as L

    return L.load()


def host_read(lib, prefix):
    nr, nz, nc = C.c_int64(), C.c_int64(), C.c_int64()
    st = lib.ofrr_csr_file_sizes(str(prefix).encode(), C.byref(nr), C.byref(nz))
    if st:
        return st, None
    ip = np.empty(nr.value + 1, np.int32)
    ix = np.empty(nz.value, np.int32)
    va = np.empty(nz.value, np.float64)
    st = lib.ofrr_csr_file_read(None, str(prefix).encode(), nr.value, nz.value, ip.ctypes.data, ix.ctypes.data,
                                va.ctypes.data, C.byref(nc), 0)
    return st, dict(indptr=ip, indices=ix, a_double=va, nrows=nr.value, ncols=nc.value)


def test_host_read_matches_oracle(lib, tmp_path):
    from oracle import ofrr_oracle as o

    A = random_csr(300, 200, 0.05, 1)
    p = tmp_path / "m"
    write_csr(p, A.indptr, A.indices, A.data, sv=np.linspace(1, 0, 7))
    st, got = host_read(lib, p)
    assert st == 0
    ref = o.read_csr_matrix(str(p))
    for k in ("indptr", "indices", "a_double"):
        assert np.array_equal(got[k], ref[k])
    assert (got["nrows"], got["ncols"]) == (ref["nrows"], ref["ncols"]) == (300, A.indices.max() + 1)
    n = C.c_int64(0)
    assert lib.ofrr_read_singular_values(str(p).encode(), C.byref(n), None) == 0 and n.value == 7
    sv = np.empty(7)
    assert lib.ofrr_read_singular_values(str(p).encode(), C.byref(n), sv.ctypes.data) == 0
    assert np.array_equal(sv, o.read_singular_values(str(p)))
    n = C.c_int64(3)  # capacity too small
    assert lib.ofrr_read_singular_values(str(p).encode(), C.byref(n), sv.ctypes.data) == 1000


def test_columns_from_largest_index(lib, tmp_path):
    """matrix_reader.cpp:40-43: trailing empty columns are not seen (cols = max index + 1)."""
    p = tmp_path / "t"
    write_csr(p, [0, 1, 2], [0, 3], [1.0, 2.0])
    st, got = host_read(lib, p)
    assert st == 0 and got["nrows"] == 2 and got["ncols"] == 4


@pytest.mark.parametrize("case,status", [
    ("missing", 5000), ("empty_values", 5001), ("partial_element", 5001), ("length_mismatch", 5001),
    ("rowptr_start", 5001), ("rowptr_decreasing", 5001), ("rowptr_end", 5001), ("negative_col", 5001)])
def test_malformed_files(lib, tmp_path, case, status):
    from oracle import ofrr_oracle as o

    p = tmp_path / case
    ip, ix, va = [0, 2, 3], [0, 1, 1], [1.0, 2.0, 3.0]
    if case == "rowptr_start":
        ip = [1, 2, 3]
    elif case == "rowptr_decreasing":
        ip = [0, 3, 2]
    elif case == "rowptr_end":
        ip = [0, 1, 2]
    elif case == "negative_col":
        ix = [0, -1, 1]
    write_csr(p, ip, ix, va)
    if case == "missing":
        (tmp_path / (case + "_values.bin")).unlink()
    elif case == "empty_values":
        (tmp_path / (case + "_values.bin")).write_bytes(b"")
    elif case == "partial_element":
        (tmp_path / (case + "_values.bin")).write_bytes(np.asarray(va).tobytes() + b"\x00")
    elif case == "length_mismatch":
        np.asarray(va[:2], np.float64).tofile(str(p) + "_values.bin")
    st, _ = host_read(lib, p)
    assert st == status
    if case in ("missing", "empty_values"):  # the reference throws here too
        with pytest.raises(RuntimeError):
            o.read_csr_matrix(str(p))


def test_singular_values_missing_is_empty(built_lib, tmp_path):
    from mixedprecisionofrr_gb300 import api

    assert api.read_singular_values(str(tmp_path / "none")).size == 0


@pytest.fixture(scope="module")
def api_gpu(built_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from mixedprecisionofrr_gb300 import api

    return api


@pytest.mark.gpu
@pytest.mark.parametrize("m,n,density", [(1000, 700, 0.01), (20000, 20000, 0.0005), (5, 3, 0.5)])
def test_device_read_equals_host_read(api_gpu, lib, tmp_path, m, n, density):
    api = api_gpu
    A = random_csr(m, n, density, m)
    if A.nnz == 0:
        A[0, 0] = 1.0
    p = tmp_path / "d"
    write_csr(p, A.indptr, A.indices, A.data)
    Ad = api.read_csr(str(p), symmetric=False)
    st, h = host_read(lib, p)
    assert st == 0
    assert np.array_equal(Ad.indptr.cpu().numpy(), h["indptr"])
    assert np.array_equal(Ad.indices.cpu().numpy(), h["indices"])
    assert np.array_equal(Ad.a_double.cpu().numpy(), h["a_double"])
    assert Ad.shape == (h["nrows"], h["ncols"])
    assert np.array_equal(Ad.a_single.cpu().numpy(), h["a_double"].astype(np.float32))
    assert np.array_equal(Ad.a_half.cpu().numpy(), h["a_double"].astype(np.float16))
    # the sparse product on the loaded operator
    X = np.random.default_rng(1).standard_normal((h["ncols"], 3))
    Y = api.to_numpy(api.csrmv(Ad, "N", X, "double", "double"))
    ref = sp.csr_matrix((h["a_double"], h["indices"], h["indptr"]), shape=Ad.shape) @ X
    assert np.allclose(Y, ref, rtol=1e-13, atol=1e-13)


@pytest.mark.gpu
def test_device_read_rejects_malformed(api_gpu, tmp_path):
    """the GPU validation pass reports the malformed structure (all accesses stay inside the arrays,
    whose lengths come from the file sizes)"""
    from mixedprecisionofrr_gb300 import _lib as L

    api = api_gpu
    for k, (ip, ix) in enumerate((([0, 3, 2], [0, 1, 1]), ([0, 2, 3], [0, -5, 1]), ([0, 1, 2], [0, 1, 1]))):
        p = tmp_path / f"bad{k}"
        write_csr(p, ip, ix, [1.0, 2.0, 3.0])
        with pytest.raises(L.OfrrError) as e:
            api.read_csr(str(p))
        assert e.value.status == 5001
    assert api.context().lib.ofrr_ctx_synchronize(api.context().h) == 0  # the context stays usable


@pytest.mark.gpu
def test_solve_on_file_operator_equals_in_memory(api_gpu, tmp_path):
    """si_eig on the 2D Laplacian read from disk equals the solve on the in-memory operator, and the
    eigenvalues stored beside it (the _singular_values file) are reached"""
    from oracle import ofrr_oracle as o

    api = api_gpu
    A = o.laplacian_2d(12).tocsr()
    A.sort_indices()
    lam = np.sort(o.laplacian_2d_eigs(12))[::-1]
    p = tmp_path / "lap"
    write_csr(p, A.indptr, A.indices, A.data, sv=lam)
    Af = api.read_csr(str(p))
    assert Af.symmetric
    Am = api.CsrMatrix(A, symmetric=True)
    n = A.shape[0]
    V0 = o.randn_block(42, n, 24)
    _, d_f, inf_f = api.subspace_iter_eig(Af, n, 24, V0=V0, nev=3, tol=1e-10, maxiter=3000, mode="fp64")
    _, d_m, inf_m = api.subspace_iter_eig(Am, n, 24, V0=V0, nev=3, tol=1e-10, maxiter=3000, mode="fp64")
    assert inf_f.status == 0 and np.array_equal(d_f, d_m)
    sv = api.read_singular_values(str(p))
    assert np.array_equal(sv, lam)
    assert np.allclose(d_f[:3], sv[:3], rtol=1e-9)
