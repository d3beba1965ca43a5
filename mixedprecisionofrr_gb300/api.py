"""Python mirror of the reference's MATLAB interface, calling libofrr_gb300.so through its C ABI.

Function names, argument meanings and defaults follow ``MATLAB/+src`` of the reference
(``subspace_iter_eig``, ``subspace_iter_svd``, ``arnoldi_hess_eig``, ``eig_rr``, ``svd_rr``,
``hessenberg``, ``scalecols``, ``gemm``, ``csrmv``), with precisions given by name
('double', 'single', 'half', 'bfloat16').  Device memory comes from PyTorch (plumbing only);
every computation is a call into the CUDA library, and a missing library raises.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import _lib as L

try:
    import torch
except Exception as e:  # pragma: no cover - torch is part of the supported environment
    raise RuntimeError("PyTorch is required for device memory management") from e

PREC = {"double": L.F64, "single": L.F32, "half": L.F16, "bfloat16": L.BF16}
TORCH_DT = {L.F64: torch.float64, L.F32: torch.float32, L.F16: torch.float16, L.BF16: torch.bfloat16}
NP_DT = {L.F64: np.float64, L.F32: np.float32, L.F16: np.float16}


def _p(name) -> int:
    if isinstance(name, int):
        return name
    return PREC[name]


def _eps(p: int) -> float:
    return {L.F64: 2.0 ** -52, L.F32: 2.0 ** -23, L.F16: 2.0 ** -10, L.BF16: 2.0 ** -7}[p]


class Context:
    """Owns an ofrr_ctx bound to a CUDA device and stream (default: torch's current stream)."""

    def __init__(self, device: int = 0, stream=None):
        self.lib = L.load()
        torch.cuda.init()
        self.device = device
        if stream is None:
            stream = torch.cuda.current_stream(device)
            if stream.cuda_stream == 0:
                # the library never runs on the legacy default stream: give torch and the library one
                # shared non-blocking stream so that tensor reads see the library's results in order
                stream = torch.cuda.Stream(device)
                torch.cuda.set_stream(stream)
        self.stream = stream
        h = C.c_void_p()
        L.check(self.lib.ofrr_ctx_create(C.byref(h), device, C.c_void_p(stream.cuda_stream)), "ofrr_ctx_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.ofrr_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def synchronize(self):
        L.check(self.lib.ofrr_ctx_synchronize(self.h), "synchronize")

    def set_trace(self, path=None):
        """Append one JSON line per solve on this context to `path` (None: tracing off)."""
        L.check(self.lib.ofrr_ctx_set_trace(self.h, str(path).encode() if path else None), "ofrr_ctx_set_trace")

    @property
    def launch_count(self) -> int:
        return int(self.lib.ofrr_ctx_launch_count(self.h))

    def reset_launch_count(self):
        self.lib.ofrr_ctx_reset_launch_count(self.h)


_CTX: Optional[Context] = None


def context() -> Context:
    global _CTX
    if _CTX is None:
        _CTX = Context(torch.cuda.current_device())
    return _CTX


# ---- column-major device buffers ----------------------------------------------------------
def empty_cm(m: int, n: int, p: int, device="cuda") -> "torch.Tensor":
    """m x n column-major device tensor (strides (1, m))."""
    return torch.empty((n, m), dtype=TORCH_DT[p], device=device).t()


def to_device_cm(x, p: int, device="cuda") -> "torch.Tensor":
    """Copy (numpy or torch, any layout) into a fresh column-major device tensor of precision p."""
    if isinstance(x, np.ndarray):
        a = x if x.ndim == 2 else x.reshape(-1, 1)
        if p in NP_DT:
            a = a.astype(NP_DT[p], copy=False)  # numpy rounds directly (no double rounding via float)
        t = torch.from_numpy(np.ascontiguousarray(a))
    else:
        t = x if x.dim() == 2 else x.reshape(-1, 1)
    out = empty_cm(t.shape[0], t.shape[1], p, device)
    out.copy_(t.to(device=device))
    return out


def is_cm(t) -> bool:
    return isinstance(t, torch.Tensor) and t.is_cuda and t.dim() == 2 and (t.stride(0) == 1 or t.shape[1] == 1)


def ld_of(t) -> int:
    return max(1, t.stride(1) if t.shape[1] > 1 else t.shape[0])


def dtype_of(t) -> int:
    for k, v in TORCH_DT.items():
        if t.dtype == v:
            return k
    raise TypeError(f"unsupported dtype {t.dtype}")


def to_numpy(t) -> np.ndarray:
    if t.dtype == torch.bfloat16:
        t = t.float()
    return t.detach().cpu().numpy()


# ---- CSR operator -----------------------------------------------------------------------------
class CsrMatrix:
    """Device CSR with value copies per precision (MATLAB/+src/+csr/sparse2csr.m:21-50)."""

    def __init__(self, A, symmetric: Optional[bool] = None, device="cuda"):
        import scipy.sparse as sp

        if isinstance(A, dict):
            indptr, indices, data = A["indptr"], A["indices"], A["a_double"]
            shape = (A["nrows"], A["ncols"])
        else:
            M = sp.csr_matrix(A, dtype=np.float64)
            M.sort_indices()
            indptr, indices, data, shape = M.indptr, M.indices, M.data, M.shape
        self.shape = shape
        self.nnz = int(len(data))
        self.indptr = torch.as_tensor(np.asarray(indptr, np.int32), device=device)
        self.indices = torch.as_tensor(np.asarray(indices, np.int32), device=device)
        d = np.asarray(data, np.float64)
        self.a_double = torch.as_tensor(d, device=device)
        self.a_single = torch.as_tensor(d.astype(np.float32), device=device)
        with np.errstate(over="ignore"):  # values beyond the FP16 range become +-inf, as sparse2csr.m's cast
            self.a_half = torch.as_tensor(d.astype(np.float16), device=device)
        if symmetric is None:
            M = sp.csr_matrix((d, np.asarray(indices), np.asarray(indptr)), shape=shape)
            symmetric = shape[0] == shape[1] and abs(M - M.T).max() == 0
        self.symmetric = bool(symmetric)

    @classmethod
    def from_device(cls, indptr, indices, a_double, shape, symmetric: Optional[bool] = None):
        """Wrap device arrays (int32 indptr / indices, FP64 values) without a host round trip; the FP32
        and FP16 value copies are rounded once from the FP64 values on the device (ofrr_cast), as
        sparse2csr.m:48-49 rounds them."""
        self = cls.__new__(cls)
        self.shape = (int(shape[0]), int(shape[1]))
        self.nnz = nnz = int(a_double.numel())
        self.indptr, self.indices, self.a_double = indptr, indices, a_double
        self.a_single = torch.empty(nnz, dtype=torch.float32, device=a_double.device)
        self.a_half = torch.empty(nnz, dtype=torch.float16, device=a_double.device)
        if nnz:
            ctx = context()
            for t, code in ((self.a_single, L.F32), (self.a_half, L.F16)):
                L.check(ctx.lib.ofrr_cast(ctx.h, L.F64, code, nnz, 1, a_double.data_ptr(), nnz, t.data_ptr(), nnz),
                        "cast")
        if symmetric is None:
            import scipy.sparse as sp

            M = sp.csr_matrix((a_double.cpu().numpy(), indices.cpu().numpy(), indptr.cpu().numpy()), shape=self.shape)
            symmetric = self.shape[0] == self.shape[1] and abs(M - M.T).max() == 0
        self.symmetric = bool(symmetric)
        return self

    def struct(self) -> L.ofrr_csr:
        s = L.ofrr_csr()
        s.nrows, s.ncols, s.nnz = self.shape[0], self.shape[1], self.nnz
        s.indptr = self.indptr.data_ptr()
        s.indices = self.indices.data_ptr() if self.nnz else None
        s.a_double = self.a_double.data_ptr() if self.nnz else None
        s.a_single = self.a_single.data_ptr() if self.nnz else None
        s.a_half = self.a_half.data_ptr() if self.nnz else None
        return s


def read_csr(prefix: str, symmetric: Optional[bool] = None, on_device: bool = True) -> CsrMatrix:
    """CPP/io/matrix_reader.cpp:8-45 (MatrixReader::read_csr_matrix): <prefix>_row_ptr.bin,
    _col_ind.bin (int32, 0-based) and _values.bin (float64) into a device CsrMatrix; columns = largest
    column index + 1.  on_device streams the files into HBM through pinned staging buffers and
    validates the structure on the GPU; otherwise they are read and checked on the host, then copied.
    Raises OfrrError (FILE_NOT_FOUND / INVALID_FORMAT) where the reference throws."""
    nrows, nnz = C.c_int64(), C.c_int64()
    pfx = os.fsencode(prefix)
    lib = L.load()
    L.check(lib.ofrr_csr_file_sizes(pfx, C.byref(nrows), C.byref(nnz)), "read_csr")
    ncols = C.c_int64()
    if on_device:
        ctx = context()
        ip = torch.empty(nrows.value + 1, dtype=torch.int32, device="cuda")
        ix = torch.empty(nnz.value, dtype=torch.int32, device="cuda")
        va = torch.empty(nnz.value, dtype=torch.float64, device="cuda")
        L.check(lib.ofrr_csr_file_read(ctx.h, pfx, nrows.value, nnz.value, ip.data_ptr(), ix.data_ptr(), va.data_ptr(),
                                       C.byref(ncols), 1), "read_csr")
        return CsrMatrix.from_device(ip, ix, va, (nrows.value, ncols.value), symmetric)
    ip = np.empty(nrows.value + 1, np.int32)
    ix = np.empty(nnz.value, np.int32)
    va = np.empty(nnz.value, np.float64)
    L.check(lib.ofrr_csr_file_read(None, pfx, nrows.value, nnz.value, ip.ctypes.data, ix.ctypes.data, va.ctypes.data,
                                   C.byref(ncols), 0), "read_csr")
    return CsrMatrix({"indptr": ip, "indices": ix, "a_double": va, "nrows": nrows.value, "ncols": ncols.value},
                     symmetric)


def rand_points(seed: int, n: int, d: int, type: int = 0):
    """n x d point set on the device (MATLAB/+src/+kernel/generate_pts.m types 20/21/22/23/30/31/32, or
    type 0: the uniform box of CPP/testproblems/gaussian_kernel.hpp:36-40), FP64, column-major."""
    ctx = context()
    X = empty_cm(n, d, L.F64)
    L.check(ctx.lib.ofrr_rand_points(ctx.h, seed, n, d, type, X.data_ptr(), ld_of(X)), "rand_points")
    return X


def gaussian(X, Y, l: float, f: float, s: float, precision_output="double"):
    """MATLAB/+src/+kernel/gaussian.m: K(X, Y) = f^2 exp(-D2 / (2 l^2)) + s^2 eye on the device."""
    ctx = context()
    Xd = X if (is_cm(X) and dtype_of(X) == L.F64) else to_device_cm(X, L.F64)
    Yd = Y if (is_cm(Y) and dtype_of(Y) == L.F64) else to_device_cm(Y, L.F64)
    po = _p(precision_output)
    K = empty_cm(Xd.shape[0], Yd.shape[0], po)
    L.check(ctx.lib.ofrr_gaussian_kernel(ctx.h, 1, Xd.shape[0], Yd.shape[0], Xd.shape[1], Xd.data_ptr(), ld_of(Xd),
                                         Yd.data_ptr(), ld_of(Yd), l, f, s, po, K.data_ptr(), ld_of(K)), "gaussian")
    return K


def generate_gaussian_kernel(f: float, l: float, s: float, seed: int, n: int, d: int, precision="double"):
    """CPP/testproblems/gaussian_kernel.hpp:14-77 on the device: points uniform in [0, n^(1/d))^d (seeded
    counter-based draws), K = f^2 (1 + s^2) on the diagonal, f^2 exp(-|x_i - x_j|^2 / (2 l^2)) off it;
    returns (K, X) on the device.  Raises OfrrError (INVALID_ARGUMENT) where the reference throws."""
    ctx = context()
    if not (l > 0 and s >= 0 and n > 0 and d > 0):
        L.check(1000, "generate_gaussian_kernel")  # OFRR_ERR_INVALID_ARGUMENT
    X = rand_points(seed, n, d, 0)
    po = _p(precision)
    K = empty_cm(n, n, po)
    L.check(ctx.lib.ofrr_gaussian_kernel(ctx.h, 0, n, n, d, X.data_ptr(), ld_of(X), X.data_ptr(), ld_of(X), l, f, s,
                                         po, K.data_ptr(), ld_of(K)), "generate_gaussian_kernel")
    return K, X


def read_singular_values(prefix: str) -> np.ndarray:
    """CPP/io/matrix_reader.cpp:47-50: <prefix>_singular_values.bin (float64); empty when the file is
    missing or unreadable, as in the reference."""
    lib = L.load()
    pfx = os.fsencode(prefix)
    n = C.c_int64(0)
    if lib.ofrr_read_singular_values(pfx, C.byref(n), None) != L.SUCCESS:
        return np.empty(0)
    out = np.empty(n.value, np.float64)
    if lib.ofrr_read_singular_values(pfx, C.byref(n), out.ctypes.data) != L.SUCCESS:
        return np.empty(0)
    return out


@dataclass
class Operator:
    """Keeps the ofrr_operator struct and the tensors it points to alive."""
    op: L.ofrr_operator
    keep: tuple
    m: int
    n: int


def operator(A, symmetric: Optional[bool] = None, dtype: str | int = "double") -> Operator:
    op = L.ofrr_operator()
    if isinstance(A, Operator):
        return A
    if isinstance(A, CsrMatrix):
        op.kind = L.OP_CSR
        op.nrows, op.ncols = A.shape
        op.symmetric = int(A.symmetric if symmetric is None else symmetric)
        op.dtype = L.F64
        op.csr = A.struct()
        return Operator(op, (A,), A.shape[0], A.shape[1])
    t = A if is_cm(A) else to_device_cm(A if not isinstance(A, np.ndarray) else A.astype(np.float64), _p(dtype))
    op.kind = L.OP_DENSE
    op.nrows, op.ncols = t.shape
    if symmetric is None:
        symmetric = t.shape[0] == t.shape[1] and bool(torch.equal(t, t.t()))
    op.symmetric = int(symmetric)
    op.dtype = dtype_of(t)
    op.data = t.data_ptr()
    op.ld = ld_of(t)
    return Operator(op, (t,), t.shape[0], t.shape[1])


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int))


# ---- building blocks --------------------------------------------------------------------------
def randn(seed: int, n: int, k: int, precision="double"):
    ctx = context()
    p = _p(precision)
    out = empty_cm(n, k, p)
    L.check(ctx.lib.ofrr_randn(ctx.h, seed, n, k, p, out.data_ptr(), max(n, 1)), "ofrr_randn")
    return out


def randn_host(seed: int, n: int, k: int) -> np.ndarray:
    out = np.zeros(n * k, np.float64)
    L.load().ofrr_randn_host(seed, n, k, _dp(out))
    return out.reshape(k, n).T.copy()


def scalecols(U, precision_compute="double", precision_output=None, return_pivots=False):
    """MATLAB/+src/+mvops/scalecols.m."""
    ctx = context()
    pc = _p(precision_compute)
    po = _p(precision_output or precision_compute)
    X = to_device_cm(U, po)
    m, n = X.shape
    piv = torch.zeros(n, dtype=torch.int32, device="cuda")
    L.check(ctx.lib.ofrr_scalecols(ctx.h, po, pc, m, n, X.data_ptr(), ld_of(X), piv.data_ptr()), "scalecols")
    return (X, piv) if return_pivots else X


def iamax(x):
    """1-based index of max |x| and the value there (CPP/linalg/blas/mvops.hpp:98)."""
    ctx = context()
    t = x if isinstance(x, torch.Tensor) and x.is_cuda else torch.as_tensor(np.asarray(x), device="cuda")
    t = t.contiguous().reshape(-1)
    idx = C.c_int()
    val = C.c_double()
    L.check(ctx.lib.ofrr_iamax(ctx.h, dtype_of(t[:, None]), t.numel(), t.data_ptr(), C.byref(idx), C.byref(val)),
            "iamax")
    return idx.value, val.value


def check_special_values(X) -> int:
    ctx = context()
    t = X if is_cm(X) else to_device_cm(X, L.F64)
    return ctx.lib.ofrr_check_special_values(ctx.h, dtype_of(t), t.shape[0], t.shape[1], t.data_ptr(), ld_of(t))


def hessenberg(A, precision_compute="double", precision_output=None, select_tol=None, precision_input=None):
    """MATLAB/+src/+qr/hessenberg.m (three-output form): returns Q (device), R, select, perm (host)."""
    ctx = context()
    pc = _p(precision_compute)
    po = _p(precision_output or precision_compute)
    pi = _p(precision_input) if precision_input else po
    X = to_device_cm(A, pi)
    m, n = X.shape
    Q = empty_cm(m, n, po)
    R = np.zeros(n * n, np.float64)
    skip = np.zeros(n, np.int32)
    perm = np.zeros(n, np.int32)
    st = -1.0 if select_tol is None else float(select_tol)
    L.check(ctx.lib.ofrr_hessenberg(ctx.h, pi, po, pc, m, n, X.data_ptr(), ld_of(X), Q.data_ptr(), ld_of(Q), st,
                                    _dp(R), _ip(skip), _ip(perm)), "hessenberg")
    return Q, R.reshape(n, n).T.copy(), skip == 0, perm.astype(np.int64)


def gemm(A, trans: str, B, precision_compute="double", precision_output=None, alpha=1.0, beta=0.0, Cin=None):
    """MATLAB/+src/+mvops/gemm.m: C = op(A) B computed in precision_compute, stored in precision_output."""
    ctx = context()
    pc = _p(precision_compute)
    po = _p(precision_output or precision_compute)
    Ad = A if is_cm(A) else to_device_cm(A, pc)
    Bd = B if is_cm(B) else to_device_cm(B, pc)
    tA = 1 if trans == "T" else 0
    M = Ad.shape[1] if tA else Ad.shape[0]
    K = Ad.shape[0] if tA else Ad.shape[1]
    N = Bd.shape[1]
    Cd = Cin if Cin is not None else empty_cm(M, N, po)
    L.check(ctx.lib.ofrr_gemm(ctx.h, tA, 0, dtype_of(Ad), dtype_of(Bd), pc, po, M, N, K, alpha, Ad.data_ptr(),
                              ld_of(Ad), Bd.data_ptr(), ld_of(Bd), beta, Cd.data_ptr(), ld_of(Cd)), "gemm")
    return Cd


def gemm_f64_emulated(A, B):
    """C = A' B for FP64 A (K x M), B (K x N) on the tensor cores through exact BF16 digit slices."""
    ctx = context()
    Ad = A if is_cm(A) else to_device_cm(A, L.F64)
    Bd = B if is_cm(B) else to_device_cm(B, L.F64)
    K, M = Ad.shape
    N = Bd.shape[1]
    Cd = empty_cm(M, N, L.F64)
    L.check(ctx.lib.ofrr_gemm_f64_emulated(ctx.h, M, N, K, Ad.data_ptr(), ld_of(Ad), Bd.data_ptr(), ld_of(Bd),
                                           Cd.data_ptr(), ld_of(Cd)), "gemm_f64_emulated")
    return Cd


def csrmv(Acsr: CsrMatrix, trans: str, x, precision_compute="double", precision_output=None):
    """MATLAB/+src/+csr/csrmv.m."""
    ctx = context()
    pc = _p(precision_compute)
    po = _p(precision_output or precision_compute)
    X = x if is_cm(x) else to_device_cm(x, pc)
    tr = 1 if trans == "T" else 0
    nout = Acsr.shape[1] if tr else Acsr.shape[0]
    Y = empty_cm(nout, X.shape[1], po)
    s = Acsr.struct()
    L.check(ctx.lib.ofrr_csrmm(ctx.h, C.byref(s), tr, dtype_of(X), pc, po, X.shape[1], X.data_ptr(), ld_of(X),
                               Y.data_ptr(), ld_of(Y)), "csrmm")
    return Y


def syev(A):
    """Ascending eigenvalues / orthonormal eigenvectors of a small symmetric matrix (FP64, device)."""
    ctx = context()
    X = to_device_cm(A, L.F64)
    n = X.shape[0]
    w = torch.zeros(n, dtype=torch.float64, device="cuda")
    L.check(ctx.lib.ofrr_syev(ctx.h, n, X.data_ptr(), ld_of(X), w.data_ptr()), "syev")
    return to_numpy(w), to_numpy(X)


def sygv(A, B):
    ctx = context()
    X = to_device_cm(A, L.F64)
    Bd = to_device_cm(B, L.F64)
    n = X.shape[0]
    w = torch.zeros(n, dtype=torch.float64, device="cuda")
    L.check(ctx.lib.ofrr_sygv(ctx.h, n, X.data_ptr(), ld_of(X), Bd.data_ptr(), ld_of(Bd), w.data_ptr()), "sygv")
    return to_numpy(w), to_numpy(X)


def gs_basis(A, classical: bool = False, precision_compute="double", precision_output=None, select_tol=None,
             orth_tol=None, reorth_tol=None, precision_input=None):
    """MATLAB/+src/+qr/mgs.m (classical=False) or cgs.m: returns (Q, R, skip) with Q on the device at
    the input's column positions (dropped columns zero), R (n x n) and skip flags on the host."""
    ctx = context()
    pc = _p(precision_compute)
    po = _p(precision_output or precision_compute)
    pin = _p(precision_input) if precision_input else po
    Ad = A if (is_cm(A) and dtype_of(A) == pin) else to_device_cm(A, pin)
    m, n = Ad.shape
    Q = empty_cm(m, n, po)
    R = np.zeros(n * n)  # column-major from the library
    skip = np.zeros(n, np.int32)
    nan = float("nan")
    L.check(ctx.lib.ofrr_gs_basis(ctx.h, int(classical), dtype_of(Ad), po, pc, m, n, Ad.data_ptr(), ld_of(Ad),
                                  Q.data_ptr(), ld_of(Q), -1.0 if select_tol is None else select_tol,
                                  nan if orth_tol is None else orth_tol, nan if reorth_tol is None else reorth_tol,
                                  R.ctypes.data_as(C.POINTER(C.c_double)), skip.ctypes.data_as(C.POINTER(C.c_int))),
            "gs_basis")
    return Q, R.reshape((n, n), order="F"), skip


def lu_basis(A, precision_compute="double", precision_output=None, select_tol=None, precision_input=None):
    """MATLAB/+src/+qr/lu.m: returns (Q, U, skip): Q the un-permuted L on the device (dropped columns
    zero), U (n x n) and skip flags on the host."""
    ctx = context()
    pc = _p(precision_compute)
    po = _p(precision_output or precision_compute)
    pin = _p(precision_input) if precision_input else po
    Ad = A if (is_cm(A) and dtype_of(A) == pin) else to_device_cm(A, pin)
    m, n = Ad.shape
    Q = empty_cm(m, n, po)
    U = np.zeros(n * n)
    skip = np.zeros(n, np.int32)
    L.check(ctx.lib.ofrr_lu_basis(ctx.h, dtype_of(Ad), po, pc, m, n, Ad.data_ptr(), ld_of(Ad), Q.data_ptr(), ld_of(Q),
                                  -1.0 if select_tol is None else select_tol,
                                  U.ctypes.data_as(C.POINTER(C.c_double)), skip.ctypes.data_as(C.POINTER(C.c_int))),
            "lu_basis")
    return Q, U.reshape((n, n), order="F"), skip


ORTH = {"hessenberg": L.ORTH_HESSENBERG, "mgs": L.ORTH_MGS, "cgs": L.ORTH_CGS, "lu": L.ORTH_LU}


# ---- solvers ------------------------------------------------------------------------------------
def options(**kw) -> L.ofrr_options:
    o = L.ofrr_options()
    L.load().ofrr_options_default(C.byref(o))
    for k, v in kw.items():
        if v is None:
            continue
        if k.startswith("p_"):
            v = _p(v)
        setattr(o, k, v)
    return o


def _prec_opts(precision_compute, precision_output, ph_c, ph_o, prr_c, prr_o):
    pc = precision_compute
    po = precision_output or pc
    return dict(p_compute=pc, p_output=po, p_hess_compute=ph_c or pc, p_hess_output=ph_o or po,
                p_rr_compute=prr_c or pc, p_rr_output=prr_o or po)


def eig_rr(A, V, precision_compute="double", precision_output=None, precision_rr_compute=None,
           precision_rr_output=None, use_generalized=False, generalized_tol=None, symmetric=None):
    """MATLAB/+src/+rr/eig_rr.m on the basis V; returns (Ritz vectors, Ritz values desc)."""
    ctx = context()
    op = operator(A, symmetric)
    po = _p(precision_output or precision_compute)
    Vd = to_device_cm(V, po)
    b = Vd.shape[1]
    gtol = generalized_tol
    if gtol is None:
        gtol = 1e-10  # eig_rr.m:105-107 (precision_eig = double)
    o = options(use_generalized=int(use_generalized), generalized_tol=gtol,
                **_prec_opts(precision_compute, precision_output, None, None, precision_rr_compute,
                             precision_rr_output))
    d = np.zeros(b)
    L.check(ctx.lib.ofrr_rr_eig(ctx.h, C.byref(op.op), C.byref(o), b, Vd.data_ptr(), ld_of(Vd), _dp(d)), "rr_eig")
    return Vd, d


def svd_rr(A, U, V, precision_compute="double", precision_output=None, precision_rr_compute=None,
           precision_rr_output=None, use_generalized=True, generalized_tol=None):
    """MATLAB/+src/+rr/svd_rr.m (generalized form) on the bases U, V."""
    ctx = context()
    op = operator(A, False)
    po = _p(precision_output or precision_compute)
    Ud = to_device_cm(U, po)
    Vd = to_device_cm(V, po)
    b = Ud.shape[1]
    o = options(use_generalized=int(use_generalized), generalized_tol=1e-10 if generalized_tol is None else float(generalized_tol),
                **_prec_opts(precision_compute, precision_output, None, None, precision_rr_compute,
                             precision_rr_output))
    s = np.zeros(b)
    L.check(ctx.lib.ofrr_rr_svd(ctx.h, C.byref(op.op), C.byref(o), b, Ud.data_ptr(), ld_of(Ud), _dp(s),
                                Vd.data_ptr(), ld_of(Vd)), "rr_svd")
    return Ud, s, Vd


@dataclass
class SolveInfo:
    status: int
    iterations: int
    matvecs: int
    converged: int
    basis_width: int
    max_residual: float
    residuals: np.ndarray
    escalations: int = 0


def _info(st, inf, res):
    return SolveInfo(st, inf.iterations, inf.matvecs, inf.converged, inf.basis_width, inf.max_residual, res,
                     inf.escalations)


def subspace_iter_eig(A, n: int, k: int, precision_compute="double", precision_output=None, seed: int = 42,
                      maxiter: int = 5, step_size: int = 1, precision_hess_compute=None, precision_hess_output=None,
                      precision_rr_compute=None, precision_rr_output=None, use_generalized=True,
                      generalized_tol=0.0, select_tol=None, symmetric=None, V0=None, mode="reference",
                      tol=0.0, nev=None, check_every=1, orth="hessenberg", step_size_f64=0):
    """MATLAB/+src/+subspace/subspace_iter_eig.m; returns (V, d, info) with V on the device.  orth: the
    basis ("hessenberg"; "mgs" = the MATLAB file's default function_orth; "cgs"; "lu")."""
    ctx = context()
    op = operator(A, symmetric)
    modes = {"reference": L.MODE_REFERENCE, "mixed": L.MODE_MIXED, "fp64": L.MODE_FP64}
    o = options(mode=modes[mode], maxiter=maxiter, step_size=step_size, block=min(k, n), nev=nev or min(k, n),
                tol=tol, use_generalized=int(use_generalized), generalized_tol=generalized_tol,
                select_tol=-1.0 if select_tol is None else select_tol, seed=seed,
                use_start_block=int(V0 is not None), check_every=check_every, orth=ORTH[orth],
                step_size_f64=step_size_f64,
                **_prec_opts(precision_compute, precision_output, precision_hess_compute, precision_hess_output,
                             precision_rr_compute, precision_rr_output))
    po = o.p_output if mode == "reference" else L.F64
    b = o.block
    V = to_device_cm(V0, po) if V0 is not None else empty_cm(n, b, po)
    d = np.zeros(b)
    res = np.zeros(b)
    inf = L.ofrr_info()
    st = ctx.lib.ofrr_si_eig(ctx.h, C.byref(op.op), C.byref(o), V.data_ptr(), ld_of(V), _dp(d), _dp(res),
                             C.byref(inf))
    if st not in (L.SUCCESS, L.ERR_SOLVER_MAX_ITERATIONS):
        L.check(st, "si_eig")
    return V, d, _info(st, inf, res)


def subspace_iter_svd(A, m: int, n: int, k: int, precision_compute="double", precision_output=None, seed: int = 42,
                      maxiter: int = 5, step_size: int = 1, precision_hess_compute=None, precision_hess_output=None,
                      precision_rr_compute=None, precision_rr_output=None, use_generalized=True,
                      generalized_tol=0.0, select_tol=None, V0=None, mode="reference", tol=0.0, nev=None,
                      check_every=1, orth="hessenberg", power_fp8=False, step_size_f64=0):
    """MATLAB/+src/+subspace/subspace_iter_svd.m; returns (U, s, V, info) with U, V on the device.  orth:
    the basis of both blocks ("hessenberg", "mgs" or "cgs").  power_fp8 (mixed mode, dense A): the FP8
    variant, E4M3 products in the 16-bit power steps.  step_size_f64 (mixed mode): power steps per outer
    iteration of the FP64 phase (0: step_size)."""
    ctx = context()
    op = operator(A, False)
    modes = {"reference": L.MODE_REFERENCE, "mixed": L.MODE_MIXED, "fp64": L.MODE_FP64}
    b = min(k, n)
    o = options(mode=modes[mode], maxiter=maxiter, step_size=step_size, block=b, nev=nev or b, tol=tol,
                use_generalized=int(use_generalized), generalized_tol=generalized_tol,
                select_tol=-1.0 if select_tol is None else select_tol, seed=seed,
                use_start_block=int(V0 is not None), check_every=check_every, orth=ORTH[orth],
                power_fp8=int(power_fp8), step_size_f64=step_size_f64,
                **_prec_opts(precision_compute, precision_output, precision_hess_compute, precision_hess_output,
                             precision_rr_compute, precision_rr_output))
    po = o.p_output if mode == "reference" else L.F64
    V = to_device_cm(V0, po) if V0 is not None else empty_cm(n, b, po)
    U = empty_cm(m, b, po)
    s = np.zeros(b)
    res = np.zeros(b)
    inf = L.ofrr_info()
    st = ctx.lib.ofrr_si_svd(ctx.h, C.byref(op.op), C.byref(o), U.data_ptr(), ld_of(U), _dp(s), V.data_ptr(),
                             ld_of(V), _dp(res), C.byref(inf))
    if st not in (L.SUCCESS, L.ERR_SOLVER_MAX_ITERATIONS):
        L.check(st, "si_svd")
    return U, s, V, _info(st, inf, res)


def arnoldi_hess_eig(A, n: int, k: int, precision_compute="double", precision_output=None, seed: int = 42,
                     maxiter: int = 5, kdim=None, select_tol=None, generalized_tol=0.0, symmetric=None, v0=None,
                     mode="reference", tol=0.0, restart_keep: int = 0):
    """MATLAB/+src/+krylov/arnoldi_hess_eig.m; returns (V, d, info).

    mode "mixed" / "fp64" with a CSR operator: the thick-restart Hessenberg process (about restart_keep
    leading Ritz values' invariant subspace kept, 0 = the default block; 1 = the reference's single-vector
    restart); maxiter is the budget of Krylov steps, precision_output the 16-bit basis type of the mixed
    mode ("half" or "bfloat16"), v0 and the returned vectors FP64."""
    ctx = context()
    op = operator(A, symmetric)
    modes = {"reference": L.MODE_REFERENCE, "mixed": L.MODE_MIXED, "fp64": L.MODE_FP64}
    kk = min(k, n)
    if mode == "mixed" and precision_output is None:
        precision_output = "half"
    o = options(mode=modes[mode], maxiter=maxiter, kdim=kdim or maxiter, nev=kk, tol=tol, use_generalized=1,
                generalized_tol=generalized_tol, select_tol=-1.0 if select_tol is None else select_tol, seed=seed,
                use_start_block=int(v0 is not None), orth=L.ORTH_HESSENBERG, restart_keep=restart_keep,
                **_prec_opts(precision_compute, precision_output, None, None, None, None))
    po = o.p_output if mode == "reference" else L.F64
    v0d = to_device_cm(v0, po) if v0 is not None else None
    X = empty_cm(n, kk, po)
    d = np.zeros(kk)
    res = np.zeros(kk)
    inf = L.ofrr_info()
    st = ctx.lib.ofrr_arnoldi_eig(ctx.h, C.byref(op.op), C.byref(o), v0d.data_ptr() if v0d is not None else None,
                                  X.data_ptr(), ld_of(X), _dp(d), _dp(res), C.byref(inf))
    if st not in (L.SUCCESS, L.ERR_SOLVER_MAX_ITERATIONS):
        L.check(st, "arnoldi_eig")
    return X, d, _info(st, inf, res)


def arnoldi_mgs_eig(A, n: int, k: int, precision_compute="double", precision_output=None, seed: int = 42,
                    maxiter: int = 5, kdim=None, reorth: bool = True, use_generalized: bool = False,
                    generalized_tol=0.0, select_tol=None, symmetric=None, v0=None, tol=0.0):
    """MATLAB/+src/+krylov/arnoldi_mgs_eig.m (orthogonal comparison path); returns (V, d, info)."""
    ctx = context()
    op = operator(A, symmetric)
    kk = min(k, n)
    o = options(mode=L.MODE_REFERENCE, maxiter=maxiter, kdim=kdim or maxiter, nev=kk, tol=tol,
                use_generalized=int(use_generalized), generalized_tol=generalized_tol,
                select_tol=-1.0 if select_tol is None else select_tol, seed=seed, use_start_block=int(v0 is not None),
                orth=L.ORTH_MGS, reorth=int(reorth), **_prec_opts(precision_compute, precision_output, None, None, None,
                                                                  None))
    po = o.p_output
    v0d = to_device_cm(v0, po) if v0 is not None else None
    X = empty_cm(n, kk, po)
    d = np.zeros(kk)
    res = np.zeros(kk)
    inf = L.ofrr_info()
    st = ctx.lib.ofrr_arnoldi_eig(ctx.h, C.byref(op.op), C.byref(o), v0d.data_ptr() if v0d is not None else None,
                                  X.data_ptr(), ld_of(X), _dp(d), _dp(res), C.byref(inf))
    if st not in (L.SUCCESS, L.ERR_SOLVER_MAX_ITERATIONS):
        L.check(st, "arnoldi_eig")
    return X, d, _info(st, inf, res)


def test_matrix_spectrum(s, m: int, n: int, seed: int = 0, symmetric: bool = False, reflectors: int = 3):
    """Dense FP64 device matrix (column-major) with singular values (symmetric: eigenvalues) exactly s:
    Householder reflectors around [diag(s); 0] (ofrr_test_matrix_spectrum)."""
    ctx = context()
    s = np.ascontiguousarray(s, dtype=np.float64)
    A = empty_cm(m, n, L.F64)
    L.check(ctx.lib.ofrr_test_matrix_spectrum(ctx.h, int(symmetric), seed, m, n, reflectors, _dp(s), A.data_ptr(),
                                              ld_of(A)), "test_matrix_spectrum")
    return A


def debug_invariant_subspace(G, M, sigma: float, p: int) -> np.ndarray:
    """Basis (n x p) of the invariant subspace of the pencil (G, M) for eigenvalues with real part above
    sigma (ofrr_debug_invariant_subspace; the restart block of the nonsymmetric Krylov path)."""
    ctx = context()
    n = G.shape[0]
    Gd = to_device_cm(np.asarray(G, np.float64), L.F64)
    Md = to_device_cm(np.asarray(M, np.float64), L.F64)
    Y = empty_cm(n, p, L.F64)
    L.check(ctx.lib.ofrr_debug_invariant_subspace(ctx.h, n, Gd.data_ptr(), Md.data_ptr(), float(sigma), p,
                                                  Y.data_ptr()), "debug_invariant_subspace")
    return to_numpy(Y)


def batch_sym_eig(A_packed, ns, offsets, nev: int = 8, block: int = 16, tol: float = 1e-7, step_size: int = 6,
                  maxiter: int = 500, p_output: str = "bfloat16", seed: int = 42, return_latency: bool = False):
    """Batched dense symmetric eigensolves in one persistent launch (ofrr_batch_sym_eig).  A_packed: FP64
    device tensor holding every matrix column-major at its element offset.  Returns (X list of device
    n_i x nev FP64 tensors, evals (count x nev), resid (count x nev), iterations, statuses)."""
    import torch

    ctx = context()
    count = len(ns)
    ns = np.ascontiguousarray(ns, dtype=np.int64)
    offsets = np.ascontiguousarray(offsets, dtype=np.int64)
    xo = np.concatenate([[0], np.cumsum(ns * nev)[:-1]]).astype(np.int64)
    X = torch.empty(int((ns * nev).sum()), dtype=torch.float64, device=A_packed.device)
    ev = np.zeros((count, nev))
    res = np.zeros((count, nev))
    its = np.zeros(count, dtype=np.int32)
    sts = np.zeros(count, dtype=np.int32)
    o = options(mode=L.MODE_MIXED, nev=nev, block=block, tol=tol, step_size=step_size, maxiter=maxiter, seed=seed,
                p_output=p_output)
    lat = np.zeros(count)
    L.check(ctx.lib.ofrr_batch_sym_eig_timed(ctx.h, count, ns.ctypes.data, offsets.ctypes.data, A_packed.data_ptr(),
                                             C.byref(o), X.data_ptr(), xo.ctypes.data, _dp(ev), _dp(res), _ip(its),
                                             _ip(sts), _dp(lat)), "batch_sym_eig")
    Xs = [X[int(xo[i]):int(xo[i] + ns[i] * nev)].view(nev, int(ns[i])).t() for i in range(count)]
    if return_latency:
        return Xs, ev, res, its, sts, lat
    return Xs, ev, res, its, sts


def profile_krylov_step(A: "CsrMatrix", precision: str, i: int, reps: int = 20):
    """Mean time (us) and algorithmic HBM bytes of one fused Krylov step (column i, basis type
    `precision`) on the CSR operator A (ofrr_profile_krylov_step)."""
    ctx = context()
    s = A.struct()
    us, by = C.c_double(), C.c_double()
    L.check(ctx.lib.ofrr_profile_krylov_step(ctx.h, C.byref(s), _p(precision), i, reps, C.byref(us), C.byref(by)),
            "profile_krylov_step")
    return us.value, by.value


def residual_norms(A, X, lam, normA: float = -1.0, symmetric=None):
    ctx = context()
    op = operator(A, symmetric)
    Xd = X if is_cm(X) else to_device_cm(X, L.F64)
    k = Xd.shape[1]
    lam = np.ascontiguousarray(lam, np.float64)
    out = np.zeros(k)
    L.check(ctx.lib.ofrr_residual_norms(ctx.h, C.byref(op.op), dtype_of(Xd), k, Xd.data_ptr(), ld_of(Xd), _dp(lam),
                                        normA, _dp(out)), "residual_norms")
    return out


# ---- solve engine: batched solves and a serving queue -----------------------------------------
class Server:
    """Worker threads with one library context each; requests run concurrently on the GPU.

    ``submit_si_eig`` / ``submit_si_svd`` return a ticket; ``wait(ticket)`` returns
    (status, latency_ms) and the request's outputs (device tensors, host arrays).  The request's
    operator and outputs are kept alive by the server until the ticket is collected."""

    def __init__(self, workers: int = 4, hbm_budget_bytes: int = 0, device: Optional[int] = None):
        self.lib = L.load()
        torch.cuda.init()
        h = C.c_void_p()
        dev = torch.cuda.current_device() if device is None else device
        L.check(self.lib.ofrr_serve_create(C.byref(h), dev, workers, hbm_budget_bytes), "ofrr_serve_create")
        self.h = h
        self._live = {}

    def _submit(self, req, keep):
        t = C.c_uint64()
        L.check(self.lib.ofrr_serve_submit(self.h, C.byref(req), C.byref(t)), "ofrr_serve_submit")
        self._live[t.value] = (req, keep)
        return t.value

    def submit_si_eig(self, A, k: int, mode: str = "mixed", tol: float = 1e-8, nev: Optional[int] = None,
                      maxiter: int = 200, step_size: int = 4, p_output: str = "half", symmetric=None, seed: int = 42,
                      check_every: int = 1):
        op = operator(A, symmetric)
        modes = {"reference": L.MODE_REFERENCE, "mixed": L.MODE_MIXED, "fp64": L.MODE_FP64}
        o = options(mode=modes[mode], maxiter=maxiter, step_size=step_size, block=min(k, op.n), nev=nev or min(k, op.n),
                    tol=tol, seed=seed, check_every=check_every, p_output=p_output if mode == "mixed" else None)
        po = o.p_output if mode == "reference" else L.F64
        V = empty_cm(op.m, o.block, po)
        d = np.zeros(o.block)
        res = np.zeros(o.block)
        inf = L.ofrr_info()
        req = L.ofrr_request(kind=L.REQ_SI_EIG, A=op.op, opt=o, V=V.data_ptr(), ldv=ld_of(V), values=_dp(d),
                             resid=_dp(res), info=C.pointer(inf))
        return self._submit(req, (op, V, d, res, inf))

    def submit_si_svd(self, A, k: int, mode: str = "mixed", tol: float = 1e-8, nev: Optional[int] = None,
                      maxiter: int = 200, step_size: int = 4, p_output: str = "half", seed: int = 42,
                      check_every: int = 1, step_size_f64: int = 0):
        op = operator(A, False)
        modes = {"reference": L.MODE_REFERENCE, "mixed": L.MODE_MIXED, "fp64": L.MODE_FP64}
        b = min(k, op.m, op.n)
        o = options(mode=modes[mode], maxiter=maxiter, step_size=step_size, block=b, nev=nev or b, tol=tol, seed=seed,
                    check_every=check_every, p_output=p_output if mode == "mixed" else None,
                    step_size_f64=step_size_f64)
        po = o.p_output if mode == "reference" else L.F64
        U = empty_cm(op.m, b, po)
        V = empty_cm(op.n, b, po)
        sv = np.zeros(b)
        res = np.zeros(b)
        inf = L.ofrr_info()
        req = L.ofrr_request(kind=L.REQ_SI_SVD, A=op.op, opt=o, V=V.data_ptr(), ldv=ld_of(V), U=U.data_ptr(),
                             ldu=ld_of(U), values=_dp(sv), resid=_dp(res), info=C.pointer(inf))
        return self._submit(req, (op, U, V, sv, res, inf))

    def submit_arnoldi_eig(self, A, k: int, kdim: int = 64, mode: str = "mixed", tol: float = 1e-8,
                           maxiter: int = 100000, p_output: str = "half", symmetric=None, seed: int = 42,
                           restart_keep: int = 0):
        """Thick-restart Krylov eigensolve of a CSR operator (ofrr_arnoldi_eig) as a request."""
        op = operator(A, symmetric)
        modes = {"reference": L.MODE_REFERENCE, "mixed": L.MODE_MIXED, "fp64": L.MODE_FP64}
        o = options(mode=modes[mode], maxiter=maxiter, kdim=kdim, nev=min(k, op.n), tol=tol, seed=seed,
                    use_generalized=1, restart_keep=restart_keep, orth=L.ORTH_HESSENBERG,
                    p_output=p_output if mode == "mixed" else None)
        X = empty_cm(op.m, o.nev, L.F64)
        d = np.zeros(o.nev)
        res = np.zeros(o.nev)
        inf = L.ofrr_info()
        req = L.ofrr_request(kind=L.REQ_ARNOLDI_EIG, A=op.op, opt=o, V=X.data_ptr(), ldv=ld_of(X), values=_dp(d),
                             resid=_dp(res), info=C.pointer(inf))
        return self._submit(req, (op, X, d, res, inf))

    def poll(self, ticket: int):
        done, st = C.c_int(), C.c_int()
        L.check(self.lib.ofrr_serve_poll(self.h, ticket, C.byref(done), C.byref(st)), "ofrr_serve_poll")
        return bool(done.value), st.value

    def wait(self, ticket: int):
        """(status, latency_ms, outputs) with outputs the request's (operator, tensors..., values, resid, info)."""
        st, lat = C.c_int(), C.c_double()
        L.check(self.lib.ofrr_serve_wait(self.h, ticket, C.byref(st), C.byref(lat)), "ofrr_serve_wait")
        req, keep = self._live.pop(ticket)
        return st.value, lat.value, keep

    def stats(self) -> dict:
        r = L.ofrr_serve_report()
        L.check(self.lib.ofrr_serve_stats(self.h, C.byref(r)), "ofrr_serve_stats")
        return {k: getattr(r, k) for k, _ in r._fields_}

    def close(self):
        if getattr(self, "h", None):
            self.lib.ofrr_serve_destroy(self.h)
            self.h = None
            self._live.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def batch_si_eig(server: Server, As, k: int, mode: str = "mixed", tol: float = 1e-7, nev: Optional[int] = None,
                 maxiter: int = 200, step_size: int = 4, p_output: str = "bfloat16", symmetric=True):
    """Independent si_eig solves of every matrix in As with shared options (ofrr_batch_si_eig).
    Returns (list of V, list of values, statuses)."""
    ops = [operator(A, symmetric) for A in As]
    cnt = len(ops)
    modes = {"reference": L.MODE_REFERENCE, "mixed": L.MODE_MIXED, "fp64": L.MODE_FP64}
    b = min([k] + [o.n for o in ops])
    o = options(mode=modes[mode], maxiter=maxiter, step_size=step_size, block=b, nev=nev or b, tol=tol,
                p_output=p_output if mode == "mixed" else None)
    po = o.p_output if mode == "reference" else L.F64
    Vs = [empty_cm(op.m, b, po) for op in ops]
    vals = [np.zeros(b) for _ in ops]
    opsarr = (L.ofrr_operator * cnt)(*[op.op for op in ops])
    Vp = (C.c_void_p * cnt)(*[V.data_ptr() for V in Vs])
    ldv = (C.c_int64 * cnt)(*[ld_of(V) for V in Vs])
    evp = (L._DP * cnt)(*[_dp(v) for v in vals])
    infos = (L.ofrr_info * cnt)()
    sts = np.zeros(cnt, dtype=np.int32)
    st = server.lib.ofrr_batch_si_eig(server.h, cnt, opsarr, C.byref(o), Vp, ldv, evp, None, infos, _ip(sts))
    L.check(st, "ofrr_batch_si_eig")
    return Vs, vals, sts


# ---- autotuner -------------------------------------------------------------------------------
def autotune_gemm16(M: int, N: int, K: int, precision: str = "half", reps: int = 5) -> dict:
    """Tile plan (BN, K split) of the 16-bit tcgen05 product C (M x N) = A' B for this shape, chosen by
    timing every candidate (ofrr_autotune_gemm16); later products of the shape use it."""
    ctx = context()
    bn, sp = np.zeros(1, np.int32), np.zeros(1, np.int32)
    us = np.zeros(1)
    L.check(ctx.lib.ofrr_autotune_gemm16(ctx.h, _p(precision), M, N, K, reps, _ip(bn), _ip(sp), _dp(us)),
            "autotune_gemm16")
    return {"M": M, "N": N, "K": K, "BN": int(bn[0]), "splits": int(sp[0]), "us": float(us[0])}


def gemm_e4m3(A, B):
    """A' B through E4M3 copies (per-column power-of-two scales) on the tensor cores; A (K x M), B (K x N)
    FP32 (ofrr_gemm_e4m3).  Returns the FP32 M x N device result."""
    ctx = context()
    Ad = A if is_cm(A) else to_device_cm(A, L.F32)
    Bd = B if is_cm(B) else to_device_cm(B, L.F32)
    K, M = Ad.shape
    N = Bd.shape[1]
    Cd = empty_cm(M, N, L.F32)
    L.check(ctx.lib.ofrr_gemm_e4m3(ctx.h, M, N, K, Ad.data_ptr(), ld_of(Ad), Bd.data_ptr(), ld_of(Bd), Cd.data_ptr(),
                                   ld_of(Cd)), "gemm_e4m3")
    return Cd


def gemm16_plan(M: int, N: int, K: int, precision: str = "half") -> dict:
    bn, sp, tu = np.zeros(1, np.int32), np.zeros(1, np.int32), np.zeros(1, np.int32)
    L.check(L.load().ofrr_gemm16_plan(_p(precision), M, N, K, _ip(bn), _ip(sp), _ip(tu)), "gemm16_plan")
    return {"BN": int(bn[0]), "splits": int(sp[0]), "tuned": bool(tu[0])}


def autotune_svd(A, m: int, n: int, nev: int, tol: float, mode: str = "mixed", blocks=(64, 96, 128),
                 steps=(4, 6, 8), reps: int = 2, min_block: int = 40, **kw):
    """Pick the block width and power-step count of subspace_iter_svd for this problem by timing
    each candidate solve (CUDA events on the library's stream, median of reps after one warm-up)
    and keeping the fastest one that converges; in mixed mode then the FP64 phase's power steps
    (step_size_f64, 0 = the same).  Returns {"block", "step_size", "step_size_f64", "ms", "iterations",
    "table"}; the table lists every candidate."""
    stream = torch.cuda.current_stream()
    table = []
    best = None
    tiles = []
    p16 = kw.get("precision_output", "half")
    for b in blocks:
        if b < max(min_block, nev) or b > min(m, n):
            continue
        if mode == "mixed":  # tile plans of the 16-bit products of this block width: A V, A' U, the Grams
            for shp in ((m, b, n), (n, b, m), (b, b, m), (b, b, n)):
                tiles.append(autotune_gemm16(*shp, precision=p16))
        for st in steps:
            args = dict(maxiter=kw.get("maxiter", 80), step_size=st, mode=mode, tol=tol, nev=nev,
                        check_every=kw.get("check_every", 1), generalized_tol=kw.get("generalized_tol", 0.0))
            U, s, V, info = subspace_iter_svd(A, m, n, b, kw.get("precision_compute", "single"),
                                              kw.get("precision_output", "half"), **args)
            ts = []
            for _ in range(reps):
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                U, s, V, info = subspace_iter_svd(A, m, n, b, kw.get("precision_compute", "single"),
                                                  kw.get("precision_output", "half"), **args)
                e1.record(stream)
                torch.cuda.synchronize()
                ts.append(e0.elapsed_time(e1))
            ms = float(np.median(ts))
            ok = info.status == 0 and info.max_residual <= tol
            table.append({"block": b, "step_size": st, "ms": ms, "iterations": info.iterations, "converged": ok})
            if ok and (best is None or ms < best["ms"]):
                best = {"block": b, "step_size": st, "ms": ms, "iterations": info.iterations}
    if best is None:
        raise RuntimeError("autotune_svd: no candidate converged")
    best["step_size_f64"] = 0
    if mode == "mixed":
        # the FP64 phase's own power steps (its iterations start from 16-bit-accurate vectors and each
        # carries a basis, a Rayleigh-Ritz and a certified check): step_size x 1, 1.5 and 2
        b, st = best["block"], best["step_size"]
        for s64 in sorted({st + st // 2, 2 * st} - {st}):
            args = dict(maxiter=kw.get("maxiter", 80), step_size=st, step_size_f64=s64, mode=mode, tol=tol, nev=nev,
                        check_every=kw.get("check_every", 1), generalized_tol=kw.get("generalized_tol", 0.0))
            subspace_iter_svd(A, m, n, b, kw.get("precision_compute", "single"), kw.get("precision_output", "half"),
                              **args)
            ts = []
            for _ in range(reps):
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                U, s, V, info = subspace_iter_svd(A, m, n, b, kw.get("precision_compute", "single"),
                                                  kw.get("precision_output", "half"), **args)
                e1.record(stream)
                torch.cuda.synchronize()
                ts.append(e0.elapsed_time(e1))
            ms = float(np.median(ts))
            ok = info.status == 0 and info.max_residual <= tol
            table.append({"block": b, "step_size": st, "step_size_f64": s64, "ms": ms, "iterations": info.iterations,
                          "converged": ok})
            if ok and ms < best["ms"]:
                best.update({"step_size_f64": s64, "ms": ms, "iterations": info.iterations})
    best["table"] = table
    best["tiles"] = tiles
    return best
