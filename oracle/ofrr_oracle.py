"""CPU oracle for the orthogonalization-free projection eigen/SVD path.

TEST INFRASTRUCTURE ONLY.  This module is the checker: only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference``
legs of ``bench.py`` may import it.  The product path (the CUDA library
``libofrr_gb300.so`` and its Python mirror) never calls into it.

It restates, in NumPy/SciPy, the reference's MATLAB algorithms (the reference's
C++ solver bodies are empty stubs, so the MATLAB code is the behavioural
definition of the path).  Every function cites the MATLAB file:line it follows.
Precision semantics follow the MATLAB code exactly: every ``precision_x(...)``
cast in the MATLAB source is a ``_cast(..., 'x')`` here, at the same place, so
that element-wise operations round identically (float16 storage, float32
compute, ...).

Deviations, each deliberate and mirrored by the CUDA path:
  * Start blocks come from the project's counter-based Gaussian generator
    (``randn_block``) instead of MATLAB's ``rng(seed); randn``, which cannot be
    reproduced outside MATLAB.  Callers may pass an explicit start block.
  * Rayleigh-Ritz returns Ritz pairs sorted by descending real part (MATLAB's
    ``eig`` order is solver-dependent); callers in the reference sort anyway
    (``arnoldi_hess_eig.m:98``, ``+tests/+test2/test.m``).
  * For an operator flagged symmetric, the projected matrix V'AV is
    symmetrised before the (generalized) symmetric eigensolve.

Pinned against the reference's own known answers in ``tests/test_oracle.py``:
SYEV / SYGV eigenvalues (``CPP/tests/mvops_test.cpp:2292-2370``,
``:2450-2530``), the 1-based planted ``iamax`` (``mvops_test.cpp:774-796``),
``dot == 55`` (``mvops_test.cpp:28-98``), Hessenberg A = QR and the duplicated-
column skip pattern {3,4,5} (``CPP/tests/hessenberg_test.cpp:30-92``), plus the
analytic spectrum of the 2D Dirichlet Laplacian.
"""
from __future__ import annotations

import math
from typing import Callable, Optional

import numpy as np
import scipy.linalg as sla
import scipy.sparse as sp

# --------------------------------------------------------------------------------------
# precision helpers (MATLAB +src/+utils/parse_precision.m, +src/+utils/eps.m)
# --------------------------------------------------------------------------------------
_DT = {"double": np.float64, "single": np.float32, "half": np.float16}


def _dt(p: str):
    return _DT[p]


def _cast(x, p: str):
    """MATLAB ``precision(x)`` cast (round-to-nearest-even, like IEEE conversions)."""
    return np.asarray(x).astype(_DT[p], copy=False)


def eps(p: str) -> float:
    """Machine epsilon per ``+src/+utils/eps.m:17-29`` (half is 2^-10)."""
    return {"double": 2.0 ** -52, "single": 2.0 ** -23, "half": 2.0 ** -10}[p]


def generalized_tol_default(p_eig: str) -> float:
    """``+src/+rr/eig_rr.m:105-113`` defaults."""
    return {"double": 1e-10, "single": 1e-5}.get(p_eig, 1e-3)


# --------------------------------------------------------------------------------------
# project RNG: counter-based Gaussian (same definition as the CUDA library's generator)
# --------------------------------------------------------------------------------------
_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix64(x: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = x + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def randn_block(seed: int, n: int, k: int) -> np.ndarray:
    """n x k block of N(0,1) samples (column-major element counter).

    Element e = i + n*j uses two 64-bit hashes h1 = splitmix64(key + 2e),
    h2 = splitmix64(key + 2e + 1) with key = splitmix64(seed); u1 = (h1>>11 + 0.5)
    * 2^-53 in (0,1), u2 = (h2>>11) * 2^-53 in [0,1) and Box-Muller
    z = sqrt(-2 ln u1) cos(2 pi u2).  Stands in for MATLAB ``rng(seed); randn(n,k)``
    (``+src/+subspace/subspace_iter_eig.m:53-54``).
    """
    key = _splitmix64(np.array([seed], dtype=np.uint64))[0]
    e = np.arange(n * k, dtype=np.uint64)
    with np.errstate(over="ignore"):
        h1 = _splitmix64(key + np.uint64(2) * e)
        h2 = _splitmix64(key + np.uint64(2) * e + np.uint64(1))
    u1 = ((h1 >> np.uint64(11)).astype(np.float64) + 0.5) * (2.0 ** -53)
    u2 = (h2 >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)
    z = np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * math.pi * u2)
    return z.reshape(k, n).T.copy()  # column-major counter -> (n, k)


# --------------------------------------------------------------------------------------
# level-1/2/3 ops (MATLAB +src/+mvops)
# --------------------------------------------------------------------------------------
def iamax(x) -> tuple[int, float]:
    """1-based index of the first max |x| and the signed value there.

    Mirrors ``CPP/linalg/blas/mvops.cu:607-876`` (strict ``>`` keeps the lowest
    index on ties) and MATLAB ``max`` (first occurrence, NaN ignored).
    """
    a = np.abs(np.asarray(x))
    if a.size == 0:
        return 0, 0.0
    if np.all(np.isnan(a)):
        return 1, float(np.asarray(x)[0])
    k = int(np.nanargmax(a))
    return k + 1, float(np.asarray(x)[k])


def _argmax_abs(v) -> int:
    a = np.abs(v)
    if np.all(np.isnan(a)):
        return 0
    return int(np.nanargmax(a))


def dot(x, y, pc: str = "double", po: str = "double"):
    """``+src/+mvops/dot.m:26-41`` (compute in pc, cast to po)."""
    return _cast(np.dot(_cast(x, pc), _cast(y, pc)), po)


def norm2(x, pc: str = "double", po: str = "double"):
    """``+src/+mvops/norm2.m:24-34``."""
    xc = _cast(x, pc)
    return _cast(np.sqrt(np.dot(xc, xc)), po)


def gemv(A, trans: str, x, pc: str, po: str):
    """``+src/+mvops/gemv.m:27-65``; half compute accumulates column by column."""
    A = _cast(A, pc)
    x = _cast(x, pc)
    if pc == "half":
        if trans == "N":
            y = A[:, 0] * x[0]
            for i in range(1, A.shape[1]):
                y = (y + A[:, i] * x[i]).astype(np.float16)
        else:
            y = A[0, :] * x[0]
            for i in range(1, A.shape[0]):
                y = (y + A[i, :] * x[i]).astype(np.float16)
    else:
        y = A @ x if trans == "N" else A.T @ x
    return _cast(y, po)


def gemm(A, trans: str, B, pc: str, po: str):
    """``+src/+mvops/gemm.m:27-59`` (C = op(A) B computed in pc, stored in po)."""
    A = _cast(A, pc)
    B = _cast(B, pc)
    if pc == "half":
        cols = [gemv(A, trans, B[:, i], "half", "half") for i in range(B.shape[1])]
        C = np.stack(cols, axis=1) if cols else np.zeros((A.shape[0 if trans == "N" else 1], 0), np.float16)
    else:
        C = A @ B if trans == "N" else A.T @ B
    return _cast(C, po)


def scalecols(U, pc: str, po: str, return_pivots: bool = False):
    """``+src/+mvops/scalecols.m:21-34``.

    Each column j: k = argmax |U(:,j)| (first occurrence), t = pc(U(k,j)); if t != 0,
    U(:,j) = po(pc(U(:,j)) / t).  Returns pivots (0-based) when asked.
    """
    U = np.array(_cast(U, po), copy=True)
    piv = np.zeros(U.shape[1], dtype=np.int64)
    for j in range(U.shape[1]):
        k = _argmax_abs(U[:, j])
        piv[j] = k
        t = _cast(U[k, j], pc)
        if t != 0.0:
            U[:, j] = _cast(_cast(U[:, j], pc) / t, po)
    return (U, piv) if return_pivots else U


# --------------------------------------------------------------------------------------
# CSR (MATLAB +src/+csr)
# --------------------------------------------------------------------------------------
def sparse2csr(A) -> dict:
    """``+src/+csr/sparse2csr.m:21-50``: CSR with FP64/FP32/FP16 value copies (0-based here)."""
    A = sp.csr_matrix(A, dtype=np.float64)
    A.sort_indices()
    with np.errstate(over="ignore"):  # half() of a value beyond the FP16 range is +-inf, as in MATLAB
        a_half = A.data.astype(np.float16)
    return {
        "nrows": A.shape[0],
        "ncols": A.shape[1],
        "indptr": A.indptr.astype(np.int32),
        "indices": A.indices.astype(np.int32),
        "a_double": A.data.astype(np.float64),
        "a_single": A.data.astype(np.float32),
        "a_half": a_half,
    }


def rand_uniform(seed: int, count: int) -> np.ndarray:
    """The library's uniform draws u(e) = (splitmix64(splitmix64(seed) + e) >> 11) 2^-53, e = 0..count-1
    (stands in for the reference's std / MATLAB ``rand``, which cannot be reproduced)."""
    key = _splitmix64(np.array([seed], dtype=np.uint64))[0]
    with np.errstate(over="ignore"):
        h = _splitmix64(key + np.arange(count, dtype=np.uint64))
    return (h >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)


def rand_points(seed: int, n: int, d: int, type: int = 0) -> np.ndarray:
    """``+src/+kernel/generate_pts.m`` (types 20, 21, 22, 23, 30, 31, 32) and the uniform box of
    ``CPP/testproblems/gaussian_kernel.hpp:36-40`` (type 0); draw j of a point i is u(i + n j)."""
    u = rand_uniform(seed, max(d, 3) * n).reshape(max(d, 3), n)
    if type in (0, 20, 30):
        return (n ** (1.0 / d)) * u[:d].T
    if type in (21, 22):
        theta = 2 * math.pi * u[0]
        r = (n / math.pi) ** 0.5 * np.sqrt(u[1]) if type == 21 else n / 2 / math.pi
        return np.stack([r * np.sin(theta), r * np.cos(theta)], axis=1)
    if type == 23:
        nx = int(round(math.sqrt(n)))
        i = np.arange(n)
        return np.stack([i % nx + 1, i // nx + 1], axis=1).astype(np.float64)
    el = np.arcsin(2.0 * u[0] - 1.0)
    az = 2 * math.pi * u[1]
    r = (3 * n / 4 / math.pi) ** (1.0 / 3) * np.cbrt(u[2]) if type == 31 else (n / 4 / math.pi) ** 0.5
    rc = r * np.cos(el)
    return np.stack([rc * np.cos(az), rc * np.sin(az), r * np.sin(el)], axis=1)


def generate_gaussian_kernel(f: float, l: float, s: float, X: np.ndarray) -> np.ndarray:
    """``CPP/testproblems/gaussian_kernel.hpp:14-77`` on given points: diagonal f^2 (1 + s^2), off the
    diagonal f^2 exp(-|x_i - x_j|^2 / (2 l^2)) with the squared distance summed in coordinate order,
    0 where the exponent is below -700."""
    if l <= 0 or s < 0:
        raise ValueError("invalid parameters (gaussian_kernel.hpp:18-29)")
    n, d = X.shape
    dist = np.zeros((n, n))
    for k in range(d):
        diff = X[:, k][:, None] - X[:, k][None, :]
        dist = dist + diff * diff
    arg = -dist / (2.0 * l * l)
    K = np.where(arg < -700.0, 0.0, np.exp(arg)) * (f * f)
    np.fill_diagonal(K, (1.0 + s * s) * (f * f))
    return K


def gaussian(X, Y, l: float, f: float, s: float) -> np.ndarray:
    """``+src/+kernel/gaussian.m:21-27``."""
    XY = X @ Y.T
    D2 = (-2 * XY + np.sum(X ** 2, 1)[:, None]) + np.sum(Y ** 2, 1)[None, :]
    return f ** 2 * np.exp(-D2 / (2 * l ** 2)) + s ** 2 * np.eye(X.shape[0], Y.shape[0])


def read_csr_matrix(prefix: str) -> dict:
    """``CPP/io/matrix_reader.cpp:8-45`` (MatrixReader::read_csr_matrix): ``<prefix>_row_ptr.bin``
    (int32), ``_col_ind.bin`` (int32, 0-based), ``_values.bin`` (float64), counts from the file sizes,
    ``cols`` = largest column index + 1 (``:40-43``).  Raises ``RuntimeError`` where the reference
    throws (a missing or empty file, ``:15-17``, ``:27-29``, ``:34-36``)."""
    out = {}
    for key, suffix, dt in (("indptr", "_row_ptr.bin", np.int32), ("indices", "_col_ind.bin", np.int32),
                            ("a_double", "_values.bin", np.float64)):
        try:
            a = np.fromfile(prefix + suffix, dtype=dt)  # whole elements only (matrix_reader.cpp:63-66)
        except OSError as e:
            raise RuntimeError(f"Failed to read {prefix + suffix}") from e
        if a.size == 0:
            raise RuntimeError(f"Failed to read {prefix + suffix}")
        out[key] = a
    out["nrows"] = out["indptr"].size - 1
    out["ncols"] = int(out["indices"].max()) + 1
    return out


def read_singular_values(prefix: str) -> np.ndarray:
    """``CPP/io/matrix_reader.cpp:47-50``: ``<prefix>_singular_values.bin`` (float64), empty when the
    file cannot be opened (``:55-59``)."""
    try:
        return np.fromfile(prefix + "_singular_values.bin", dtype=np.float64)
    except OSError:
        return np.empty(0)


def _csr_values(Acsr: dict, pc: str):
    return {"double": Acsr["a_double"], "single": Acsr["a_single"], "half": Acsr["a_half"]}[pc]


def csrmv(Acsr: dict, trans: str, x, pc: str, po: str):
    """``+src/+csr/csrmv.m:27-78``: row-wise CSR product with the pc value copy."""
    x = _cast(x, pc)
    squeeze = x.ndim == 1
    if squeeze:
        x = x[:, None]
    aa = _csr_values(Acsr, pc)
    M = sp.csr_matrix((aa, Acsr["indices"], Acsr["indptr"]), shape=(Acsr["nrows"], Acsr["ncols"]))
    if pc == "half":
        # element products in half, row sums in half (sum(aa .* x)), csrmv.m:50-53
        ip, ix = Acsr["indptr"], Acsr["indices"]
        nout = Acsr["nrows"] if trans == "N" else Acsr["ncols"]
        y = np.zeros((nout, x.shape[1]), dtype=np.float16)
        if trans == "N":
            for i in range(Acsr["nrows"]):
                sl = slice(ip[i], ip[i + 1])
                prod = (aa[sl][:, None] * x[ix[sl], :]).astype(np.float16)
                acc = np.zeros(x.shape[1], np.float16)
                for r in prod:
                    acc = (acc + r).astype(np.float16)
                y[i, :] = acc
        else:
            for i in range(Acsr["nrows"]):
                sl = slice(ip[i], ip[i + 1])
                y[ix[sl], :] = (y[ix[sl], :] + (aa[sl][:, None] * x[i, :][None, :]).astype(np.float16)).astype(np.float16)
    else:
        y = (M @ x) if trans == "N" else (M.T @ x)
        y = _cast(y, pc)
    y = _cast(y, po)
    return y[:, 0] if squeeze else y


def matvec_auto(A, trans: str, x, pc: str, po: str):
    """Dispatch like the MATLAB ``matvec`` option: CSR struct -> csrmv, dense -> gemm."""
    if isinstance(A, dict):
        return csrmv(A, trans, x, pc, po)
    if x.ndim == 1:
        return gemv(A, trans, x, pc, po)
    return gemm(A, trans, x, pc, po)


# --------------------------------------------------------------------------------------
# oblique basis: Hessenberg process (MATLAB +src/+qr/hessenberg.m)
# --------------------------------------------------------------------------------------
def hessenberg(A, pc: str = "double", po: Optional[str] = None, select_tol: Optional[float] = None):
    """Left-looking pivoted elimination, ``+src/+qr/hessenberg.m:45-85``.

    For column i: v = A(:,i); for each earlier selected j: R(j,i) = v(perm(j)),
    v = po(pc(v) - pc(R(j,i)) * pc(Q(:,j))); k = argmax|v| (lowest index on ties);
    R(i,i) = v(k); if |R(i,i)| < select_tol the column is deselected (Q(:,i) = 0),
    otherwise Q(:,i) = po(pc(v) / pc(R(i,i))) and perm(i) = k.

    Returns (Q, R, select, perm) in the full three-output form (perm 0-based, -1 if
    the column was deselected).
    """
    po = po or pc
    A = _cast(A, po)
    m, n = A.shape
    assert m >= n, "A must be a tall-thin matrix"
    st = eps(po) if select_tol is None else float(_cast(select_tol, po))
    Q = np.zeros((m, n), dtype=_dt(po))
    R = np.zeros((n, n), dtype=_dt(po))
    perm = np.full(n, -1, dtype=np.int64)
    select = np.ones(n, dtype=bool)
    for i in range(n):
        v = A[:, i].copy()
        for j in range(i):
            if select[j]:
                R[j, i] = v[perm[j]]
                v = _cast(_cast(v, pc) - _cast(R[j, i], pc) * _cast(Q[:, j], pc), po)
        k = _argmax_abs(v)
        R[i, i] = v[k]
        if abs(float(R[i, i])) < st:
            select[i] = False
        else:
            v = _cast(_cast(v, pc) / _cast(R[i, i], pc), po)
            perm[i] = k
            Q[:, i] = v
    return Q, R, select, perm


def hessenberg_economic(A, pc="double", po=None, select_tol=None):
    """Two-output form ``[Q,R] = hessenberg(...)`` (``hessenberg.m:71-73``)."""
    Q, R, select, _ = hessenberg(A, pc, po, select_tol)
    return Q[:, select], R[select, :]


def _orth_gs(A, classical: bool, pc: str, po: Optional[str], select_tol, orth_tol, reorth_tol):
    """Shared body of ``+src/+qr/mgs.m:49-101`` (classical=False) and ``+src/+qr/cgs.m:49-110``
    (classical=True).  Column i: ``normv = norm2(v)``; below select_tol the column is dropped;
    projections against the selected earlier columns (MGS: dot then update per j; CGS: all dots,
    then the updates in j order); then, while ``t = norm2(v)`` is at least orth_tol and below
    reorth_tol * normv, one more projection pass accumulated into R; finally v / t, R(i,i) = t, or
    the column is dropped when t < select_tol."""
    po = po or pc
    A = _cast(A, po)
    m, n = A.shape
    assert m >= n, "A must be a tall-thin matrix"
    e = eps(po)
    stol = e if select_tol is None else float(_cast(select_tol, po))
    otol = e if orth_tol is None else float(_cast(orth_tol, po))
    rtol = float(1.0 / np.sqrt(2.0)) if reorth_tol is None else float(_cast(reorth_tol, po))
    Q = np.zeros((m, n), dtype=_dt(po))
    R = np.zeros((n, n), dtype=_dt(po))
    select = np.ones(n, dtype=bool)

    def project(v, rcol, accumulate):
        js = [j for j in range(i) if select[j]]
        if classical:
            r = {j: dot(v, Q[:, j], pc, po) for j in js}
        for j in js:
            rj = r[j] if classical else dot(v, Q[:, j], pc, po)
            v = _cast(_cast(v, pc) - _cast(rj, pc) * _cast(Q[:, j], pc), po)
            rcol[j] = _cast(_cast(rcol[j], pc) + _cast(rj, pc), po) if accumulate else rj
        return v

    for i in range(n):
        v = A[:, i].copy()
        normv = float(norm2(v, pc, po))
        if normv < stol:
            select[i] = False
            continue
        rcol = R[:, i]
        v = project(v, rcol, False)
        t = float(norm2(v, pc, po))
        while rtol >= 0 and (t >= otol and t < rtol * normv):
            normv = t
            v = project(v, rcol, True)
            t = float(norm2(v, pc, po))
        if t < stol:
            select[i] = False
        else:
            Q[:, i] = _cast(_cast(v, pc) / _cast(t, pc), po)
            R[i, i] = t
    return Q, R, select


def mgs(A, pc: str = "double", po: Optional[str] = None, select_tol: Optional[float] = None,
        orth_tol: Optional[float] = None, reorth_tol: Optional[float] = None, full: bool = False):
    """Orthogonal comparison basis, ``+src/+qr/mgs.m`` (the default ``function_orth`` of
    ``subspace_iter_eig.m:114-115``).  Returns ``(Q(:,select), R(select,:))`` as the two-output form
    (``mgs.m:103-105``), or ``(Q, R, select)`` with ``full``."""
    Q, R, select = _orth_gs(A, False, pc, po, select_tol, orth_tol, reorth_tol)
    return (Q, R, select) if full else (Q[:, select], R[select, :])


def cgs(A, pc: str = "double", po: Optional[str] = None, select_tol: Optional[float] = None,
        orth_tol: Optional[float] = None, reorth_tol: Optional[float] = None, full: bool = False):
    """Classical Gram-Schmidt with the same adaptive re-orthogonalisation, ``+src/+qr/cgs.m``."""
    Q, R, select = _orth_gs(A, True, pc, po, select_tol, orth_tol, reorth_tol)
    return (Q, R, select) if full else (Q[:, select], R[select, :])


# --------------------------------------------------------------------------------------
# small dense (generalized) eigen-solves in FP64 (stand-in for MATLAB eig / LAPACK)
# --------------------------------------------------------------------------------------
def syev(A):
    """Symmetric eigen-decomposition, ascending (LAPACK dsyev, ``mvops.cu:1601-1630``)."""
    w, V = np.linalg.eigh(np.asarray(A, dtype=np.float64))
    return w, V


def sygv(A, B):
    """Symmetric-definite generalized eigenproblem, ascending, B-orthonormal vectors
    (LAPACK dsygv itype 1, ``mvops.cu:1633-1664``)."""
    w, V = sla.eigh(np.asarray(A, np.float64), np.asarray(B, np.float64))
    return w, V


def _pencil_eig(G, M, symmetric: bool):
    """eig(G, M) (or eig(G) if M is None); pairs sorted by descending real part."""
    if symmetric:
        Gs = 0.5 * (G + G.T)
        if M is None:
            w, U = np.linalg.eigh(Gs)
        else:
            w, U = sla.eigh(Gs, 0.5 * (M + M.T))
    else:
        if M is None:
            w, U = np.linalg.eig(G)
        else:
            w, U = sla.eig(G, M)
        w = np.real(w)
        U = np.real(U)
    idx = np.argsort(-np.real(w), kind="stable")
    return np.real(w)[idx], U[:, idx]


# --------------------------------------------------------------------------------------
# Rayleigh-Ritz (MATLAB +src/+rr)
# --------------------------------------------------------------------------------------
def eig_rr(A, V, pmc: str = "double", pmo: Optional[str] = None, pAmc: Optional[str] = None,
           pAmo: Optional[str] = None, peig: str = "double", use_generalized: bool = False,
           generalized_tol: Optional[float] = None, symmetric: bool = True,
           matvec: Callable = matvec_auto):
    """``+src/+rr/eig_rr.m:46-57``.

    AV = pmc(matvec(A,'N',pAmc(V), pAmc, pAmo)); VAV = peig(gemm(V,'T',AV, pmc, pmo));
    generalized: VV = peig(gemm(V,'T',V, pmc, pmo)), eig(VAV, VV + tol*I); else eig(VAV);
    V = gemm(V,'N',U, pmc, pmo) cast back to V's precision.
    Returns (V, d) with d the Ritz values (descending real part).
    """
    pmo = pmo or pmc
    pAmc = pAmc or pmc
    pAmo = pAmo or pAmc
    gtol = generalized_tol_default(peig) if generalized_tol is None else generalized_tol
    pV = {np.dtype(np.float64): "double", np.dtype(np.float32): "single", np.dtype(np.float16): "half"}[V.dtype]
    AV = _cast(matvec(A, "N", _cast(V, pAmc), pAmc, pAmo), pmc)
    VAV = _cast(gemm(V, "T", AV, pmc, pmo), peig).astype(np.float64)
    if use_generalized:
        VV = _cast(gemm(V, "T", V, pmc, pmo), peig).astype(np.float64)
        d, U = _pencil_eig(VAV, VV + gtol * np.eye(V.shape[1]), symmetric)
    else:
        d, U = _pencil_eig(VAV, None, symmetric)
    Vn = gemm(V, "N", U, pmc, pmo)
    return _cast(Vn, pV), d


def svd_rr(A, U, V, pmc: str = "double", pmo: Optional[str] = None, pAmc: Optional[str] = None,
           pAmo: Optional[str] = None, peig: str = "double", use_generalized: bool = False,
           generalized_tol: Optional[float] = None, matvec: Callable = matvec_auto):
    """``+src/+rr/svd_rr.m:50-91``.

    Generalized form: eig([[0,B],[B',0]], blkdiag(U'U, V'V) + tol*I) with B = U'AV,
    sorted descending, top k = min(ku,kv) pairs; U = sqrt(2)*U*Z, V = sqrt(2)*V*W.
    Returns (U, s, V).
    """
    pmo = pmo or pmc
    pAmc = pAmc or pmc
    pAmo = pAmo or pAmc
    gtol = generalized_tol_default(peig) if generalized_tol is None else generalized_tol
    pV = {np.dtype(np.float64): "double", np.dtype(np.float32): "single", np.dtype(np.float16): "half"}[V.dtype]
    AV = _cast(matvec(A, "N", _cast(V, pAmc), pAmc, pAmo), pmc)
    UAV = _cast(gemm(U, "T", AV, pmc, pmo), peig).astype(np.float64)
    if use_generalized:
        UU = _cast(gemm(U, "T", U, pmc, pmo), peig).astype(np.float64)
        VV = _cast(gemm(V, "T", V, pmc, pmo), peig).astype(np.float64)
        ku, kv = UU.shape[0], VV.shape[0]
        k = min(ku, kv)
        Aext = np.block([[np.zeros((ku, ku)), UAV], [UAV.T, np.zeros((kv, kv))]])
        Mext = np.block([[UU, np.zeros((ku, kv))], [np.zeros((kv, ku)), VV]])
        d, X = _pencil_eig(Aext, Mext + gtol * np.eye(ku + kv), True)
        s = d[:k]
        Z = X[:ku, :k]
        W = X[ku:, :k]
    else:
        Z, s, Wt = np.linalg.svd(UAV)
        W = Wt.T
    Z = _cast(Z, pmo)
    W = _cast(W, pmo)
    r2 = _cast(np.sqrt(2.0), pmo) if use_generalized else _cast(1.0, pmo)
    Un = gemm(U, "N", Z, pmc, pmo)
    Un = _cast(_cast(r2 * Un, pmo), pV)
    Vn = gemm(V, "N", W, pmc, pmo)
    Vn = _cast(_cast(r2 * Vn, pmo), pV)
    return Un, np.asarray(s, dtype=np.float64), Vn


# --------------------------------------------------------------------------------------
# solvers (MATLAB +src/+subspace, +src/+krylov)
# --------------------------------------------------------------------------------------
def subspace_iter_eig(A, n: int, k: int, pc: str = "double", po: Optional[str] = None, seed: int = 42,
                      maxiter: int = 5, step_size: int = 1, orth: str = "hessenberg",
                      ph_c: Optional[str] = None, ph_o: Optional[str] = None,
                      prr_c: Optional[str] = None, prr_o: Optional[str] = None, peig: str = "double",
                      use_generalized: bool = True, generalized_tol: float = 0.0,
                      select_tol: Optional[float] = None, symmetric: bool = True,
                      V0: Optional[np.ndarray] = None, callback: Optional[Callable] = None):
    """``+src/+subspace/subspace_iter_eig.m:50-68`` with the orth/rr wrappers that the
    reference's experiments pass (``+tests/+test2/test.m:358-397``):
    orth = hessenberg(ph_c, ph_o), rr = eig_rr(prr_c, prr_o, A-matvec in (pc, po), peig,
    use_generalized, generalized_tol).
    """
    po = po or pc
    ph_c = ph_c or pc
    ph_o = ph_o or po
    prr_c = prr_c or pc
    prr_o = prr_o or po
    k = min(k, n)
    V = _cast(randn_block(seed, n, k) if V0 is None else V0, po)
    V = scalecols(V, pc, po)
    if not isinstance(A, dict):
        A = _cast(A, po)
    d = np.zeros(V.shape[1])
    for it in range(maxiter):
        for _ in range(step_size):
            V = matvec_auto(A, "N", V, pc, po)
            V = scalecols(V, pc, po)
        Q = _basis(V, orth, ph_c, ph_o, select_tol)
        V, d = eig_rr(A, Q, prr_c, prr_o, pc, po, peig, use_generalized, generalized_tol, symmetric)
        V = _cast(V, po)
        if callback is not None:
            callback(it, V, d)
    return V, d


def lu(A, pc: str = "double", po: Optional[str] = None, select_tol: Optional[float] = None, full: bool = False):
    """``+src/+qr/lu.m:47-94``: right-looking LU with partial pivoting on A_work (rows swapped in
    place; the pivot is the first maximum of |A_work(j:m, j)| in the current row order); a column whose
    maximum is below select_tol is dropped (its row j is consumed all the same and U(j, j:n) keeps the
    row).  Returns ``(L(rperm, select), U(select, :))`` as the two-output form, or
    ``(L, U, perm, select)`` (0-based perm) with ``full``."""
    po = po or pc
    A = _cast(A, po)
    m, n = A.shape
    assert m >= n, "A must be a tall-thin matrix"
    st = eps(po) if select_tol is None else float(_cast(select_tol, po))
    W = A.copy()
    L = np.zeros((m, n), dtype=_dt(po))
    U = np.zeros((n, n), dtype=_dt(po))
    perm = np.arange(m)
    select = np.ones(n, dtype=bool)
    for j in range(n):
        col = np.abs(W[j:, j].astype(np.float64))
        p = j + int(np.argmax(col))  # first maximum (MATLAB max)
        if float(col[p - j]) < st:
            select[j] = False
            U[j, j:] = W[j, j:]
            continue
        if p != j:
            W[[j, p], :] = W[[p, j], :]
            L[[j, p], :j] = L[[p, j], :j]
            perm[[j, p]] = perm[[p, j]]
        U[j, j:] = W[j, j:]
        L[j:, j] = _cast(_cast(W[j:, j], pc) / _cast(W[j, j], pc), po)
        # rows i > j, every one as lu.m's loop (one product, one difference, each rounded)
        W[j + 1:, j + 1:] = _cast(_cast(W[j + 1:, j + 1:], pc) - _cast(L[j + 1:, j], pc)[:, None]
                                  * _cast(W[j, j + 1:], pc)[None, :], po)
    if full:
        return L, U, perm, select
    rperm = np.empty(m, dtype=np.int64)
    rperm[perm] = np.arange(m)
    return L[rperm][:, select], U[select, :]


def _basis(V, orth: str, ph_c: str, ph_o: str, select_tol):
    """``function_orth`` of ``subspace_iter_eig.m:65``: hessenberg (the orthogonalization-free runs),
    mgs (the file's default, ``:114-115``) or cgs; the two-output (economic) form."""
    if orth == "hessenberg":
        return hessenberg_economic(V, ph_c, ph_o, select_tol)[0]
    if orth == "cgs":
        return cgs(V, ph_c, ph_o, select_tol)[0]
    if orth == "lu":
        return lu(V, ph_c, ph_o, select_tol)[0]
    return mgs(V, ph_c, ph_o, select_tol)[0]


def subspace_iter_svd(A, m: int, n: int, k: int, pc: str = "double", po: Optional[str] = None,
                      seed: int = 42, maxiter: int = 5, step_size: int = 1, orth: str = "hessenberg",
                      ph_c: Optional[str] = None, ph_o: Optional[str] = None,
                      prr_c: Optional[str] = None, prr_o: Optional[str] = None, peig: str = "double",
                      use_generalized: bool = True, generalized_tol: float = 0.0,
                      select_tol: Optional[float] = None, V0: Optional[np.ndarray] = None,
                      callback: Optional[Callable] = None):
    """``+src/+subspace/subspace_iter_svd.m:53-77`` with Hessenberg orth and svd_rr
    (``+tests/+test3``'s wrappers)."""
    po = po or pc
    ph_c = ph_c or pc
    ph_o = ph_o or po
    prr_c = prr_c or pc
    prr_o = prr_o or po
    k = min(k, n)
    V = _cast(randn_block(seed, n, k) if V0 is None else V0, po)
    V = scalecols(V, pc, po)
    if not isinstance(A, dict):
        A = _cast(A, po)
    U = None
    s = np.zeros(k)
    for it in range(maxiter):
        for _ in range(step_size):
            U = matvec_auto(A, "N", V, pc, po)
            U = scalecols(U, pc, po)
            V = matvec_auto(A, "T", U, pc, po)
            V = scalecols(V, pc, po)
        P = _basis(U, orth, ph_c, ph_o, select_tol)
        Q = _basis(V, orth, ph_c, ph_o, select_tol)
        U, s, V = svd_rr(A, P, Q, prr_c, prr_o, pc, po, peig, use_generalized, generalized_tol)
        U = _cast(U, po)
        V = _cast(V, po)
        if callback is not None:
            callback(it, U, s, V)
    return U, s, V


def arnoldi_hess_eig(A, n: int, k: int, pc: str = "double", po: Optional[str] = None, peig: str = "double",
                     seed: int = 42, maxiter: int = 5, kdim: Optional[int] = None,
                     select_tol: Optional[float] = None, generalized_tol: float = 0.0,
                     symmetric: bool = False, v0: Optional[np.ndarray] = None):
    """Hessenberg-process Krylov eigensolver, ``+src/+krylov/arnoldi_hess_eig.m:51-107``.

    Returns (V, d, info) with V the k Ritz vectors, d the k Ritz values (descending
    real part) and info = {'cycles', 'matvecs', 'perms'}.
    """
    po = po or pc
    kdim = maxiter if kdim is None else kdim
    st = eps(po) if select_tol is None else select_tol
    k = min(k, n)
    V = np.zeros((n, kdim + 1), dtype=_dt(po))
    V[:, 0] = _cast(randn_block(seed, n, 1)[:, 0] if v0 is None else v0, po)
    tits = 1
    d = np.zeros(0)
    info = {"cycles": 0, "matvecs": 0, "perms": []}
    Vout = V[:, :0]
    while tits < maxiter:
        perm = np.zeros(kdim + 1, dtype=np.int64)
        l = _argmax_abs(V[:, 0])
        perm[0] = l
        if abs(float(V[l, 0])) < st:
            break
        V[:, 0] = _cast(_cast(V[:, 0], pc) / _cast(V[l, 0], pc), po)
        ncols = kdim + 1
        for i in range(1, kdim + 1):
            V[:, i] = _cast(matvec_auto(A, "N", _cast(V[:, i - 1], pc), pc, pc), po)
            info["matvecs"] += 1
            for j in range(i):
                V[:, i] = _cast(_cast(V[:, i], pc) - _cast(V[perm[j], i], pc) * _cast(V[:, j], pc), po)
            l = _argmax_abs(V[:, i])
            perm[i] = l
            if abs(float(V[l, i])) < st:
                tits = maxiter
                ncols = i  # the invariant-subspace column and any stale tail are left out of RR
                break
            V[:, i] = _cast(_cast(V[:, i], pc) / _cast(V[l, i], pc), po)
            tits += 1
        info["perms"].append(perm.copy())
        info["cycles"] += 1
        Vb = V[:, :ncols]
        Vr, d = eig_rr(A, Vb, pc, po, pc, pc, peig, True, generalized_tol, symmetric)
        # Ritz pairs already sorted descending (real part)
        if tits < maxiter:
            V[:, 0] = Vr[:, 0]
        else:
            Vout = Vr[:, :k]
            d = d[:k]
    info["V_basis"] = V
    return Vout, d, info


def arnoldi_thick_eig(A, n: int, k: int, kdim: int, tol: float, keep: Optional[int] = None, maxsteps: int = 100000,
                      v0: Optional[np.ndarray] = None, seed: int = 42, symmetric: bool = False,
                      generalized_tol: float = 0.0, callback: Optional[Callable] = None):
    """Thick-restart Hessenberg-process Krylov eigensolver in FP64: the restatement of the library's
    production Krylov path (its FP64 mode), for parity tests.

    The Krylov steps follow ``+src/+krylov/arnoldi_hess_eig.m:73-87`` (A times the previous column,
    eliminations in MGS order with the coefficients read at the earlier pivot rows, pivot on the first
    largest entry, scale) and the Rayleigh-Ritz step its generalized form (``:89-95``, eig(V'AV, V'V)).
    The restart is new (``:99-106`` keeps the leading Ritz vector alone): a basis Y of the invariant
    subspace of the projected pencil for its leading eigenvalues (about ``keep`` of them -- by default k for
    a nonsymmetric operator and max(k + 4, 1.2 k) for a symmetric one -- cut at the widest gap of the real
    parts within keep-3 .. keep+4: the Ritz vectors for a symmetric operator, sorted real Schur vectors
    otherwise) and the Galerkin residual direction f = A v_last - V (V'V)^-1 V' A v_last;
    the next basis is the Hessenberg basis of [Y, f] (columns first scaled to a unit maximum,
    near-dependent ones dropped below 1e-12) continued by Krylov steps from f.  Stops when the k leading
    Ritz pairs have ||A x - l x|| / (max|l| ||x||) <= tol or after ``maxsteps`` Krylov steps.  Returns
    (X (n x k, unit columns), d (k), info) with info = {'cycles', 'steps', 'residuals'}.
    """
    k = min(k, n)
    if keep is None or keep <= 0:  # the library's default: k for a nonsymmetric operator, more for a symmetric one
        keep = min(max(k + 4, (k * 6 + 4) // 5) if symmetric else k, kdim - 2)
    keep = min(max(keep, k), kdim - 2)
    nb = kdim + 1
    W = (randn_block(seed, n, 1) if v0 is None else np.asarray(v0, dtype=np.float64).reshape(n, 1)).copy()
    info = {"cycles": 0, "steps": 0, "residuals": None}
    while True:
        W = scalecols(W, "double", "double")
        Q, R, sel, perm = hessenberg(W, "double", "double", select_tol=1e-12)
        cols = [Q[:, j].copy() for j in range(W.shape[1]) if sel[j]]
        piv = [int(perm[j]) for j in range(W.shape[1]) if sel[j]]
        stop = False
        while len(cols) < nb:
            w = matvec_auto(A, "N", cols[-1], "double", "double")
            info["steps"] += 1
            for q, pv in zip(cols, piv):
                w = w - w[pv] * q
            w[piv] = 0.0
            l = _argmax_abs(w)
            if w[l] == 0.0:
                stop = True
                break
            cols.append(w / w[l])
            piv.append(l)
        V = np.column_stack(cols)
        AV = np.column_stack([matvec_auto(A, "N", V[:, j], "double", "double") for j in range(V.shape[1])])
        G = V.T @ AV
        M = V.T @ V + generalized_tol * np.eye(V.shape[1])
        if symmetric:
            lam, Z = sla.eigh(0.5 * (G + G.T), M)
            idx = np.argsort(-lam, kind="stable")
            w_all, Z = lam[idx].astype(complex), Z[:, idx].astype(complex)
        else:
            w_all, Z = sla.eig(G, M)
            idx = np.argsort(-w_all.real, kind="stable")
            w_all, Z = w_all[idx], Z[:, idx]
        kk = min(k, V.shape[1])
        X = (V @ Z[:, :kk]).real
        lam = w_all[:kk].real
        AX = matvec_auto(A, "N", X, "double", "double")
        nrm = np.linalg.norm(X, axis=0)
        scale = max(np.max(np.abs(lam)), 1e-300)
        res = np.linalg.norm(AX - X * lam[None, :], axis=0) / (scale * nrm)
        info["cycles"] += 1
        info["residuals"] = res
        if callback is not None:
            callback(info["cycles"], lam, res)
        if np.max(res) <= tol or stop or info["steps"] >= maxsteps:
            return X / nrm[None, :], lam, info
        nc = V.shape[1]
        re = w_all.real
        pp, best = min(keep, nc - 1), -1.0
        for c in range(max(k, keep - 3), min(keep + 4, nc - 2) + 1):  # the widest gap near `keep`
            if re[c - 1] - re[c] > best:
                best, pp = re[c - 1] - re[c], c
        if best <= 0:
            pp = min(keep, nc - 1)
        if symmetric:
            Y = V @ Z[:, :pp].real
        else:
            # the invariant subspace of the eigenvalues with real part above sigma (sorted real Schur form;
            # the GPU path gets the same subspace from the matrix sign function)
            sigma = 0.5 * (re[pp - 1] + re[pp])
            Lc = np.linalg.cholesky(M)
            C = sla.solve_triangular(Lc, sla.solve_triangular(Lc, G.T, lower=True).T, lower=True)
            T, S, sdim = sla.schur(C, output="real", sort=lambda x, y: x > sigma)
            Y = V @ sla.solve_triangular(Lc.T, S[:, :sdim], lower=False)
        f = AV[:, -1] - V @ np.linalg.solve(M, G[:, -1])
        W = np.column_stack([Y, f])


def arnoldi_mgs_eig(A, n: int, k: int, pc: str = "double", po: Optional[str] = None, peig: str = "double",
                    seed: int = 42, maxiter: int = 5, kdim: Optional[int] = None, reorth: bool = True,
                    use_generalized: bool = False, generalized_tol: float = 0.0,
                    select_tol: Optional[float] = None, symmetric: bool = False,
                    v0: Optional[np.ndarray] = None):
    """Orthogonal Arnoldi (MGS + optional reorth), ``+src/+krylov/arnoldi_mgs_eig.m:54-113``."""
    po = po or pc
    kdim = maxiter if kdim is None else kdim
    st = eps(po) if select_tol is None else select_tol
    k = min(k, n)
    V = np.zeros((n, kdim + 1), dtype=_dt(po))
    V[:, 0] = _cast(randn_block(seed, n, 1)[:, 0] if v0 is None else v0, po)
    tits = 1
    d = np.zeros(0)
    Vout = V[:, :0]
    while tits < maxiter:
        t = norm2(V[:, 0], pc, po)
        if float(t) < st:
            break
        V[:, 0] = _cast(_cast(V[:, 0], pc) / _cast(t, pc), po)
        ncols = kdim + 1
        for i in range(1, kdim + 1):
            V[:, i] = _cast(matvec_auto(A, "N", _cast(V[:, i - 1], pc), pc, pc), po)
            for j in range(i):
                r = dot(V[:, i], V[:, j], pc, po)
                V[:, i] = _cast(_cast(V[:, i], pc) - _cast(r, pc) * _cast(V[:, j], pc), po)
                if reorth:
                    r = dot(V[:, i], V[:, j], pc, po)
                    V[:, i] = _cast(_cast(V[:, i], pc) - _cast(r, pc) * _cast(V[:, j], pc), po)
            t = norm2(V[:, i], pc, po)
            if float(t) < st:
                tits = maxiter
                ncols = i
                break
            V[:, i] = _cast(_cast(V[:, i], pc) / _cast(t, pc), po)
            tits += 1
        Vb = V[:, :ncols]
        Vr, d = eig_rr(A, Vb, pc, po, pc, pc, peig, use_generalized, generalized_tol, symmetric)
        if tits < maxiter:
            V[:, 0] = Vr[:, 0]
        else:
            Vout = Vr[:, :k]
            d = d[:k]
    return Vout, d


# --------------------------------------------------------------------------------------
# residuals (MATLAB +tests/+test4/test.m:340-350) and FP64 truth
# --------------------------------------------------------------------------------------
def residual_norms(A, X, lam, normA: Optional[float] = None):
    """Per pair: ||A x - lam x||_2 / (normA * ||x||_2) in FP64 (normA defaults to max|lam|).

    The reference's own form (``+tests/+test4/test.m:340-350``) is ||Av - lam v|| / lam with an
    unnormalised v; ``residual_norms_reference`` returns that one.
    """
    X = np.asarray(X, dtype=np.float64)
    lam = np.asarray(lam, dtype=np.float64)
    AX = matvec_auto(A if isinstance(A, dict) else np.asarray(A, np.float64), "N", X, "double", "double")
    R = AX - X * lam[None, :]
    nA = float(np.max(np.abs(lam))) if normA is None else normA
    return np.linalg.norm(R, axis=0) / (nA * np.linalg.norm(X, axis=0))


def residual_norms_reference(A, X, lam):
    X = np.asarray(X, dtype=np.float64)
    AX = matvec_auto(A if isinstance(A, dict) else np.asarray(A, np.float64), "N", X, "double", "double")
    return np.linalg.norm(AX - X * lam[None, :], axis=0) / np.asarray(lam, np.float64)


def svd_residual_norms(A, U, s, V, normA: Optional[float] = None):
    """max(||A v - s u||, ||A' u - s v||) / normA per triplet, with u, v normalised."""
    A = np.asarray(A, np.float64)
    U = np.asarray(U, np.float64)
    V = np.asarray(V, np.float64)
    U = U / np.linalg.norm(U, axis=0)
    V = V / np.linalg.norm(V, axis=0)
    s = np.asarray(s, np.float64)
    nA = float(np.max(np.abs(s))) if normA is None else normA
    r1 = np.linalg.norm(A @ V - U * s, axis=0)
    r2 = np.linalg.norm(A.T @ U - V * s, axis=0)
    return np.maximum(r1, r2) / nA


# --------------------------------------------------------------------------------------
# test problems (the synthetic inputs of the benchmark configurations)
# --------------------------------------------------------------------------------------
def laplacian_2d(nx: int, ny: Optional[int] = None):
    """5-point Dirichlet Laplacian on an nx x ny interior grid (stencil 4, -1 x 4), CSR."""
    ny = nx if ny is None else ny
    Tx = sp.diags([-np.ones(nx - 1), 2 * np.ones(nx), -np.ones(nx - 1)], [-1, 0, 1])
    Ty = sp.diags([-np.ones(ny - 1), 2 * np.ones(ny), -np.ones(ny - 1)], [-1, 0, 1])
    A = sp.kron(sp.identity(ny), Tx) + sp.kron(Ty, sp.identity(nx))
    return sp.csr_matrix(A)


def laplacian_2d_eigs(nx: int, ny: Optional[int] = None):
    """Analytic spectrum 4 - 2cos(i pi/(nx+1)) - 2cos(j pi/(ny+1)), descending."""
    ny = nx if ny is None else ny
    i = np.arange(1, nx + 1)
    j = np.arange(1, ny + 1)
    lam = (2 - 2 * np.cos(i * np.pi / (nx + 1)))[:, None] + (2 - 2 * np.cos(j * np.pi / (ny + 1)))[None, :]
    return np.sort(lam.ravel())[::-1]


def laplacian_3d(nx: int):
    T = sp.diags([-np.ones(nx - 1), 2 * np.ones(nx), -np.ones(nx - 1)], [-1, 0, 1])
    I = sp.identity(nx)
    A = sp.kron(sp.kron(I, I), T) + sp.kron(sp.kron(I, T), I) + sp.kron(sp.kron(T, I), I)
    return sp.csr_matrix(A)


def convdiff_3d(N: int, Pe: float = 10.0, w=(1.0, 0.5, 0.25)):
    """-Lap u + Pe w.grad u on the unit cube, N^3 interior points, central differences.

    Row stencil per dimension d (h = 1/(N+1)): diagonal 2/h^2, neighbours
    -1/h^2 -/+ Pe w_d/(2h) (minus side gets +, plus side gets -).  Sign convention:
    operator = -Lap + Pe w.grad.  Eigenvalues are real when Pe w_d h/2 < 1.
    """
    h = 1.0 / (N + 1)
    mats = []
    for wd in w:
        c = Pe * wd / (2 * h)
        lo = (-1.0 / h ** 2 - c) * np.ones(N - 1)
        up = (-1.0 / h ** 2 + c) * np.ones(N - 1)
        mats.append(sp.diags([lo, (2.0 / h ** 2) * np.ones(N), up], [-1, 0, 1]))
    I = sp.identity(N)
    A = sp.kron(sp.kron(I, I), mats[0]) + sp.kron(sp.kron(I, mats[1]), I) + sp.kron(sp.kron(mats[2], I), I)
    return sp.csr_matrix(A)


def convdiff_3d_eigs(N: int, Pe: float = 10.0, w=(1.0, 0.5, 0.25)):
    """Analytic spectrum: sum_d [2/h^2 + 2 sqrt(a_d c_d) cos(k_d pi/(N+1))], descending."""
    h = 1.0 / (N + 1)
    k = np.arange(1, N + 1)
    parts = []
    for wd in w:
        c = Pe * wd / (2 * h)
        ac = (1.0 / h ** 2) ** 2 - c ** 2
        parts.append(2.0 / h ** 2 - 2.0 * np.sqrt(ac) * np.cos(k * np.pi / (N + 1)))
    lam = parts[0][:, None, None] + parts[1][None, :, None] + parts[2][None, None, :]
    return np.sort(lam.ravel())[::-1]


def haar(n: int, k: int, seed: int):
    """n x k with orthonormal columns: Q of QR of a seeded Gaussian block, sign-fixed."""
    G = randn_block(seed, n, k)
    Q, R = np.linalg.qr(G)
    return Q * np.sign(np.diag(R))[None, :]


def dense_svd_problem(m: int, n: int, seed: int = 42, smin: float = 1e-6):
    """A = U diag(s) V' with Haar U, V and geometric s from 1 to smin."""
    U = haar(m, n, seed)
    V = haar(n, n, seed + 1)
    s = smin ** (np.arange(n) / (n - 1))
    return (U * s[None, :]) @ V.T, U, s, V


def dense_sym_problem(n: int, seed: int, lam_lo: float = 1e-4, lam_hi: float = 1.0):
    """Q diag(lam) Q' with Haar Q and lam log-uniform in [lam_lo, lam_hi]."""
    Q = haar(n, n, seed)
    u = (randn_block(seed + 7, n, 1)[:, 0])
    # log-uniform via the normal CDF of the project generator
    from scipy.special import ndtr
    lam = np.exp(np.log(lam_lo) + (np.log(lam_hi) - np.log(lam_lo)) * ndtr(u))
    A = (Q * lam[None, :]) @ Q.T
    return 0.5 * (A + A.T), np.sort(lam)[::-1]
