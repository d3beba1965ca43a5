"""ctypes binding of libofrr_gb300.so (the C ABI declared in include/ofrr.h).

The library is the product; this module only declares its entry points.  Importing it on a
machine where the library was not built raises immediately: there is no fallback path.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libofrr_gb300.so"

# ---- enums (include/ofrr.h) -----------------------------------------------------------------
F64, F32, F16, BF16 = 0, 1, 2, 3
OP_DENSE, OP_CSR = 0, 1
MODE_REFERENCE, MODE_MIXED, MODE_FP64 = 0, 1, 2
ORTH_HESSENBERG, ORTH_MGS, ORTH_CGS, ORTH_LU = 0, 1, 2, 3

SUCCESS = 0
ERR_SOLVER_MAX_ITERATIONS = 4001


class ofrr_csr(C.Structure):
    _fields_ = [
        ("nrows", C.c_int64), ("ncols", C.c_int64), ("nnz", C.c_int64),
        ("indptr", C.c_void_p), ("indices", C.c_void_p),
        ("a_double", C.c_void_p), ("a_single", C.c_void_p), ("a_half", C.c_void_p),
    ]


class ofrr_operator(C.Structure):
    _fields_ = [
        ("kind", C.c_int), ("nrows", C.c_int64), ("ncols", C.c_int64), ("symmetric", C.c_int),
        ("dtype", C.c_int), ("data", C.c_void_p), ("ld", C.c_int64),
        ("csr", ofrr_csr),
    ]


class ofrr_options(C.Structure):
    _fields_ = [
        ("mode", C.c_int), ("maxiter", C.c_int), ("step_size", C.c_int), ("block", C.c_int),
        ("nev", C.c_int), ("kdim", C.c_int), ("tol", C.c_double), ("use_generalized", C.c_int),
        ("generalized_tol", C.c_double), ("select_tol", C.c_double), ("seed", C.c_uint64),
        ("use_start_block", C.c_int), ("orth", C.c_int), ("reorth", C.c_int),
        ("p_compute", C.c_int), ("p_output", C.c_int), ("p_hess_compute", C.c_int),
        ("p_hess_output", C.c_int), ("p_rr_compute", C.c_int), ("p_rr_output", C.c_int),
        ("check_every", C.c_int), ("restart_keep", C.c_int), ("power_fp8", C.c_int), ("step_size_f64", C.c_int),
    ]


class ofrr_info(C.Structure):
    _fields_ = [
        ("iterations", C.c_int), ("matvecs", C.c_int), ("converged", C.c_int), ("basis_width", C.c_int),
        ("max_residual", C.c_double), ("escalations", C.c_int), ("status_detail", C.c_int),
    ]


# name -> (restype, argtypes)
class ofrr_request(C.Structure):
    _fields_ = [("kind", C.c_int), ("A", ofrr_operator), ("opt", ofrr_options), ("V", C.c_void_p), ("ldv", C.c_int64),
                ("U", C.c_void_p), ("ldu", C.c_int64), ("v0", C.c_void_p), ("values", C.POINTER(C.c_double)),
                ("resid", C.POINTER(C.c_double)), ("info", C.POINTER(ofrr_info))]


class ofrr_serve_report(C.Structure):
    _fields_ = [("completed", C.c_uint64), ("failed", C.c_uint64), ("queued", C.c_uint64),
                ("charged_bytes", C.c_size_t), ("budget_bytes", C.c_size_t), ("wall_ms", C.c_double),
                ("busy_ms", C.c_double), ("p50_ms", C.c_double), ("p99_ms", C.c_double)]


REQ_SI_EIG, REQ_SI_SVD, REQ_ARNOLDI_EIG = 0, 1, 2

_P = C.c_void_p
_I64 = C.c_int64
_D = C.c_double
_DP = C.POINTER(C.c_double)
_IP = C.POINTER(C.c_int)
SIGNATURES = {
    "ofrr_ctx_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int, _P]),
    "ofrr_ctx_destroy": (C.c_int, [_P]),
    "ofrr_ctx_set_stream": (C.c_int, [_P, _P]),
    "ofrr_ctx_get_stream": (_P, [_P]),
    "ofrr_ctx_synchronize": (C.c_int, [_P]),
    "ofrr_ctx_launch_count": (C.c_uint64, [_P]),
    "ofrr_ctx_reset_launch_count": (None, [_P]),
    "ofrr_ctx_workspace_bytes": (C.c_size_t, [_P]),
    "ofrr_status_string": (C.c_char_p, [C.c_int]),
    "ofrr_version": (C.c_char_p, []),
    "ofrr_randn": (C.c_int, [_P, C.c_uint64, _I64, _I64, C.c_int, _P, _I64]),
    "ofrr_randn_host": (None, [C.c_uint64, _I64, _I64, _DP]),
    "ofrr_iamax": (C.c_int, [_P, C.c_int, _I64, _P, _IP, _DP]),
    "ofrr_matrix_iamax": (C.c_int, [_P, C.c_int, _I64, _I64, _P, _I64, _P]),
    "ofrr_scalecols": (C.c_int, [_P, C.c_int, C.c_int, _I64, _I64, _P, _I64, _P]),
    "ofrr_cast": (C.c_int, [_P, C.c_int, C.c_int, _I64, _I64, _P, _I64, _P, _I64]),
    "ofrr_check_special_values": (C.c_int, [_P, C.c_int, _I64, _I64, _P, _I64]),
    "ofrr_hessenberg": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, _I64, _I64, _P, _I64, _P, _I64, _D,
                                  _DP, _IP, _IP]),
    "ofrr_gemm": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _I64, _I64, _I64, _D,
                            _P, _I64, _P, _I64, _D, _P, _I64]),
    "ofrr_gemm_f64_emulated": (C.c_int, [_P, _I64, _I64, _I64, _P, _I64, _P, _I64, _P, _I64]),
    "ofrr_autotune_gemm16": (C.c_int, [_P, C.c_int, _I64, _I64, _I64, C.c_int, _IP, _IP, _DP]),
    "ofrr_gemm_e4m3": (C.c_int, [_P, _I64, _I64, _I64, _P, _I64, _P, _I64, _P, _I64]),
    "ofrr_gemm16_plan": (C.c_int, [C.c_int, _I64, _I64, _I64, _IP, _IP, _IP]),
    "ofrr_profile_gemm_f64_emulated": (C.c_int, [_P, _I64, _I64, _I64, _P, _I64, _P, _I64, _P, _I64, C.c_int,
                                                  _DP, _DP]),
    "ofrr_csrmm": (C.c_int, [_P, C.POINTER(ofrr_csr), C.c_int, C.c_int, C.c_int, C.c_int, _I64, _P, _I64, _P,
                             _I64]),
    "ofrr_profile_krylov_step": (C.c_int, [_P, C.POINTER(ofrr_csr), C.c_int, C.c_int, C.c_int, _DP, _DP]),
    "ofrr_test_matrix_spectrum": (C.c_int, [_P, C.c_int, C.c_uint64, _I64, _I64, C.c_int, _DP, _P, _I64]),
    "ofrr_debug_invariant_subspace": (C.c_int, [_P, C.c_int, _P, _P, _D, C.c_int, _P]),
    "ofrr_batch_sym_eig": (C.c_int, [_P, C.c_int, _P, _P, _P, C.POINTER(ofrr_options), _P, _P, _DP, _DP, _IP,
                                     _IP]),
    "ofrr_batch_sym_eig_timed": (C.c_int, [_P, C.c_int, _P, _P, _P, C.POINTER(ofrr_options), _P, _P, _DP, _DP,
                                           _IP, _IP, _DP]),
    "ofrr_syev": (C.c_int, [_P, C.c_int, _P, C.c_int, _P]),
    "ofrr_sygv": (C.c_int, [_P, C.c_int, _P, C.c_int, _P, C.c_int, _P]),
    "ofrr_options_default": (None, [C.POINTER(ofrr_options)]),
    "ofrr_si_eig": (C.c_int, [_P, C.POINTER(ofrr_operator), C.POINTER(ofrr_options), _P, _I64, _DP, _DP,
                              C.POINTER(ofrr_info)]),
    "ofrr_rr_eig": (C.c_int, [_P, C.POINTER(ofrr_operator), C.POINTER(ofrr_options), _I64, _P, _I64, _DP]),
    "ofrr_ofrr_eig": (C.c_int, [_P, C.POINTER(ofrr_operator), C.POINTER(ofrr_operator),
                                C.POINTER(ofrr_options), _I64, _P, _I64, _DP]),
    "ofrr_si_svd": (C.c_int, [_P, C.POINTER(ofrr_operator), C.POINTER(ofrr_options), _P, _I64, _DP, _P, _I64,
                              _DP, C.POINTER(ofrr_info)]),
    "ofrr_rr_svd": (C.c_int, [_P, C.POINTER(ofrr_operator), C.POINTER(ofrr_options), _I64, _P, _I64, _DP, _P,
                              _I64]),
    "ofrr_arnoldi_eig": (C.c_int, [_P, C.POINTER(ofrr_operator), C.POINTER(ofrr_options), _P, _P, _I64, _DP,
                                   _DP, C.POINTER(ofrr_info)]),
    "ofrr_residual_norms": (C.c_int, [_P, C.POINTER(ofrr_operator), C.c_int, _I64, _P, _I64, _DP, _D, _DP]),
    "ofrr_hessenberg_noalloc": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, _I64, _I64, _P, _I64, _P, _I64, _D, _P,
                                          _P, _P]),
    "ofrr_hessenberg_noalloc_scratch_bytes": (C.c_size_t, []),
    "ofrr_serve_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.c_int, C.c_size_t]),
    "ofrr_serve_destroy": (C.c_int, [_P]),
    "ofrr_serve_submit": (C.c_int, [_P, C.POINTER(ofrr_request), C.POINTER(C.c_uint64)]),
    "ofrr_serve_poll": (C.c_int, [_P, C.c_uint64, _IP, _IP]),
    "ofrr_serve_wait": (C.c_int, [_P, C.c_uint64, _IP, _DP]),
    "ofrr_serve_stats": (C.c_int, [_P, C.POINTER(ofrr_serve_report)]),
    "ofrr_batch_si_eig": (C.c_int, [_P, C.c_int, C.POINTER(ofrr_operator), C.POINTER(ofrr_options), C.POINTER(_P),
                                    C.POINTER(_I64), C.POINTER(_DP), C.POINTER(_DP), C.POINTER(ofrr_info), _IP]),
    "ofrr_ctx_trim": (C.c_int, [_P]),
    "ofrr_debug_bounded_wait": (C.c_int, [_P, _I64]),
    "ofrr_debug_scale_slice": (C.c_int, [_P, C.c_int, _I64, _I64, _I64, _P, _I64, _P, _I64, _P, _I64, _P, _P]),
    "ofrr_gs_basis": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, C.c_int, _I64, _I64, _P, _I64, _P, _I64, _D, _D, _D,
                                _DP, _IP]),
    "ofrr_rand_points": (C.c_int, [_P, C.c_uint64, _I64, C.c_int, C.c_int, _P, _I64]),
    "ofrr_gaussian_kernel": (C.c_int, [_P, C.c_int, _I64, _I64, C.c_int, _P, _I64, _P, _I64, _D, _D, _D, C.c_int, _P,
                                       _I64]),
    "ofrr_lu_basis": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, _I64, _I64, _P, _I64, _P, _I64, _D, _DP, _IP]),
    "ofrr_csr_file_sizes": (C.c_int, [C.c_char_p, C.POINTER(_I64), C.POINTER(_I64)]),
    "ofrr_csr_file_read": (C.c_int, [_P, C.c_char_p, _I64, _I64, _P, _P, _P, C.POINTER(_I64), C.c_int]),
    "ofrr_read_singular_values": (C.c_int, [C.c_char_p, C.POINTER(_I64), _P]),
    "ofrr_debug_gemm16_scalecols": (C.c_int, [_P, C.c_int, _I64, _I64, _I64, _P, _I64, _P, _I64, _P, _I64, C.c_int]),
    "ofrr_ctx_set_trace": (C.c_int, [_P, C.c_char_p]),
}

_lib = None


def load(path: os.PathLike | str | None = None):
    """Load the shared library (once) and declare every entry point of include/ofrr.h."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"{p} is not built; run `python -c 'import __graft_entry__ as g; g.build()'` "
            "(the CUDA library is required: there is no CPU fallback)")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class OfrrError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        msg = load().ofrr_status_string(status).decode()
        super().__init__(f"{what}: status {status} ({msg})" if what else f"status {status} ({msg})")


def check(status: int, what: str = "") -> int:
    if status != SUCCESS:
        raise OfrrError(status, what)
    return status
