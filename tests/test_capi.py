"""CPU tests of the C ABI library: it builds, loads and exports every symbol of include/ofrr.h.

No compute entry point runs here (there is no GPU); only host-side functions are called.
"""
import ctypes as C
import re
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    hdr = (ROOT / "include" / "ofrr.h").read_text()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    return sorted(set(re.findall(r"\b(ofrr_[a-z0-9_]+)\s*\(", hdr)))


def test_every_declared_symbol_is_exported(built_lib):
    lib = C.CDLL(str(built_lib))
    syms = declared_symbols()
    assert len(syms) >= 25
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_python_binding_covers_header(built_lib):
    from mixedprecisionofrr_gb300 import _lib

    assert set(declared_symbols()) <= set(_lib.SIGNATURES)


def test_host_rng_matches_oracle(built_lib):
    from mixedprecisionofrr_gb300 import _lib
    from oracle import ofrr_oracle as orc

    lib = _lib.load()
    n, k = 333, 7
    out = np.zeros(n * k)
    lib.ofrr_randn_host(42, n, k, out.ctypes.data_as(C.POINTER(C.c_double)))
    ref = orc.randn_block(42, n, k)
    assert np.max(np.abs(out.reshape(k, n).T - ref)) < 1e-13


def test_status_strings_and_defaults(built_lib):
    from mixedprecisionofrr_gb300 import _lib

    lib = _lib.load()
    assert lib.ofrr_status_string(4001).decode() == "Solver reached max iterations"
    assert lib.ofrr_status_string(0).decode() == "Success"
    o = _lib.ofrr_options()
    lib.ofrr_options_default(C.byref(o))
    # MATLAB defaults: maxiter 5, step 1, seed 42 (subspace_iter_eig.m:105-113)
    assert (o.maxiter, o.step_size, o.seed, o.use_generalized) == (5, 1, 42, 1)
    assert o.select_tol < 0  # eps(output precision) by default
    assert o.step_size_f64 == 0  # the FP64 phase of the mixed mode takes step_size unless set


def _header_structs():
    """Field names, in order, of every `typedef struct { ... } name;` in include/ofrr.h."""
    import re
    from pathlib import Path

    txt = (Path(__file__).resolve().parents[1] / "include" / "ofrr.h").read_text()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    txt = re.sub(r"//[^\n]*", "", txt)
    out = {}
    for body, name in re.findall(r"typedef\s+struct\s*\{(.*?)\}\s*(\w+)\s*;", txt, flags=re.S):
        fields = []
        for decl in body.split(";"):
            decl = " ".join(decl.split())
            if not decl:
                continue
            # "type a, b" or "const int32_t* indptr": the names are the comma-separated tails
            first, *rest = decl.split(",")
            fields.append(first.replace("*", " ").split()[-1])
            fields += [r.replace("*", " ").strip() for r in rest]
        out[name] = fields
    return out


def test_ctypes_structs_follow_the_header():
    """The Python binding's structures list the C structures' fields in the header's order (an option
    added to one side only would shift every later field across the ABI)."""
    from mixedprecisionofrr_gb300 import _lib

    hdr = _header_structs()
    for name in ("ofrr_csr", "ofrr_operator", "ofrr_options", "ofrr_info", "ofrr_request", "ofrr_serve_report"):
        assert name in hdr, name
        py = [f[0] for f in getattr(_lib, name)._fields_]
        assert py == hdr[name], (name, py, hdr[name])
