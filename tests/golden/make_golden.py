"""Generate the committed golden fixtures (run in a checkout that has the reference beside it).

known_answers.json -- the reference's own known answers, read as text from its C++ tests:
    SYEV / SYGV true eigenvalues (CPP/tests/mvops_test.cpp:2292-2370, :2450-2530), the planted
    iamax case (mvops_test.cpp:774-796) and dot(1..10, 1..10) = 55 (mvops_test.cpp:28-98).
golden.npz -- oracle outputs on seeded inputs (Hessenberg bases in half/single/double,
    scalecols, small subspace-iteration and Krylov solves), used to pin the CUDA library and to
    regression-pin the oracle itself.

Usage: python tests/golden/make_golden.py --reference PATH
"""
from __future__ import annotations

import argparse
import json
import re
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from oracle import ofrr_oracle as orc  # noqa: E402


def parse_true_eigs(text: str, test_name: str):
    start = text.index(f"TEST(MvopsTest, {test_name})")
    block = text[start:]
    m = re.search(r"double true_eigenvalues\[n\]\s*=\s*\{([^}]*)\}", block)
    return [float(x) for x in m.group(1).replace("\n", " ").split(",") if x.strip()]


def known_answers(reference: Path) -> dict:
    txt = (reference / "CPP/tests/mvops_test.cpp").read_text()
    planted = re.search(r"const int expected_idx = (\d+);\s*x\[expected_idx\] = (-?[\d.]+);", txt)
    n_iamax = re.search(r"TEST\(MvopsTest, Iamax\).*?const int n = (\d+);", txt, re.S)
    return {
        "source": "CPP/tests/mvops_test.cpp of the reference",
        "syev_true_eigenvalues": parse_true_eigs(txt, "SYEV"),
        "sygv_true_eigenvalues": parse_true_eigs(txt, "SYGV"),
        "syev_tol": 1e-10,
        "iamax_n": int(n_iamax.group(1)),
        "iamax_planted_index0": int(planted.group(1)),
        "iamax_planted_value": float(planted.group(2)),
        "dot_1_to_10": 55.0,
        "hessenberg_skip_columns": [3, 4, 5],
        "hessenberg_tols": {"double": 1e-10, "single": 1e-5, "half": 5e-2},
        "hessenberg_select_tols": {"double": 1e-12, "single": 1e-6, "half": 1e-2},
    }


def golden() -> dict:
    g = {}
    rng = np.random.default_rng(2024)
    # Hessenberg bases (hessenberg.m) in the three precision pairs of the reference's tests
    for tag, pc, po, shape in (("half", "single", "half", (1200, 48)), ("single", "single", "single", (1000, 40)),
                               ("double", "double", "double", (800, 32))):
        A = rng.uniform(-1, 1, shape).astype(orc._dt(po))
        Q, R, sel, perm = orc.hessenberg(A, pc, po)
        g[f"hess_{tag}_A"] = A
        g[f"hess_{tag}_Q"] = Q
        g[f"hess_{tag}_R"] = R
        g[f"hess_{tag}_perm"] = perm
    # duplicated-column skip pattern (hessenberg_test.cpp:73-91), half storage
    A = rng.uniform(-1, 1, (600, 16)).astype(np.float16)
    A[:, 3:6] = A[:, 0:3]
    Q, R, sel, perm = orc.hessenberg(A, "single", "half", select_tol=1e-2)
    g["hess_dup_A"], g["hess_dup_sel"], g["hess_dup_Q"] = A, sel, Q
    # scalecols (scalecols.m) half storage / single compute
    U = (rng.standard_normal((900, 12)) * 3).astype(np.float16)
    g["scal_U"], g["scal_out"] = U, orc.scalecols(U, "single", "half")
    # subspace iteration on a 20x20 Laplacian (C1 shape scaled down), FP64 and half/single
    L = orc.laplacian_2d(20)
    Ac = orc.sparse2csr(L)
    V0 = orc.randn_block(42, L.shape[0], 16)
    g["si_V0"] = V0
    _, d = orc.subspace_iter_eig(Ac, L.shape[0], 16, "double", maxiter=8, step_size=2, V0=V0)
    g["si_d_double"] = d
    _, d = orc.subspace_iter_eig(Ac, L.shape[0], 16, "single", "half", maxiter=8, step_size=2, V0=V0)
    g["si_d_half"] = d
    # Krylov (arnoldi_hess_eig.m) on the same Laplacian
    v0 = orc.randn_block(7, L.shape[0], 1)[:, 0]
    g["kr_v0"] = v0
    _, d, info = orc.arnoldi_hess_eig(Ac, L.shape[0], 6, "double", maxiter=61, kdim=30, symmetric=True, v0=v0)
    g["kr_d_double"] = d
    g["kr_perm0"] = info["perms"][0]
    return g


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True, help="checkout of the reference repository (read as text)")
    a = ap.parse_args()
    ka = known_answers(Path(a.reference))
    (HERE / "known_answers.json").write_text(json.dumps(ka, indent=1) + "\n")
    g = golden()
    np.savez_compressed(HERE / "golden.npz", **g)
    print("wrote", HERE / "known_answers.json", HERE / "golden.npz")


if __name__ == "__main__":
    main()
