"""Benchmark: converged singular triplets per second at residual <= 1e-8 on the dense truncated SVD
workload (A = U diag(s) V', 8192 x 2048, Haar U and V from seeded Gaussians, s geometric 1 -> 1e-6,
top 32 triplets), mixed-precision GB300 path vs the plain FP64 GPU path, with p50/p99 solve latency.

One step = one complete solve (start block -> 32 triplets with max residual <= 1e-8 checked in FP64).
`value` times solves whose input A is already resident in HBM; `e2e` times the same solve through the
C ABI with A in pinned host memory (host->device copy of A and device->host copy of U, s, V inside the
timed region).  `--impl reference` times the reference's algorithm on the host cores (the NumPy/SciPy
restatement: the reference's own solver path exists only in MATLAB).

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

M_ROWS, N_COLS, NEV, TOL = 8192, 2048, 32, 1e-8
BLOCK, STEP, MAXITER = 64, 8, 80  # defaults (the reference arm's); main() autotunes each GPU path
CFG = {"mixed": (BLOCK, STEP, 0), "fp64": (BLOCK, STEP, 0)}  # block, power steps, FP64-phase steps (0: same)
METRIC = "converged singular triplets/s at residual <= 1e-8 (dense 8192x2048 geometric-spectrum SVD, top 32)"
UNIT = "triplets/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--profile-solve", action="store_true",
                    help="run one warm-up and one mixed solve only (for a profiler's launch list)")
    ap.add_argument("--roofline-only", action="store_true",
                    help="run only the live timing of the roofline kernel (for an ncu capture of it)")
    ap.add_argument("--orth-compare", action="store_true",
                    help="basis build and FP64 solve of the dense SVD with the Hessenberg, LU, MGS and CGS bases")
    ap.add_argument("--kernel-gen", action="store_true",
                    help="time the Gaussian kernel generator (16384 points in 3D) against the HBM peak")
    ap.add_argument("--csr-load", action="store_true",
                    help="time reading the 128^3 7-point CSR operator (on-disk format) into HBM")
    ap.add_argument("--config", default="c2", choices=["c2", "c3", "c4", "c5"],
                    help="c2: the dense SVD headline (default; also runs a compact C3 leg); c3: the 128^3 "
                         "convection-diffusion Krylov workload alone; c5: the serving stream")
    ap.add_argument("--requests", type=int, default=400, help="c5: requests replayed from the seeded stream")
    ap.add_argument("--batch-count", type=int, default=None,
                    help="c4: matrices in the batch (default 4096; smaller only for profiler captures)")
    ap.add_argument("--time-scale", type=float, default=1.0,
                    help="c5: arrival times multiplied by this (1 = the stream's 2000 req/s)")
    ap.add_argument("--no-c3", action="store_true", help="skip the C3 leg of the default run")
    ap.add_argument("--mixed-config", default=None, metavar="B,S[,S64]",
                    help="block width, power steps (and FP64-phase power steps) of the mixed path instead of the "
                         "autotuner's choice")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def make_problem_host(seed=42):
    """A = U diag(s) V' in FP64 on the host: U, V = Q factors of seeded Gaussian blocks (the library's
    counter-based generator), sign-fixed; s geometric from 1 to 1e-6.  Input synthesis only."""
    from mixedprecisionofrr_gb300 import api

    def haar(n, k, sd):
        G = api.randn_host(sd, n, k)
        Q, R = np.linalg.qr(G)
        return Q * np.sign(np.diag(R))[None, :]

    U = haar(M_ROWS, N_COLS, seed)
    V = haar(N_COLS, N_COLS, seed + 1)
    s = 1e-6 ** (np.arange(N_COLS) / (N_COLS - 1))
    return (U * s[None, :]) @ V.T, s


def make_problem_gpu(seed=42):
    from mixedprecisionofrr_gb300 import api

    A, s = make_problem_host(seed)
    return api.to_device_cm(A, api.PREC["double"]), s


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    def __init__(self, index: int = 0):
        self.index = index
        self.proc = None
        self.path = Path(os.environ.get("TMPDIR", "/tmp")) / f"ofrr_clocks_{os.getpid()}.csv"

    def __enter__(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index),
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
                "samples": len(sm)}


def flush_l2(buf):
    buf.add_(1.0)


def run_solver(api, A, mode, V0=None, fp8=False):
    b, st, st64 = CFG.get(mode, (BLOCK, STEP, 0))
    return api.subspace_iter_svd(A, M_ROWS, N_COLS, b, "single", "half", maxiter=MAXITER, step_size=st,
                                 mode=mode, tol=TOL, nev=NEV, check_every=1, V0=V0, generalized_tol=0.0,
                                 power_fp8=fp8, step_size_f64=st64)


def time_solves(api, A, mode, steps, warmup, flush_buf, fp8=False):
    import torch

    stream = torch.cuda.current_stream()
    for _ in range(warmup):
        run_solver(api, A, mode, fp8=fp8)
    torch.cuda.synchronize()
    times, infos = [], []
    ctx = api.context()
    ctx.reset_launch_count()
    for _ in range(steps):
        flush_l2(flush_buf)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        U, s, V, info = run_solver(api, A, mode, fp8=fp8)
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
        infos.append(info)
    launches = ctx.launch_count
    return np.array(times), infos, launches, s


def time_e2e(api, A_host_pinned, steps, warmup):
    """Through the C ABI with host buffers: H2D of A, solve, D2H of U, s, V per step."""
    import torch
    from mixedprecisionofrr_gb300 import _lib as L

    ctx = api.context()
    stream = torch.cuda.current_stream()
    BLOCK, STEP, STEP64 = CFG["mixed"]
    A_dev = api.empty_cm(M_ROWS, N_COLS, L.F64)
    U_dev = api.empty_cm(M_ROWS, BLOCK, L.F64)
    V_dev = api.empty_cm(N_COLS, BLOCK, L.F64)
    U_host = torch.empty((BLOCK, M_ROWS), dtype=torch.float64).pin_memory()
    V_host = torch.empty((BLOCK, N_COLS), dtype=torch.float64).pin_memory()
    s = np.zeros(BLOCK)
    res = np.zeros(BLOCK)
    inf = L.ofrr_info()
    op = L.ofrr_operator()
    op.kind, op.nrows, op.ncols, op.symmetric = L.OP_DENSE, M_ROWS, N_COLS, 0
    op.dtype, op.data, op.ld = L.F64, A_dev.data_ptr(), M_ROWS
    o = api.options(mode=L.MODE_MIXED, maxiter=MAXITER, step_size=STEP, block=BLOCK, nev=NEV, tol=TOL,
                    use_generalized=1, generalized_tol=0.0, seed=42, check_every=1, p_compute="single",
                    p_output="half", p_hess_compute="single", p_hess_output="half", p_rr_compute="single",
                    p_rr_output="single", step_size_f64=STEP64)
    lib = ctx.lib
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731

    def one():
        A_dev.t().copy_(A_host_pinned, non_blocking=True)
        st = lib.ofrr_si_svd(ctx.h, C.byref(op), C.byref(o), U_dev.data_ptr(), M_ROWS, dp(s), V_dev.data_ptr(),
                             N_COLS, dp(res), C.byref(inf))
        U_host.copy_(U_dev.t(), non_blocking=True)
        V_host.copy_(V_dev.t(), non_blocking=True)
        return st

    for _ in range(warmup):
        one()
    torch.cuda.synchronize()
    ts = []
    for _ in range(steps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        st = one()
        e1.record(stream)
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1) / 1e3)
    h2d = M_ROWS * N_COLS * 8
    d2h = (M_ROWS + N_COLS) * BLOCK * 8 + BLOCK * 8
    return np.array(ts), st, h2d, d2h, float(np.max(res[:NEV]))


def gemm_roofline(api, steps=20):
    """Live CUDA-event timing of the dominant contraction of the low-precision phase: the 16-bit
    A.V product (8192 x 2048 by 2048 x 64, FP32 accumulation), on the library's stream.  A' (33.5 MB)
    fits in L2, so a 256 MB buffer is written between launches and each launch is timed alone."""
    import torch
    from mixedprecisionofrr_gb300 import _lib as L

    ctx = api.context()
    # the solver keeps A' (K-contiguous rows of A) and runs A V as the TN product (A')' V
    BLOCK = CFG["mixed"][0]
    At = api.randn(7, N_COLS, M_ROWS, "half")
    X = api.randn(8, N_COLS, BLOCK, "half")
    Y = api.empty_cm(M_ROWS, BLOCK, L.F16)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    lib = ctx.lib

    def call():
        st = lib.ofrr_gemm(ctx.h, 1, 0, L.F16, L.F16, L.F32, L.F16, M_ROWS, BLOCK, N_COLS, 1.0, At.data_ptr(), N_COLS,
                           X.data_ptr(), N_COLS, 0.0, Y.data_ptr(), M_ROWS)
        assert st == 0

    for _ in range(3):
        call()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    ts = []
    for i in range(steps):
        flush.fill_(float(i))
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        call()
        e1.record(stream)
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1) / 1e3)
    dt = float(np.median(ts))
    algo_bytes = (M_ROWS * N_COLS + N_COLS * BLOCK + M_ROWS * BLOCK) * 2
    flops = 2.0 * M_ROWS * N_COLS * BLOCK
    del flush
    return dt, algo_bytes, flops


def sliced_roofline(api, reps=20):
    """Live CUDA-event timing of the dominant kernel of the solve, the fused exact-slice product
    k_sliced_tn, on the solver's A V shape (C 8192 x 64 = A_op' V, A_op the 5-digit stack of A',
    K = 2048): the library slices both operands once and times reps launches of the kernel alone
    on its stream.  The A digit stack (168 MB) is larger than L2, so every launch streams it."""
    import torch
    import ctypes as C
    from mixedprecisionofrr_gb300 import _lib as L

    ctx = api.context()
    BLOCK = CFG["mixed"][0]
    At = api.randn(11, N_COLS, M_ROWS, "double")  # A' (K x M, FP64)
    X = api.randn(12, N_COLS, BLOCK, "double")
    Y = api.empty_cm(M_ROWS, BLOCK, L.F64)
    us = C.c_double()
    nbytes = C.c_double()
    st = ctx.lib.ofrr_profile_gemm_f64_emulated(ctx.h, M_ROWS, BLOCK, N_COLS, At.data_ptr(), N_COLS, X.data_ptr(),
                                                N_COLS, Y.data_ptr(), M_ROWS, reps, C.byref(us), C.byref(nbytes))
    assert st == 0, st
    torch.cuda.synchronize()
    del At, X, Y
    return us.value * 1e-6, nbytes.value


def profiled_traffic(name="k_sliced_tn_av_8192x64x2048.md"):
    """DRAM bytes per launch of a roofline kernel, from its committed ncu summary (None if absent)."""
    p = ROOT / "profiles" / name
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return int(float(line.split(":", 1)[1].strip()))
            except ValueError:
                return None
    return None


def orth_compare_run(api, A, reps=3):
    """The paper's comparison on the dense 8192 x 2048 problem: one basis build of an 8192 x 64 FP64 block
    (scaled power iterate) with each basis, and the FP64-mode solve (top 32, residual <= 1e-8) with the
    same basis for both blocks; CUDA events around each, median of reps."""
    import torch

    stream = torch.cuda.current_stream()

    def timed(fn):
        ts, out = [], None
        for r in range(reps + 1):
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            out = fn()
            e1.record(stream)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        return float(np.median(ts[1:])), out

    X = api.scalecols(api.gemm(A, "N", api.randn(42, N_COLS, 64), "double", "double"), "double", "double")
    res = {"orth_compare": True, "block": [M_ROWS, 64]}
    for orth in ("hessenberg", "lu", "mgs", "cgs"):
        if orth == "hessenberg":
            ms_b, _ = timed(lambda: api.hessenberg(X, "double", "double"))
        elif orth == "lu":
            ms_b, _ = timed(lambda: api.lu_basis(X, "double", "double"))
        else:
            ms_b, _ = timed(lambda: api.gs_basis(X, orth == "cgs", "double", "double"))
        b, st, _ = CFG.get("fp64", (BLOCK, STEP, 0))
        ms_s, out = timed(lambda: api.subspace_iter_svd(A, M_ROWS, N_COLS, b, "double", "double", maxiter=MAXITER,
                                                        step_size=st, mode="fp64", tol=TOL, nev=NEV, orth=orth))
        info = out[3]
        res[orth] = {"basis_ms": ms_b, "fp64_solve_ms": ms_s, "iterations": info.iterations,
                     "max_residual": info.max_residual, "status": info.status}
    return res


def max_over_ranks(x: float, world: int, device: str = "cuda") -> float:
    """The slowest rank's time of the timed region (every rank runs its own replica of the workload;
    the whole-job value is the units all ranks processed over this time), then a barrier."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.barrier()
    return float(t.item())


def job_value(steps: int, world: int, total_seconds: float) -> float:
    """Whole-job throughput: NEV triplets per solve, `steps` solves on each of `world` replicas."""
    return NEV * steps * world / total_seconds


def measured_hbm_peak():
    pk = ROOT / "MEASURED_PEAKS.json"
    return json.loads(pk.read_text()).get("hbm_gbs") if pk.exists() else None


def kernel_gen_run(api, n=16384, d=3, reps=5):
    """generate_gaussian_kernel's matrix for n points in [0, n^(1/3))^3 (the largest dense size of the
    serving mix), one launch writing n^2 entries: CUDA events, median of reps, HBM-write rate against
    the measured copy peak."""
    import torch
    from mixedprecisionofrr_gb300 import _lib as L

    ctx = api.context()
    X = api.rand_points(1, n, d, 0)
    out = {"kernel_gen": True, "n": n, "d": d}
    peak = measured_hbm_peak()
    for prec, code, es in (("double", L.F64, 8), ("single", L.F32, 4), ("half", L.F16, 2)):
        K = api.empty_cm(n, n, code)
        ts = []
        for r in range(reps + 1):
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            L.check(ctx.lib.ofrr_gaussian_kernel(ctx.h, 0, n, n, d, X.data_ptr(), n, X.data_ptr(), n, 1.0, 1.0, 0.1,
                                                 code, K.data_ptr(), n), "gaussian_kernel")
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        ms = float(np.median(ts[1:]))
        gbs = n * n * es / ms / 1e6
        out[prec] = {"ms": ms, "write_GBps": gbs, "frac_of_hbm_peak": gbs / peak if peak else None}
        del K
    return out


def csr_load_run(api, N=128, reps=3):
    """The on-disk CSR format (<prefix>_row_ptr.bin / _col_ind.bin / _values.bin) of a 7-point
    operator on an N^3 grid (n = 2,097,152 and nnz = 14,581,760 at N = 128, seeded values), written to
    a temporary directory and read into HBM by read_csr (pinned staging, GPU validation); the page
    cache holds the files after the first read, so the figure is the loader's, not the disk's."""
    import tempfile
    import scipy.sparse as sp
    import torch

    T = sp.diags([-np.ones(N - 1), 2 * np.ones(N), -np.ones(N - 1)], [-1, 0, 1], format="csr")
    I = sp.identity(N, format="csr")
    A = (sp.kron(sp.kron(I, I), T) + sp.kron(sp.kron(I, T), I) + sp.kron(sp.kron(T, I), I)).tocsr()
    A.sort_indices()
    A.data = A.data * (1.0 + 0.01 * np.random.default_rng(42).standard_normal(A.nnz))
    nbytes = 4 * (A.shape[0] + 1) + 12 * A.nnz
    with tempfile.TemporaryDirectory() as d:
        prefix = os.path.join(d, "convdiff128")
        A.indptr.astype(np.int32).tofile(prefix + "_row_ptr.bin")
        A.indices.astype(np.int32).tofile(prefix + "_col_ind.bin")
        A.data.astype(np.float64).tofile(prefix + "_values.bin")
        times = {}
        for on_device in (True, False):
            ts = []
            for r in range(reps + 1):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                M = api.read_csr(prefix, symmetric=False, on_device=on_device)
                torch.cuda.synchronize()
                ts.append(time.perf_counter() - t0)
            times[on_device] = float(np.median(ts[1:]))
            ok = (M.shape == A.shape and torch.equal(M.indices.cpu(), torch.from_numpy(A.indices.astype(np.int32)))
                  and torch.equal(M.a_double.cpu(), torch.from_numpy(A.data)))
            if not ok:
                raise RuntimeError("read_csr returned different arrays")
            del M
    return {"csr_load": True, "n": int(A.shape[0]), "nnz": int(A.nnz), "file_bytes": nbytes,
            "ms_device_path": times[True] * 1e3, "GBps_device_path": nbytes / times[True] / 1e9,
            "ms_host_path": times[False] * 1e3, "GBps_host_path": nbytes / times[False] / 1e9}


C3_N, C3_NEV, C3_KDIM, C3_TOL = 128, 20, 64, 1e-8
C3_METRIC = ("converged eigenpairs/s at residual <= 1e-8 (3D 7-point convection-diffusion 128^3, Pe 10, "
             "20 eigenvalues of largest real part, Krylov dim 64 with thick restarts)")


def c3_solve(api, Acsr, mode):
    """One thick-restart Krylov solve of the 128^3 convection-diffusion operator; returns (X, d, info)."""
    return api.arnoldi_hess_eig(Acsr, Acsr.shape[0], C3_NEV, "single", "half" if mode == "mixed" else None,
                                maxiter=40000, kdim=C3_KDIM, mode=mode, tol=C3_TOL)


def c3_cpu_sample(A, steps_total, cycles, nsteps=12, i_mid=32):
    """The host cores on a bounded sample of the C3 solve (FP64 NumPy/SciPy, the oracle's arithmetic):
    nsteps Krylov steps at the mean basis width (CSR matvec + eliminations against i_mid columns) and one
    Rayleigh-Ritz (A V for 65 columns, the two Gram matrices), scaled to the GPU solve's step and cycle
    counts.  Returns (seconds per solve, sample description)."""
    from oracle import ofrr_oracle as orc

    n = A.shape[0]
    Ac = orc.sparse2csr(A)
    rng = np.random.default_rng(0)
    V = rng.standard_normal((n, C3_KDIM + 1))
    piv = list(rng.choice(n, i_mid, replace=False))
    t0 = time.perf_counter()
    for _ in range(nsteps):
        w = orc.matvec_auto(Ac, "N", V[:, i_mid], "double", "double")
        w = w - V[:, :i_mid] @ w[piv]
        w[piv] = 0.0
        V[:, i_mid] = w / w[int(np.argmax(np.abs(w)))]
    t_step = (time.perf_counter() - t0) / nsteps
    t0 = time.perf_counter()
    AV = orc.matvec_auto(Ac, "N", V, "double", "double")
    G = V.T @ AV
    M = V.T @ V
    t_rr = time.perf_counter() - t0
    assert np.isfinite(G[0, 0] + M[0, 0])
    secs = steps_total * t_step + cycles * t_rr
    return secs, (f"{nsteps} FP64 Krylov steps at basis width {i_mid} ({1e3 * t_step:.0f} ms each) and one "
                  f"Rayleigh-Ritz ({t_rr:.2f} s) on the 128^3 operator, scaled to the GPU solve's {steps_total} "
                  f"operator applications and {cycles} cycles")


def c3_run(api, steps, warmup, cpu=True):
    """The nonsymmetric sparse workload: mixed path (16-bit then FP64 phase) vs the plain FP64 path."""
    import torch
    from mixedprecisionofrr_gb300 import problems

    A = problems.convdiff_3d(C3_N)
    ex = problems.convdiff_3d_eigs(C3_N, count=C3_NEV)
    Acsr = api.CsrMatrix(A, symmetric=False)
    stream = api.context().stream
    out = {"workload": "3D convection-diffusion 128^3 (n 2,097,152, nnz 14,581,760), Pe 10, w (1,0.5,0.25), "
                       "20 eigenvalues of largest real part, kdim 64, tol 1e-8",
           "metric": C3_METRIC, "unit": "eigenpairs/s"}
    for _ in range(warmup):
        c3_solve(api, Acsr, "mixed")
    ts, infos = [], []
    d = None
    for _ in range(steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        X, d, info = c3_solve(api, Acsr, "mixed")
        e1.record(stream)
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1) / 1e3)
        infos.append(info)
    ts = np.array(ts)
    out.update({"value": C3_NEV * len(ts) / float(ts.sum()), "ms_per_solve": 1e3 * float(ts.mean()),
                "p50_ms": 1e3 * float(np.percentile(ts, 50)), "p99_ms": 1e3 * float(np.percentile(ts, 99)),
                "status": sorted({i.status for i in infos}), "cycles": infos[-1].iterations,
                "matvecs": infos[-1].matvecs, "escalations": infos[-1].escalations,
                "max_residual": float(max(i.max_residual for i in infos)),
                "max_rel_eig_err": float(np.max(np.abs(d - ex)) / ex[0]),
                "dtype": "f16 basis / f32 matvec+arithmetic, then f64 (Grams and Ritz products emulated on tcgen05)"})
    # plain FP64 GPU path (same algorithm, every operand FP64, library DGEMM for the Gram and Ritz products)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    X64, d64, i64 = c3_solve(api, Acsr, "fp64")
    e1.record(stream)
    torch.cuda.synchronize()
    t64 = e0.elapsed_time(e1) / 1e3
    out["fp64_path"] = {"value": C3_NEV / t64, "ms_per_solve": 1e3 * t64, "cycles": i64.iterations,
                        "matvecs": i64.matvecs, "status": i64.status, "max_residual": i64.max_residual,
                        "max_rel_eig_err": float(np.max(np.abs(d64 - ex)) / ex[0])}
    out["speedup_vs_fp64"] = out["value"] / out["fp64_path"]["value"]
    # end to end: CSR arrays from pinned host memory, the solve, Ritz vectors and values back
    ip = torch.from_numpy(A.indptr.astype(np.int32)).pin_memory()
    ix = torch.from_numpy(A.indices.astype(np.int32)).pin_memory()
    vd = torch.from_numpy(A.data.astype(np.float64)).pin_memory()
    vs = torch.from_numpy(A.data.astype(np.float32)).pin_memory()
    Xh = torch.empty((C3_NEV, A.shape[0]), dtype=torch.float64).pin_memory()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    Ae = api.CsrMatrix.__new__(api.CsrMatrix)
    Ae.shape, Ae.nnz, Ae.symmetric = A.shape, A.nnz, False
    Ae.indptr, Ae.indices = ip.to("cuda", non_blocking=True), ix.to("cuda", non_blocking=True)
    Ae.a_double, Ae.a_single = vd.to("cuda", non_blocking=True), vs.to("cuda", non_blocking=True)
    Ae.a_half = Ae.a_single  # never read by this path
    torch.cuda.synchronize()
    Xe, de, ie = c3_solve(api, Ae, "mixed")
    Xh.copy_(Xe.t(), non_blocking=True)
    torch.cuda.synchronize()
    te = time.perf_counter() - t0
    h2d = (A.indptr.size + A.indices.size) * 4 + A.data.size * 12
    out["e2e"] = {"value": C3_NEV / te, "unit": "eigenpairs/s", "ms_per_step": 1e3 * te, "h2d_bytes_per_step": h2d,
                  "d2h_bytes_per_step": C3_NEV * A.shape[0] * 8 + C3_NEV * 8, "status": ie.status}
    # roofline of the dominant kernel, the fused Krylov step (live CUDA events; the operator and the basis,
    # 125 + 272 MB, exceed L2, so back-to-back launches stream from HBM)
    pk = ROOT / "MEASURED_PEAKS.json"
    peaks = json.loads(pk.read_text()) if pk.exists() else {}
    hbm = peaks.get("hbm_gbs", 6800.0)
    roof = {"peak_GBps": hbm, "peak_source": "measured" if "hbm_gbs" in peaks else "fallback"}
    for prec, i in (("half", 16), ("half", 40), ("half", 64), ("double", 40)):
        us, by = api.profile_krylov_step(Acsr, prec, i, reps=20)
        roof[f"{prec}_i{i}"] = {"us": us, "bytes": by, "GBps": by / us / 1e3, "frac": by / us / 1e3 / hbm}
    out["roofline_krylov_step"] = roof
    # the Rayleigh-Ritz SpMM of the FP64 phase: A times the 65 FP64 basis columns (live CUDA events, 5 launches)
    Xs = api.randn(13, A.shape[0], C3_KDIM + 1, "double")
    api.csrmv(Acsr, "N", Xs, "double")
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(5):
        Ys = api.csrmv(Acsr, "N", Xs, "double")
    e1.record(stream)
    torch.cuda.synchronize()
    t_sp = e0.elapsed_time(e1) / 5 * 1e-3
    nrhs = C3_KDIM + 1
    by_sp = A.nnz * 12 + (A.shape[0] + 1) * 4 + A.shape[0] * nrhs * 16
    # the FP64 kernel's bound is GB300's FP64 pipe, not HBM: nnz * nrhs FMAs against 1.68 FMA per clock per
    # SM (stand-alone probe) x 152 SMs x 2070 MHz
    fma_peak = 152 * 1.68 * 2.070e9
    out["roofline_spmm"] = {"kernel": f"k_csrmm_n FP64, {nrhs} right-hand sides", "us": t_sp * 1e6, "bytes": by_sp,
                            "GBps": by_sp / t_sp / 1e9, "frac": by_sp / t_sp / 1e9 / hbm,
                            "fp64_fma": A.nnz * nrhs, "fp64_fma_peak_per_s": fma_peak,
                            "fp64_fma_frac": A.nnz * nrhs / t_sp / fma_peak}
    del Xs, Ys
    if cpu:
        secs, sample = c3_cpu_sample(A, out["matvecs"], out["cycles"])
        out["cpu_baseline"] = {"value": C3_NEV / secs, "unit": "eigenpairs/s", "cores": os.cpu_count(),
                               "kind": "port", "sample": sample}
    return out


C4_COUNT, C4_NEV, C4_TOL = 4096, 8, 1e-7
C4_METRIC = ("converged eigenpairs/s at residual <= 1e-7 (4096 dense symmetric Q diag(l) Q', n uniform in "
             "[64, 1024], l log-uniform in [1e-4, 1], top 8 each, one persistent launch)")


def c4_problem(api, count=C4_COUNT, seed=4096):
    """The batch: n_i uniform in [64, 1024], eigenvalues log-uniform in [1e-4, 1], each matrix built on the
    GPU from Householder reflectors around diag(l) (exact spectrum), packed column-major in one buffer."""
    import torch

    rng = np.random.default_rng(seed)
    ns = rng.integers(64, 1025, count).astype(np.int64)
    offs = np.concatenate([[0], np.cumsum(ns * ns)[:-1]]).astype(np.int64)
    buf = torch.empty(int((ns * ns).sum()), dtype=torch.float64, device="cuda")
    lams = []
    ctx = api.context()
    for i, n in enumerate(ns):
        lam = np.sort(np.exp(np.log(1e-4) + np.log(1e4) * rng.random(int(n))))[::-1].copy()
        lams.append(lam[:C4_NEV])
        ptr = buf.data_ptr() + int(offs[i]) * 8
        api.L.check(ctx.lib.ofrr_test_matrix_spectrum(ctx.h, 1, seed * 10007 + i, int(n), int(n), 3, api._dp(lam), ptr,
                                                      int(n)), "test_matrix_spectrum")
    torch.cuda.synchronize()
    return buf, ns, offs, np.array(lams)


def c4_run(api, steps, warmup, cpu=True, count=None):
    """The batched workload: 4096 matrices in one persistent launch (the FP64 refinement in the same CTAs)."""
    import torch

    buf, ns, offs, lams = c4_problem(api, count=count or C4_COUNT)
    stream = api.context().stream
    # power steps per outer iteration: tuned on the batch itself (one untimed run per candidate; more steps
    # per Rayleigh-Ritz amortise its on-chip work, fewer avoid wasted products on easy matrices)
    tune = []
    for st in (3, 4, 6, 8):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        _, _, res_t, _, _ = api.batch_sym_eig(buf, ns, offs, nev=C4_NEV, tol=C4_TOL, step_size=st)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        tune.append({"step_size": st, "s": dt, "converged_pairs": int(np.sum(res_t <= C4_TOL))})
    step = max(tune, key=lambda t: t["converged_pairs"] / t["s"])["step_size"]
    for _ in range(warmup):
        api.batch_sym_eig(buf, ns, offs, nev=C4_NEV, tol=C4_TOL, step_size=step)
    ts = []
    for _ in range(steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        Xs, ev, res, its, sts, lat = api.batch_sym_eig(buf, ns, offs, nev=C4_NEV, tol=C4_TOL, step_size=step,
                                                       return_latency=True)
        e1.record(stream)
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1) / 1e3)
    ts = np.array(ts)
    conv = int(np.sum(res <= C4_TOL))
    err = float(np.max(np.abs(ev - lams) / lams[:, :1]))
    abytes = float((ns * ns).sum()) * 2  # the 16-bit copy of A streamed once per product of the first phase
    out = {"workload": "4096 dense symmetric Q diag(l) Q', n ~ U[64,1024], l log-uniform [1e-4,1], top 8, tol 1e-7",
           "metric": C4_METRIC, "unit": "eigenpairs/s", "value": conv * len(ts) / float(ts.sum()) / len(ts) * len(ts),
           "ms_per_batch": 1e3 * float(ts.mean()), "converged_pairs": conv, "pairs": int(res.size),
           "matrices_failed": int(np.sum(sts != 0)), "max_residual": float(res.max()),
           "max_rel_eig_err": err, "iterations_mean": float(its.mean()), "iterations_max": int(its.max()),
           "per_matrix_latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99))},
           "bytes_16bit_A": abytes, "step_size": step, "tuning": tune,
           "failed": [{"matrix": int(i), "n": int(ns[i]), "iterations": int(its[i]), "max_residual": float(res[i].max()),
                       "status": int(sts[i])} for i in np.nonzero(sts != 0)[0][:20]],
           "dtype": "bf16 A / f32 accumulate, then f32 A; f64 refinement of the 8 leading pairs"}
    out["value"] = conv / float(ts.mean())
    if cpu:
        from oracle import ofrr_oracle as orc

        idx = np.random.default_rng(7).choice(len(ns), 12, replace=False)
        t0 = time.perf_counter()
        npairs = 0
        class Stop(Exception):
            pass

        for i in idx:
            n = int(ns[i])
            A = buf[int(offs[i]):int(offs[i] + n * n)].view(n, n).t().cpu().numpy()

            def cb(it, V, d, A=A):
                r = orc.residual_norms(A, V[:, :C4_NEV], d[:C4_NEV], normA=float(np.max(np.abs(d[:C4_NEV]))))
                if np.max(r) <= C4_TOL:
                    raise Stop()

            try:
                orc.subspace_iter_eig(A, n, 16, "double", maxiter=400, step_size=2, callback=cb)
            except Stop:
                npairs += C4_NEV
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": npairs / dt, "unit": "eigenpairs/s", "cores": os.cpu_count(), "kind": "port",
                               "sample": f"FP64 NumPy subspace iteration (block 16, 2 power steps) on 12 matrices drawn "
                                         f"from the batch (n {sorted(int(ns[i]) for i in idx)}), {dt:.1f} s"}
    return out


def c5_run(api, count, time_scale, parity_every=25):
    """The serving stream: the first `count` requests of the seeded Poisson stream (2000 req/s, 60 % dense
    SVD, 40 % Laplacian eigenproblems, k in [4, 64], tol in {1e-6, 1e-8, 1e-10}) replayed in real time
    through the solve engine with a 150 GB budget; then every parity_every-th request solved alone and
    compared with its result in the mix."""
    from mixedprecisionofrr_gb300 import serve_stream as ss

    reqs = ss.make_stream(seed=2024, count=count)
    out = ss.run_stream(reqs, time_scale=time_scale)
    recs = out.pop("records")
    byidx = {r["idx"]: r for r in recs}
    parity = []
    for req in reqs[::parity_every]:
        st, keep = ss.solve_alone(req)
        r = byidx[req.idx]
        va, vm = np.asarray(keep[-3])[:req.k], np.asarray(r["values"])[:req.k]
        scale = float(np.max(np.abs(va))) if va.size else 1.0
        rel = float(np.max(np.abs(va - vm)) / scale) if va.size else 0.0
        parity.append({"idx": req.idx, "kind": req.kind, "tol": req.tol, "status_alone": st, "status_mix": r["status"],
                       "identical": bool(np.array_equal(va, vm, equal_nan=True)), "max_rel_diff": rel,
                       "within_tol": bool(rel <= req.tol)})
    for r in recs:
        r.pop("values", None)
    # one row per request: index, kind, n, k, tol, status, solve ms, latency ms, max residual
    rows = [[r["idx"], r["kind"], r["n"], r["k"], r["tol"], r["status"], round(r["solve_ms"], 1),
             round(r["latency_ms"], 1), float("%.3g" % r["max_residual"])] for r in sorted(recs, key=lambda r: r["idx"])]
    kinds = {}
    for r in recs:
        kk = kinds.setdefault(r["kind"], {"count": 0, "ok": 0, "lat": []})
        kk["count"] += 1
        kk["ok"] += int(r["status"] == 0)
        kk["lat"].append(r["latency_ms"])
    for kk in kinds.values():
        lat = np.array(kk.pop("lat"))
        kk["p50_ms"], kk["p99_ms"] = float(np.percentile(lat, 50)), float(np.percentile(lat, 99))
    out.update({"metric": "serving stream: requests/s, converged eigen/singular pairs/s, p50/p99 latency "
                          "(arrival to completion)", "stream": {"seed": 2024, "requests": count, "rate_req_s": 2000,
                                                                "time_scale": time_scale},
                "by_kind": kinds, "parity_sample": parity,
                "request_rows": {"columns": ["idx", "kind", "n", "k", "tol", "status", "solve_ms", "latency_ms",
                                             "max_residual"], "rows": rows}})
    return out


CPU_GRID = ((64, 96, 128), (4, 6, 8))  # block widths x power steps, the GPU autotuner's grid


def _cpu_solve(orc, A_host, b, st, max_seconds):
    """One FP64 oracle solve with block b and st power steps, stopped at max residual <= 1e-8 (or after
    max_seconds); returns (seconds, outer iterations, max residual)."""
    state = {"it": 0, "res": np.inf}
    t0 = time.perf_counter()

    class Stop(Exception):
        pass

    def cb(it, U, s, V):
        r = orc.svd_residual_norms(A_host, U[:, :NEV], s[:NEV], V[:, :NEV])
        state["it"], state["res"] = it + 1, float(np.max(r))
        if state["res"] <= TOL or time.perf_counter() - t0 > max_seconds:
            raise Stop()

    try:
        orc.subspace_iter_svd(A_host, M_ROWS, N_COLS, b, "double", maxiter=MAXITER, step_size=st,
                              generalized_tol=0.0, callback=cb)
    except Stop:
        pass
    return time.perf_counter() - t0, state["it"], state["res"]


def cpu_tune(A_host):
    """Block width and power steps of the host-side solve, chosen the same way in both bench arms: over
    the GPU autotuner's grid, the converged candidate with the fewest modelled flops (outer iterations x
    (power-step products 4 m n b per step + bases and Gram products ~8 (m + n) b^2)).  Iteration counts
    are deterministic, so both arms pick the same configuration."""
    from oracle import ofrr_oracle as orc

    best, table = None, []
    for b in CPU_GRID[0]:
        for st in CPU_GRID[1]:
            dt, it, res = _cpu_solve(orc, A_host, b, st, 20.0)
            flops = it * (st * 4.0 * M_ROWS * N_COLS * b + 8.0 * (M_ROWS + N_COLS) * b * b)
            table.append({"block": b, "step_size": st, "iterations": it, "max_residual": res, "gflop": flops / 1e9,
                          "seconds": dt})
            if res <= TOL and (best is None or flops < best[0]):
                best = (flops, b, st)
    if best is None:
        return (BLOCK, STEP), table
    return (best[1], best[2]), table


def cpu_baseline_run(A_host, cfg, max_seconds=60.0):
    """The oracle (FP64 NumPy/SciPy restatement of the reference's MATLAB path) on this host's cores:
    one full solve with the block / step cfg and the same tolerance, stopped at max residual <= 1e-8."""
    from oracle import ofrr_oracle as orc

    dt, it, res = _cpu_solve(orc, A_host, cfg[0], cfg[1], max_seconds)
    return dt, {"it": it, "res": res}


def bench_config(world):
    """The workload description, identical in both arms (tuning choices are reported under "tuning")."""
    return {"workload": "dense truncated SVD 8192x2048, top 32 triplets, tol 1e-8",
            "l2_flush": "256 MB write between timed GPU solves (A is 134 MB in FP64)",
            "parallelism": "replicas" if world > 1 else "single GPU"}


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        return main_reference(args, rank, world)
    import torch

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from mixedprecisionofrr_gb300 import api

    if args.roofline_only and args.config == "c3":
        # the fused Krylov step alone on the 128^3 operator (FP64 basis, column 40, then FP16, column 40)
        from mixedprecisionofrr_gb300 import problems

        Acsr = api.CsrMatrix(problems.convdiff_3d(C3_N), symmetric=False)
        res = {}
        for prec, i in (("double", 40), ("half", 40)):
            us, by = api.profile_krylov_step(Acsr, prec, i, reps=5)
            res[f"{prec}_i{i}"] = {"us": us, "bytes": by, "GBps": by / us / 1e3}
        print(json.dumps({"roofline_only": True, "config": "c3", "k_kry_step": res}))
        return
    if args.roofline_only:
        dt_s, bytes_s = sliced_roofline(api)
        dt_g, bytes_g, flops_g = gemm_roofline(api)
        print(json.dumps({"roofline_only": True, "k_sliced_tn_us": dt_s * 1e6, "k_sliced_tn_GBps": bytes_s / dt_s / 1e9,
                          "k_gemm_tn_us": dt_g * 1e6, "k_gemm_tn_GBps": bytes_g / dt_g / 1e9}))
        return
    if args.kernel_gen:
        print(json.dumps(kernel_gen_run(api)))
        return
    if args.csr_load:
        print(json.dumps(csr_load_run(api)))
        return
    if args.config == "c3":
        if args.profile_solve:  # one mixed solve (for launch lists and captures)
            from mixedprecisionofrr_gb300 import problems

            Acsr = api.CsrMatrix(problems.convdiff_3d(C3_N), symmetric=False)
            X, d, info = c3_solve(api, Acsr, "mixed")
            torch.cuda.synchronize()
            print(json.dumps({"profile_solve": True, "config": "c3", "status": info.status, "cycles": info.iterations,
                              "matvecs": info.matvecs, "max_residual": info.max_residual}))
            return
        print(json.dumps(c3_run(api, args.steps, args.warmup)))
        return
    if args.config == "c4":
        print(json.dumps(c4_run(api, args.steps, args.warmup, cpu=not args.no_cpu_baseline, count=args.batch_count)))
        return
    if args.config == "c5":
        print(json.dumps(c5_run(api, args.requests, args.time_scale)))
        return
    A, s_true = make_problem_gpu()
    if args.orth_compare:
        print(json.dumps(orth_compare_run(api, A)))
        return
    if args.profile_solve:
        if args.mixed_config:
            CFG["mixed"] = tuple(int(x) for x in (args.mixed_config + ",0").split(",")[:3])
        run_solver(api, A, "mixed")
        torch.cuda.synchronize()
        U, s, V, info = run_solver(api, A, "mixed")
        torch.cuda.synchronize()
        print(json.dumps({"profile_solve": True, "status": info.status, "iterations": info.iterations,
                          "max_residual": info.max_residual}))
        return
    flush_buf = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    # block width and power steps per path from the solver autotuner (untimed; b >= 40)
    tune = {}
    for mode in ("mixed",) + (() if args.no_fp64 else ("fp64",)):
        if mode == "mixed" and args.mixed_config:
            b, st, st64 = (int(x) for x in (args.mixed_config + ",0").split(",")[:3])
            CFG[mode] = (b, st, st64)
            tune[mode] = {"block": b, "step_size": st, "step_size_f64": st64, "fixed": True}
            continue
        t = api.autotune_svd(A, M_ROWS, N_COLS, NEV, TOL, mode=mode, blocks=(64, 96, 128), steps=(4, 6, 8),
                             reps=1 if mode == "fp64" else 3, maxiter=MAXITER)
        CFG[mode] = (t["block"], t["step_size"], t["step_size_f64"])
        tune[mode] = {"block": t["block"], "step_size": t["step_size"], "step_size_f64": t["step_size_f64"],
                      "candidates": len(t["table"])}
        for row in t["table"]:
            print(f"autotune {mode}: {row}", file=sys.stderr)
    # mixed path (the product) -----------------------------------------------------------------
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        times, infos, launches, s = time_solves(api, A, "mixed", args.steps, args.warmup, flush_buf)
    if world > 1:
        total = max_over_ranks(float(times.sum()), world, "cuda")
    else:
        total = float(times.sum())
    value = job_value(args.steps, world, total)
    err = float(np.max(np.abs(s[:NEV] - s_true[:NEV]) / s_true[:NEV]))
    maxres = float(max(i.max_residual for i in infos))
    statuses = sorted({i.status for i in infos})
    iters = float(np.mean([i.iterations for i in infos]))
    out = None
    if rank == 0:
        # FP64 GPU comparison path
        fp64 = None
        if not args.no_fp64:
            k64 = max(1, min(2, args.steps))
            t64, inf64, _, s64 = time_solves(api, A, "fp64", k64, 1, flush_buf)
            fp64 = {"value": NEV * k64 / float(t64.sum()), "unit": UNIT, "ms_per_solve": 1e3 * float(t64.mean()),
                    "iterations": float(np.mean([i.iterations for i in inf64])),
                    "max_residual": float(max(i.max_residual for i in inf64))}
        # the FP8 (E4M3, per-column power-of-two scales) power-step variant on the same configuration
        t8, inf8, _, s8 = time_solves(api, A, "mixed", args.steps, 1, flush_buf, fp8=True)
        fp8 = {"value": NEV * args.steps / float(t8.sum()), "unit": UNIT, "ms_per_solve": 1e3 * float(t8.mean()),
               "iterations": float(np.mean([i.iterations for i in inf8])),
               "max_residual": float(max(i.max_residual for i in inf8)),
               "status": sorted({i.status for i in inf8}),
               "max_rel_sigma_err": float(np.max(np.abs(s8[:NEV] - s_true[:NEV]) / s_true[:NEV])),
               "dtype": "e4m3 power steps (per-column 2^e scales, FP32 accumulate), f16 basis / Gram, f64 pencil"}
        # end to end through the C ABI with host buffers
        A_host = torch.empty((N_COLS, M_ROWS), dtype=torch.float64).pin_memory()
        A_host.copy_(A.t())
        te, st_e, h2d, d2h, res_e = time_e2e(api, A_host, args.steps, 1)
        e2e = {"value": NEV * args.steps / float(te.sum()), "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "ms_per_step": 1e3 * float(te.mean()), "status": int(st_e),
               "max_residual": res_e}
        # roofline of the dominant kernel (live CUDA events): the fused exact-slice product of the FP64
        # refinement phase; the 16-bit tensor-core GEMM of the first phase is reported beside it
        peaks = {}
        pk = ROOT / "MEASURED_PEAKS.json"
        if pk.exists():
            peaks = json.loads(pk.read_text())
        hbm_peak = peaks.get("hbm_gbs", 6800.0)
        src = "measured" if "hbm_gbs" in peaks else "fallback"
        dt_s, bytes_s = sliced_roofline(api)
        bb = CFG["mixed"][0]
        roof = {"kernel": f"k_sliced_tn: exact-slice FP64 A.V, 8192x{bb} = (5-digit A' 2048x8192)' V", "bound": "hbm",
                "achieved": bytes_s / dt_s / 1e9, "peak": hbm_peak, "unit": "GB/s",
                "frac": bytes_s / dt_s / 1e9 / hbm_peak, "traffic": profiled_traffic() if bb == 64 else None,
                "algorithmic_bytes": bytes_s, "peak_source": src, "us_per_launch": dt_s * 1e6}
        # the same launch against the FP64 operands it stands for (A 8 B per element instead of its 10 B digit
        # stack, V and the FP64 result C once)
        fp64_bytes = 8.0 * (M_ROWS * N_COLS + N_COLS * bb + M_ROWS * bb)
        roof["frac_fp64_operand"] = fp64_bytes / dt_s / 1e9 / hbm_peak
        roof["fp64_operand_bytes"] = fp64_bytes
        dt_g, bytes_g, flops_g = gemm_roofline(api)
        roof16 = {"kernel": f"k_gemm_tn: A.V 16-bit TN GEMM 8192x2048x{bb} (FP32 accumulate, incl. split-K reduce)",
                  "bound": "hbm", "achieved": bytes_g / dt_g / 1e9, "peak": hbm_peak, "unit": "GB/s",
                  "frac": bytes_g / dt_g / 1e9 / hbm_peak,
                  "traffic": profiled_traffic("k_gemm_tn_av_8192x64x2048.md") if bb == 64 else None,
                  "algorithmic_bytes": bytes_g,
                  "peak_source": src, "us_per_launch": dt_g * 1e6, "tflops": flops_g / dt_g / 1e12}
        cpu = None
        cpu_tuning = None
        if not args.no_cpu_baseline:
            A_np = A.cpu().numpy()
            cpu_cfg, cpu_table = cpu_tune(A_np)
            cpu_tuning = {"block": cpu_cfg[0], "step_size": cpu_cfg[1], "table": cpu_table}
            dt_c, stc = cpu_baseline_run(A_np, cpu_cfg)
            cpu = {"value": NEV / dt_c if stc["res"] <= TOL else NEV / dt_c * 0.0, "unit": UNIT,
                   "cores": os.cpu_count(), "kind": "port",
                   "sample": f"one full FP64 NumPy/SciPy solve of the same workload (block {cpu_cfg[0]}, "
                             f"{cpu_cfg[1]} power steps, {stc['it']} outer iterations, "
                             f"max residual {stc['res']:.2e}, {dt_c:.1f} s)",
                   "seconds": dt_c}
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f16 basis / f32 accumulate / f64 pencil",
            "data": "synthetic (seeded Haar U, V; geometric s 1..1e-6)",
            "config": bench_config(world),
            "tuning": {"gpu_mixed": {"block": CFG["mixed"][0], "step_size": CFG["mixed"][1],
                                     "step_size_f64": CFG["mixed"][2]}, "gpu_autotune": tune,
                       "cpu": cpu_tuning},
            "p50_ms": 1e3 * float(np.percentile(times, 50)), "p99_ms": 1e3 * float(np.percentile(times, 99)),
            "iterations": iters, "max_residual": maxres, "max_rel_sigma_err": err, "status": statuses,
            "fp64_path": fp64,
            "speedup_vs_fp64": (value / fp64["value"]) if fp64 else None,
            "fp8_variant": fp8,
            "e2e": e2e, "gpu_launches": int(launches), "clocks": clk.summary(), "roofline": roof,
            "roofline_16bit_phase": roof16, "cpu_baseline": cpu,
            "c3": None if args.no_c3 else c3_run(api, min(args.steps, 2), 1, cpu=not args.no_cpu_baseline),
        }
        print(json.dumps(out))
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()


def main_reference(args, rank, world):
    """The reference's algorithm on the host cores: the NumPy/SciPy restatement (FP64), every thread."""
    if rank != 0:
        return
    from oracle import ofrr_oracle as orc

    A, U, s, V = orc.dense_svd_problem(M_ROWS, N_COLS, seed=42)
    cfg, table = cpu_tune(A)  # same rule as the other arm's cpu_baseline leg
    for _ in range(args.warmup):
        cpu_baseline_run(A, cfg, max_seconds=30.0)
    ts, its, ress = [], [], []
    for _ in range(args.steps):
        dt, st = cpu_baseline_run(A, cfg, max_seconds=60.0)
        ts.append(dt)
        its.append(st["it"])
        ress.append(st["res"])
    ts = np.array(ts)
    value = NEV * len(ts) / float(ts.sum())
    cpu = {"value": value, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
           "sample": f"full FP64 NumPy/SciPy solves of the workload (block {cfg[0]}, {cfg[1]} power steps, "
                     f"{int(np.mean(its))} outer iterations each, max residual {max(ress):.2e})"}
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * float(ts.mean()), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Haar U, V; geometric s 1..1e-6)",
        "config": bench_config(world),
        "tuning": {"cpu": {"block": cfg[0], "step_size": cfg[1], "table": table}},
        "p50_ms": 1e3 * float(np.percentile(ts, 50)), "p99_ms": 1e3 * float(np.percentile(ts, 99)),
        "cpu_baseline": cpu,
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


if __name__ == "__main__":
    main()
