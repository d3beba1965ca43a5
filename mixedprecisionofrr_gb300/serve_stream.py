"""Serving-stream driver: a seeded stream of mixed eigen/SVD requests with Poisson arrivals, fed to the
solve engine (ofrr_serve_*) as the requests arrive, with per-request latency (arrival to completion).

The stream (sizes and tolerances from the serving workload's description):
* arrivals: Poisson at `rate` requests/s (exponential inter-arrival times from the seed);
* 60 % dense SVD: m uniform in [512, 16384], n uniform in [m/8, m/4], singular values geometric from 1 to
  1e-6 (the matrix built on the GPU from Householder reflectors around diag(s): exact spectrum);
* 40 % Laplacian eigenproblems: 2D or 3D Dirichlet Laplacian (integer stencil) with n uniform in
  [1e4, 1e6], grid sides N, N+1 (, N+2) so that no eigenvalue is exactly repeated, largest eigenvalues
  by the thick-restart Krylov solver (Krylov dimension max(2k, k + 24), at most 127);
* k uniform in [4, 64], tol uniform over {1e-6, 1e-8, 1e-10}; mixed precision throughout; SVD requests
  run at most 400 outer iterations (6 power steps per 16-bit iteration, 12 per FP64 iteration),
  Laplacian requests LAP_STEP_BUDGET Krylov steps.

Admission: the engine's HBM budget (default 150 GB) charges each request's solver workspace; the replay
loop additionally holds back arrivals while the inputs it has placed on the GPU exceed `input_cap` bytes.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from . import api, problems


@dataclass
class Request:
    idx: int
    arrival: float  # seconds from the stream start
    kind: str       # "svd" or "lap"
    m: int
    n: int
    k: int
    tol: float
    dim: int = 0
    grid: tuple = ()
    seed: int = 0


def make_stream(seed: int, count: int, rate: float = 2000.0) -> list:
    """The first `count` requests of the seeded stream (request i does not depend on count)."""
    rng = np.random.default_rng(seed)
    out = []
    t_now = 0.0
    for i in range(count):
        t_now += float(rng.exponential(1.0 / rate))
        k = int(rng.integers(4, 65))
        tol = float(rng.choice([1e-6, 1e-8, 1e-10]))
        if rng.random() < 0.6:
            m = int(rng.integers(512, 16385))
            n = int(rng.integers(max(m // 8, 2 * k + 16), max(m // 4, 2 * k + 16) + 1))
            n = min(n, m)
            out.append(Request(i, t_now, "svd", m, n, min(k, n // 2), tol, seed=seed * 1000003 + i))
        else:
            dim = int(rng.choice([2, 3]))
            ntot = int(rng.integers(10_000, 1_000_001))
            if dim == 2:
                N = max(int(np.sqrt(ntot)), 8)
                grid = (N, N + 1)
            else:
                N = max(int(round(ntot ** (1.0 / 3.0))), 8)
                grid = (N, N + 1, N + 2)
            nn = int(np.prod(grid))
            out.append(Request(i, t_now, "lap", nn, nn, k, tol, dim=dim, grid=grid, seed=seed * 1000003 + i))
    return out


def laplacian_grid(grid: tuple):
    """Dirichlet Laplacian (integer stencil: 2 d on the diagonal, -1 per grid neighbour) on a rectangular
    grid of d sides, as a sorted CSR matrix (SciPy)."""
    import scipy.sparse as sp

    Ts = [sp.diags([-np.ones(N - 1), 2.0 * np.ones(N), -np.ones(N - 1)], [-1, 0, 1], format="csr") for N in grid]
    A = None
    for d, T in enumerate(Ts):
        term = T
        for e, N in enumerate(grid):
            if e == d:
                continue
            I = sp.identity(N, format="csr")
            term = sp.kron(term, I, format="csr") if e > d else sp.kron(I, term, format="csr")
        A = term if A is None else A + term
    A = sp.csr_matrix(A)
    A.sort_indices()
    return A


def svd_spectrum(n: int) -> np.ndarray:
    return 1e-6 ** (np.arange(n) / max(n - 1, 1))


@dataclass
class Submitted:
    req: Request
    ticket: int
    t_arrival: float
    t_submit: float
    input_bytes: int
    keep: tuple = field(default_factory=tuple)


def build_inputs(req: Request):
    """Device operator for a request (generated on the GPU for dense SVD, uploaded CSR for Laplacians)."""
    if req.kind == "svd":
        A = api.test_matrix_spectrum(svd_spectrum(req.n), req.m, req.n, seed=req.seed)
        return A, req.m * req.n * 8
    Acsr = api.CsrMatrix(laplacian_grid(req.grid), symmetric=True)
    return Acsr, Acsr.nnz * 18 + (req.n + 1) * 4


# Krylov steps allowed per Laplacian request: the clustered top of a large Laplacian's spectrum can take
# hundreds of thousands of steps to resolve; a request that has not converged within the budget
# completes with status 4001 (its best Ritz pairs and residuals are still returned)
LAP_STEP_BUDGET = 20_000


def submit(server: "api.Server", req: Request, A):
    if req.kind == "svd":
        return server.submit_si_svd(A, max(req.k + 16, int(1.5 * req.k)), mode="mixed", tol=req.tol, nev=req.k,
                                    maxiter=400, step_size=6, step_size_f64=12, seed=req.seed & 0xFFFFFFFF)
    kdim = min(max(2 * req.k, req.k + 24), 127)
    return server.submit_arnoldi_eig(A, req.k, kdim=kdim, mode="mixed", tol=req.tol, maxiter=LAP_STEP_BUDGET,
                                     seed=req.seed & 0xFFFFFFFF)


def run_stream(reqs: list, workers: int = 4, hbm_budget: float = 150e9, input_cap: float = 60e9,
               time_scale: float = 1.0) -> dict:
    """Replays the stream in real time (arrival times scaled by time_scale) through the engine; returns
    latency percentiles, throughput and per-request records."""
    import torch

    server = api.Server(workers=workers, hbm_budget_bytes=int(hbm_budget))
    live = []
    recs = []
    in_flight_bytes = 0
    t0 = time.perf_counter()

    def drain(block: bool):
        nonlocal in_flight_bytes
        still = []
        for s in live:
            done, st = server.poll(s.ticket)
            if done or block:
                status, lat, keep = server.wait(s.ticket)
                t_done = time.perf_counter() - t0
                inf = keep[-1]
                vals = np.array(keep[-3], copy=True)  # singular / eigenvalues of the request
                recs.append({"idx": s.req.idx, "kind": s.req.kind, "m": s.req.m, "n": s.req.n, "k": s.req.k,
                             "tol": s.req.tol, "status": status, "arrival": s.t_arrival, "submit": s.t_submit,
                             "done": t_done, "latency_ms": 1e3 * (t_done - s.t_arrival),
                             "solve_ms": lat, "converged": int(inf.converged),
                             "max_residual": float(inf.max_residual), "values": vals})
                in_flight_bytes -= s.input_bytes
            else:
                still.append(s)
        live[:] = still

    for req in reqs:
        target = req.arrival * time_scale
        while True:
            now = time.perf_counter() - t0
            drain(False)
            if now >= target and in_flight_bytes < input_cap:
                break
            time.sleep(min(0.002, max(target - now, 0.0005)))
        A, nbytes = build_inputs(req)
        torch.cuda.current_stream().synchronize()
        ticket = submit(server, req, A)
        live.append(Submitted(req, ticket, target, time.perf_counter() - t0, nbytes, (A,)))
        in_flight_bytes += nbytes
    while live:
        drain(False)
        time.sleep(0.002)
    wall = time.perf_counter() - t0
    stats = server.stats()
    server.close()
    lat = np.array([r["latency_ms"] for r in recs])
    ok = [r for r in recs if r["status"] == 0]
    return {"requests": len(recs), "completed_ok": len(ok), "wall_s": wall,
            "offered_rate": len(reqs) / max(reqs[-1].arrival * time_scale, 1e-9) if reqs else 0.0,
            "throughput_req_s": len(recs) / wall,
            "converged_pairs_per_s": sum(r["converged"] for r in recs) / wall,
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "engine": {k: stats[k] for k in ("completed", "failed", "budget_bytes", "busy_ms")},
            "records": recs}


def solve_alone(req: Request):
    """The same request solved on its own (fresh engine, one worker): the reference for the parity check."""
    server = api.Server(workers=1)
    A, _ = build_inputs(req)
    t = submit(server, req, A)
    status, lat, keep = server.wait(t)
    server.close()
    return status, keep
