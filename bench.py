#!/usr/bin/env python
"""Benchmark of the LOBPCG hot path on GB300 (one JSON line on stdout).

Workload (default, --config c3m): time to k eigenpairs at residual 1e-8 of
the matrix-free variable-coefficient 7-point stencil (faces exp(N(0,1)),
seed 2), k = 64, X0 = 2*drand48()-1 from seed 2, preconditioner 20
Jacobi-CG steps on A, in mixed precision with the plain FP64 GPU path
beside: timed as whole solves at 128^3 (n = 2,097,152), and the 256^3 case
(n = 16,777,216) solved once per arm beside it (`full_size`), each with its
eigenvalue error and largest subspace angle against the FP64 arm.  One
step = one full lobpcg_solve_double call from X0 to exit.  Synthetic data
from the seeded builders in blopex_gb300/problems.py.  Other workloads:
--config c2 (CSR Laplacian 128^3, k = 32, Jacobi, maxit 300), c4 (2D
diffusion forward + gradient), c5 (generalized 27-point 100^3, k = 128,
forward + gradient), c1 (20^3).

value  = seconds per solve with X0, the operator and the preconditioner
         resident in HBM (max over ranks), CUDA events on the solver stream;
e2e    = the same through the C ABI with X0 uploaded from pinned host memory
         and the Ritz vectors + eigenvalues read back, every step;
roofline = the kernel class with the largest share of the timed region,
         from the library's CUDA-event timers (algorithmic bytes per launch /
         event-timed duration), against MEASURED_PEAKS.json;
cpu_baseline = the C restatement of the reference (oracle/, scalar loops,
         one core) on a bounded sample, scaled to the full workload;
adjoint = the c4 derivative configuration (2D diffusion 512^2, forward solve
         + reverse-mode gradient) measured once beside the headline: forward
         and backward times and their ratio (--no-adjoint skips it).

--impl reference times that CPU implementation alone (the reference's own
algorithm on one host core, its LAPACK calls single-threaded; the compiled
reference itself is not available on the GPU host).  Under torchrun each
rank runs an independent replica (the solver does not shard: replicas only).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

if "--impl" in sys.argv and "reference" in sys.argv:
    # the reference is single-threaded: its LAPACK calls too (set before the
    # BLAS library loads)
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CONFIGS = {
    "c1": dict(kind="csr", grid=(20, 20, 20), k=10, seed=0, tol=1e-6, maxit=100, jacobi=False,
               label="3D 7-point Laplacian 20^3 CSR, k=10, no preconditioner, tol 1e-6, maxit 100"),
    "c2": dict(kind="csr", grid=(128, 128, 128), k=32, seed=1, tol=1e-8, maxit=300, jacobi=True,
               label="3D 7-point Laplacian 128^3 CSR (n=2097152), k=32, Jacobi, tol 1e-8, maxit 300"),
    # differentiation: forward solve + reverse-mode gradient in theta
    "c4": dict(kind="adjoint5", grid=(512, 512), k=8, seed=3, tol=1e-8, maxit=3000,
               jacobi=True, adjoint_tol=1e-8, inner_cg=20,
               label="2D 5-point diffusion 512^2, c = exp(theta), theta GRF (length 0.1, seed 3), "
                     "k=8, loss = sum(lambda) + (x_1'v)^2, d loss / d theta; FP64, tol 1e-8, "
                     "preconditioner 20 Jacobi-CG steps on A"),
    # generalized problem with gradients in the A weights and the B diagonal
    "c5": dict(kind="gen27", grid=(100, 100, 100), k=128, seed=4, mass_seed=14, shift=0.5,
               tol=1e-8, maxit=1000, inner_cg=20, adjoint_tol=1e-8,
               label="generalized A x = lambda B x: 27-point graph Laplacian 100^3 (n=1000000), "
                     "edge weights U[0.5,1.5] seed 4, shift 0.5; B = diag(U[0.5,1.5] seed 14); "
                     "k=128, mixed precision, tol 1e-8, preconditioner 20 Jacobi-CG steps on A; "
                     "loss = sum(lambda) + (x_1'v)^2, gradient w.r.t. the 13 n edge weights and "
                     "the n entries of B"),
    # the metric's own configuration: time to k eigenpairs at residual 1e-8,
    # mixed precision against the plain FP64 GPU path
    "c3": dict(kind="stencil7", grid=(256, 256, 256), k=64, seed=2, tol=1e-8, maxit=1000,
               jacobi=True, precond="pcg20", fp64_iterations=565,
               label="matrix-free variable-coefficient 7-point stencil 256^3 (n=16777216), face "
                     "coefficients exp(N(0,1)) seed 2, k=64, X0 drand48 seed 2, tol 1e-8, "
                     "preconditioner 20 Jacobi-CG steps on A"),
    # the same operator family at 128^3: a full solve takes seconds, so it can
    # be repeated as the timed step; the 256^3 case runs once beside it
    "c3m": dict(kind="stencil7", grid=(128, 128, 128), k=64, seed=2, tol=1e-8, maxit=1000,
                jacobi=True, precond="pcg20", full="c3", fp64_iterations=176, adjoint="c4",
                label="matrix-free variable-coefficient 7-point stencil 128^3 (n=2097152), face "
                      "coefficients exp(N(0,1)) seed 2, k=64, X0 drand48 seed 2, tol 1e-8, "
                      "preconditioner 20 Jacobi-CG steps on A"),
}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return p, "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax = float(parts[2])
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def fp64_peak_tflops(torch, n: int = 8192) -> float:
    """FP64 GEMM throughput of this GPU (torch.matmul float64, best of 3,
    CUDA events): the roof of the FP64 kernels, absent from the measured
    peaks file."""
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    best = None
    for _ in range(3):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) / 1e3
        best = t if best is None else min(best, t)
    del a, b
    torch.cuda.empty_cache()
    return 2.0 * n ** 3 / best / 1e12


# kernel classes whose arithmetic is FP64 in the FP64 path
FP64_CLASSES = {"gram", "xc_update", "spmm_csr", "stencil7", "stencil5", "stencil27",
                "diag_scale", "residual", "blas1"}


def nested(name):
    """Timer classes recorded inside another one: the Rayleigh-Ritz stages
    (rr_*) and the gate of its fallback run within the sygv class's record."""
    return name.startswith("rr_") or name == "sygv_fp64_gate"


def top_level_ms(kt):
    """Summed event time of the classes that are not nested in another."""
    return sum(v["ms"] for nm, v in kt.items() if not nested(nm)) or 1.0


def roofline_entry(name, v, hbm_peak, fp64_peak, traffic, fp64_arith=True, tf32_peak=None):
    """Bound = whichever of HBM bytes / HBM peak and flops / compute peak is
    longer (FP64 pipe for the FP64 classes, TF32 tensor rate for the tcgen05
    classes); achieved = algorithmic bytes or flops per launch / event-timed
    launch duration."""
    sec = v["ms"] / 1e3
    t_mem = v["bytes"] / (hbm_peak * 1e9)
    t_fp = v["flops"] / (fp64_peak * 1e12) if (fp64_arith and name in FP64_CLASSES) else 0.0
    t_tc = v["flops"] / (tf32_peak * 1e12) if (tf32_peak and name.startswith("tc_")) else 0.0
    tr = traffic.get(name)
    if t_fp > t_mem:
        ach = v["flops"] / sec / 1e12
        out = {"kernel": name, "bound": "fp64", "achieved": ach, "peak": fp64_peak,
               "unit": "TFLOP/s", "frac": ach / fp64_peak,
               "peak_kind": "measured in this run (torch.matmul float64 8192^3)"}
    elif t_tc > t_mem:
        ach = v["flops"] / sec / 1e12
        out = {"kernel": name, "bound": "tensor", "achieved": ach, "peak": tf32_peak,
               "unit": "TFLOP/s", "frac": ach / tf32_peak,
               "peak_kind": "dense TF32 = half the measured bf16 burst rate"}
    else:
        ach = v["bytes"] / sec / 1e9
        out = {"kernel": name, "bound": "hbm", "achieved": ach, "peak": hbm_peak, "unit": "GB/s",
               "frac": ach / hbm_peak}
    out.update({"traffic": tr["bytes_per_launch"] if tr else None,
                "algorithmic_bytes_per_launch": v["bytes"] / v["launches"],
                "algorithmic_flops_per_launch": v["flops"] / v["launches"],
                "launches": v["launches"], "avg_launch_ms": v["ms"] / v["launches"]})
    return out


def load_traffic(config: str):
    """DRAM bytes per launch of a kernel class on this workload, from the
    committed ncu summary (profiles/traffic.json); entries name the workload
    they were captured on."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            entries = json.load(f)
    except (OSError, ValueError):
        return {}
    return {k: v for k, v in entries.items() if v.get("config") == config}


def build_problem(cfg, grid=None):
    """(n, operator description, host X0 or None, Jacobi diagonal or None).
    X0 = 2*drand48()-1 from the config's seed; for the large stencil case it
    is generated on the device (bit-identical) instead of on the host."""
    from blopex_gb300 import problems as P
    nx, ny, nz = grid or cfg["grid"]
    n = nx * ny * nz
    if cfg["kind"] == "csr":
        op = ("csr", P.laplacian3d_csr(nx, ny, nz))
        diag = P.csr_diagonal(*op[1])
    else:
        cx, cy, cz = P.stencil7_coefficients(nx, ny, nz, seed=cfg["seed"])
        op = ("stencil7", (cx, cy, cz))
        diag = P.stencil7_diagonal(cx, cy, cz)
    x0 = P.drand48_block(n, cfg["k"], cfg["seed"]) if n * cfg["k"] <= (1 << 27) else None
    tdiag = 1.0 / diag if cfg["jacobi"] else None
    return n, op, x0, tdiag


def cpu_baseline(cfg, iterations=None, sample_grid=32):
    """The oracle (C restatement of the reference, scalar loops, one core):
    for a small configuration (n <= 100,000) the whole solve as configured,
    measured; otherwise a bounded sample: a 32^3 grid (24^3 for the
    reference arm) with the same k, 1 and 3 iterations; the per-iteration time is scaled by n
    (the work per iteration is linear in n at fixed k) to the full grid and
    multiplied by the iteration count of the FP64 GPU path on the workload
    (the same algorithm: iteration counts agree within 2 where parity is
    pinned), or by the configuration's recorded count.  Extrapolated: a full
    CPU solve of the 256^3 case would take days.  The preconditioner is the
    configuration's: Jacobi, or the inner CG (HYPRE's -pcgitr) on the
    sample's operator with Jacobi inside."""
    from blopex_gb300 import problems as P
    from oracle import oracle as O
    O.build(ref=False)
    nx, ny, nz = cfg["grid"]
    n_full = nx * ny * nz
    if n_full <= 100_000:
        # small enough for the whole solve, as configured, in a second or so
        n, op, x0, tdiag = build_problem(cfg)
        csr = op[1] if op[0] == "csr" else P.stencil7_to_csr(*op[1])
        A = O.csr(*csr)
        T = O.diag(tdiag) if tdiag is not None else O.NONE
        t0 = time.perf_counter()
        r = O.solve(A, x0, T=T, atol=cfg["tol"], maxit=cfg["maxit"], history=False)
        secs = time.perf_counter() - t0
        return {"value": secs, "unit": "s", "cores": 1, "host_cores": os.cpu_count(),
                "kind": "port",
                "sample": f"oracle C restatement, the whole solve ({r.iterations} iterations, "
                          f"exit flag {r.flag}), measured", "iterations_assumed": r.iterations,
                "measured_s": secs, "extrapolated": False}
    s = min(sample_grid, nx)
    n, op, x0, tdiag = build_problem(dict(cfg, jacobi=True), (s, s, s))
    csr = op[1] if op[0] == "csr" else P.stencil7_to_csr(*op[1])
    A = O.csr(*csr)
    T = O.diag(tdiag)
    precond = cfg.get("precond", "")
    if precond.startswith("pcg"):
        T = O.pcg(A, T, int(precond[3:]))
    t0 = time.perf_counter()
    O.solve(A, x0, T=T, atol=cfg["tol"], maxit=1, history=False)
    t1 = time.perf_counter()
    O.solve(A, x0, T=T, atol=cfg["tol"], maxit=3, history=False)
    t2 = time.perf_counter()
    per_it = max((t2 - t1) - (t1 - t0), 1e-9) / 2.0
    setup = max((t1 - t0) - per_it, 0.0)
    scale = n_full / n
    its = iterations or cfg.get("fp64_iterations") or cfg["maxit"]
    value = (setup + its * per_it) * scale
    return {"value": value, "unit": "s", "cores": 1, "host_cores": os.cpu_count(),
            "kind": "port",
            "sample": f"oracle C restatement, {s}^3 grid k={cfg['k']} "
                      f"{'inner CG ' + precond[3:] + ' steps' if precond.startswith('pcg') else 'Jacobi'}, "
                      f"1 and 3 iterations "
                      f"({t2 - t0:.1f} s measured), per-iteration {per_it:.3f} s scaled by n "
                      f"x{scale:.0f} and to {its} iterations (extrapolated)",
            "per_iteration_s_full_n": per_it * scale, "iterations_assumed": its,
            "measured_s": t2 - t0, "extrapolated": True}


def run_adjoint(args, cfg):
    """--config c4: forward LOBPCG solve and reverse-mode gradient of the
    loss through the adjoint module.  value = forward + backward ms per step
    (device-resident coefficients and blocks, CUDA events on the solver
    stream); e2e = the torch.autograd path from a host theta to host
    d loss / d theta."""
    import torch
    world, rank, local, dist = dist_setup()
    torch.cuda.set_device(local)
    line = measure_adjoint(cfg, args.steps, args.warmup, world, local, dist)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def measure_adjoint(cfg, steps, warmup, world, local, dist):
    """The adjoint configuration's measurement (its JSON line as a dict):
    `warmup` untimed forward + backward steps, then `steps` timed ones."""
    import torch
    from blopex_gb300 import adjoint as AD
    from blopex_gb300 import problems as P
    from blopex_gb300 import solver as S
    nx, ny = cfg["grid"]
    n, k = nx * ny, cfg["k"]
    theta = 0.5 * P.gaussian_random_field(nx, ny, 0.1, cfg["seed"])
    cx, cy = P.stencil5_from_cells(np.exp(theta))
    v = np.random.default_rng(cfg["seed"]).standard_normal(n)
    v /= np.linalg.norm(v)
    ctx = S.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", local))
    A = S.Stencil5(ctx, cx, cy)
    J = S.Diagonal(ctx, 1.0 / A.diagonal())
    T = S.PCGPreconditioner(ctx, A, J, cfg["inner_cg"])
    X = S.MultiVector(ctx, n, k)
    ctx.set_options(precision=S.FP64)
    glam = np.ones(k)

    def forward():
        X.set_random(1)
        return S.lobpcg_solve_double(X, A, T=T, atol=cfg["tol"], rtol=1e-50, maxit=cfg["maxit"],
                                     history=False)

    def backward(r):
        x1 = X.to_host()[:, 0]
        G = np.zeros((n, k), order="F")
        G[:, 0] = 2.0 * (x1 @ v) * v
        adj = AD.eigenvector_adjoint(X, r.lam, A, G=G, glam=glam, T=T, tol=cfg["adjoint_tol"],
                                     maxit=20000)
        return adj, AD.operator_gradient(A, X, adj.W)

    def timed(f, *a):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        out = f(*a)
        e1.record(stream)
        torch.cuda.synchronize()
        return out, e0.elapsed_time(e1)

    for _ in range(warmup):
        backward(forward())
    ctx.profiling(True)
    ctx.reset_kernel_times()
    sampler = ClockSampler(local)
    if dist is not None:
        dist.barrier()
    sampler.start()
    launches0 = ctx.lib.gpu_KernelLaunchCount()
    fwd, bwd, its, aits, res = [], [], 0, 0, 0.0
    for _ in range(steps):
        r, tf = timed(forward)
        (adj, g), tb = timed(backward, r)
        fwd.append(tf)
        bwd.append(tb)
        its, aits, res = r.iterations, adj.iterations, adj.max_rel_residual
    launches = ctx.lib.gpu_KernelLaunchCount() - launches0
    clocks = sampler.stop()
    kt = ctx.kernel_times()
    ctx.profiling(False)
    tf = max_over_ranks(statistics.median(fwd), dist, "cuda")
    tb = max_over_ranks(statistics.median(bwd), dist, "cuda")

    # e2e: host theta -> torch autograd -> host gradient, every step
    opts = AD.SolveOptions(k=k, atol=cfg["tol"], maxit=cfg["maxit"], adjoint_tol=cfg["adjoint_tol"],
                           adjoint_maxit=20000, inner_cg=cfg["inner_cg"])
    vt = torch.from_numpy(v)
    e2e = []
    for _ in range(max(1, steps)):
        th = torch.from_numpy(theta).requires_grad_(True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        c = torch.exp(th)
        fx, fy = AD.stencil5_faces_torch(c)
        lam, Xh = AD.Stencil5Eigs.apply(fx, fy, ctx, opts)
        loss = lam.sum() + (Xh[:, 0] @ vt) ** 2
        (gt,) = torch.autograd.grad(loss, th)
        e2e.append((time.perf_counter() - t0) * 1e3)
    pk, _ = peaks()
    total = top_level_ms(kt)
    e2e_ms = max_over_ranks(statistics.median(e2e), dist, "cuda")
    line = {"metric": "fwd+bwd ms (forward solve + reverse-mode gradient)", "value": tf + tb,
            "unit": "ms", "n_gpus": world, "steps": steps, "warmup": warmup,
            "ms_per_step": tf + tb, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": cfg["label"], "n": n, "k": k, "tol": cfg["tol"],
                       "adjoint_tol": cfg["adjoint_tol"], "parallelism": "replicas",
                       "l2": "inputs smaller than L2 (n*k*8 = 16.8 MB)"},
            "forward_ms": tf, "backward_ms": tb, "fwd_plus_bwd_over_fwd": (tf + tb) / tf,
            "lobpcg_iterations": its, "adjoint_cg_iterations": aits,
            "adjoint_max_rel_residual": res,
            "kernels": {nm: {"share": x["ms"] / total, "launches": x["launches"],
                             "avg_ms": x["ms"] / x["launches"]}
                        for nm, x in sorted(kt.items(), key=lambda kv: -kv[1]["ms"])[:8]},
            "e2e": {"value": e2e_ms, "unit": "ms",
                    "h2d_bytes_per_step": 8 * (cx.size + cy.size),
                    "d2h_bytes_per_step": 8 * (n * k + k + cx.size + cy.size)},
            "gpu_launches": int(launches), "clocks": clocks,
            "roofline": None}
    return line


def run_generalized(args, cfg):
    """--config c5: forward solve of the generalized problem in mixed
    precision and in FP64 (same X0), then the reverse-mode gradient of the
    loss w.r.t. the A edge weights and the B diagonal through the adjoint
    module, from the mixed result.  value = mixed forward + backward ms; the
    FP64 forward, the eigenvalue error and the largest B-subspace angle of
    the mixed eigenvectors against the FP64 ones are reported beside."""
    import torch
    from blopex_gb300 import adjoint as AD
    from blopex_gb300 import problems as P
    from blopex_gb300 import solver as S
    world, rank, local, dist = dist_setup()
    torch.cuda.set_device(local)
    nx, ny, nz = cfg["grid"]
    n, k = nx * ny * nz, cfg["k"]
    w = P.stencil27_weights(nx, ny, nz, seed=cfg["seed"])
    bdiag = P.mass_diagonal(n, seed=cfg["mass_seed"])
    v = np.random.default_rng(cfg["seed"]).standard_normal(n)
    v /= np.linalg.norm(v)
    ctx = S.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", local))
    A = S.Stencil27(ctx, nx, ny, nz, w, cfg["shift"])
    B = S.Diagonal(ctx, bdiag)
    J = S.Diagonal(ctx, 1.0 / A.diagonal())
    T = S.PCGPreconditioner(ctx, A, J, cfg["inner_cg"])
    glam = np.ones(k)
    maxit = args.maxit or cfg["maxit"]

    def timed(f, *a):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        out = f(*a)
        e1.record(stream)
        torch.cuda.synchronize()
        return out, e0.elapsed_time(e1)

    def forward(X, mode):
        X.set_random(cfg["seed"])
        ctx.set_options(precision=S.MIXED if mode == "mixed" else S.FP64)
        return S.lobpcg_solve_double(X, A, B=B, T=T, atol=cfg["tol"], rtol=1e-50, maxit=maxit,
                                     history=False)

    def forward_restarting(X, mode):
        """The plain algorithm breaks down on this problem near the tolerance
        (its B-Gram stops being definite: dsygv fails, exit -1, in the
        reference as here): restart from the current block, as the
        reference's callers do, up to maxit iterations in all."""
        r = forward(X, mode)
        its, restarts = r.iterations, 0
        while r.flag == -1 and its < maxit and restarts < 20:
            r = S.lobpcg_solve_double(X, A, B=B, T=T, atol=cfg["tol"], rtol=1e-50,
                                      maxit=maxit - its, history=False)
            its += r.iterations
            restarts += 1
        r.iterations = its
        return r, restarts

    def true_residual(X, lam):
        """max_i ||A x_i - lambda_i B x_i|| from fresh operator applications
        (the solver's own norms use the implicitly updated A X and B X)."""
        AXb, BXb = S.MultiVector(ctx, n, k), S.MultiVector(ctx, n, k)
        A.apply(X, AXb)
        B.apply(X, BXb)
        res = np.linalg.norm(AXb.to_host() - BXb.to_host() * lam[None, :], axis=0)
        AXb.close()
        BXb.close()
        return float(np.max(res))

    def backward(X, r):
        x1 = X.to_host()[:, 0]
        G = np.zeros((n, k), order="F")
        G[:, 0] = 2.0 * (x1 @ v) * v
        adj = AD.eigenvector_adjoint(X, r.lam, A, G=G, glam=glam, B=B, T=T,
                                     tol=cfg["adjoint_tol"], maxit=20000)
        return adj, AD.operator_gradient(A, X, adj.W), AD.mass_gradient(B, X, adj.W, r.lam, adj.xg)

    Xm, Xf = S.MultiVector(ctx, n, k), S.MultiVector(ctx, n, k)
    for _ in range(args.warmup):
        forward(Xm, "mixed")
    ctx.profiling(True)
    ctx.reset_kernel_times()
    sampler = ClockSampler(local)
    if dist is not None:
        dist.barrier()
    sampler.start()
    launches0 = ctx.lib.gpu_KernelLaunchCount()
    fwd, bwd = [], []
    for _ in range(args.steps):
        rm, tf = timed(forward, Xm, "mixed")
        st_m = dict(rm.stats)
        (adj, ga, gb), tb = timed(backward, Xm, rm)
        fwd.append(tf)
        bwd.append(tb)
    launches = ctx.lib.gpu_KernelLaunchCount() - launches0
    clocks = sampler.stop()
    kt = ctx.kernel_times()
    ctx.profiling(False)
    (rf, restarts), tf64 = timed(forward_restarting, Xf, "fp64")
    true_res = {"mixed": true_residual(Xm, rm.lam), "fp64": true_residual(Xf, rf.lam)}
    # eigenvalue error and the largest principal angle in the B inner product
    xm, xf = Xm.to_host(), Xf.to_host()
    d = xm - xf @ (xf.T @ (bdiag[:, None] * xm))
    dd = d.T @ (bdiag[:, None] * d)
    sin_max = float(np.sqrt(max(np.linalg.eigvalsh(0.5 * (dd + dd.T))[-1], 0.0)))
    xbx = xm.T @ (bdiag[:, None] * xm)
    tf_ = max_over_ranks(statistics.median(fwd), dist, "cuda")
    tb_ = max_over_ranks(statistics.median(bwd), dist, "cuda")
    total = top_level_ms(kt)
    line = {"metric": "fwd+bwd ms (mixed-precision generalized solve + reverse-mode gradient)",
            "value": tf_ + tb_, "unit": "ms", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": tf_ + tb_, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32/f64 mixed", "data": "synthetic",
            "config": {"workload": cfg["label"], "n": n, "k": k, "tol": cfg["tol"],
                       "maxit": maxit, "adjoint_tol": cfg["adjoint_tol"],
                       "parallelism": "replicas",
                       "l2": "inputs larger than L2 (X alone is n*k*8 = 1.02 GB)"},
            "forward_ms": tf_, "backward_ms": tb_, "fwd_plus_bwd_over_fwd": (tf_ + tb_) / tf_,
            "mixed": arm_summary(rm, tf_ / 1e3) | {"stats": {
                kk: st_m[kk] for kk in ("iterations_fp32", "iterations_fp64", "handover_reason",
                                        "explicit_undos", "explicit_p_drops")}},
            "fp64": arm_summary(rf, tf64 / 1e3) | {"restarts_after_breakdown": restarts},
            "max_true_residual": true_res,
            "mixed_over_fp64_forward_speedup": tf64 / tf_,
            "max_rel_lambda_error_vs_fp64": float(np.max(np.abs(rm.lam - rf.lam) / np.abs(rf.lam))),
            "largest_subspace_angle_rad": float(np.arcsin(min(sin_max, 1.0))),
            "orthonormality_xtbx_minus_i_fro": float(np.linalg.norm(xbx - np.eye(k))),
            "adjoint_cg_iterations": adj.iterations,
            "adjoint_max_rel_residual": adj.max_rel_residual,
            "gradient_norms": {"a_weights": float(np.linalg.norm(ga)),
                               "b_diagonal": float(np.linalg.norm(gb))},
            "kernels": {nm: {"share": x["ms"] / total, "launches": x["launches"],
                             "avg_ms": x["ms"] / x["launches"]}
                        for nm, x in sorted(kt.items(), key=lambda kv: -kv[1]["ms"])[:10]},
            "gpu_launches": int(launches), "clocks": clocks, "roofline": None}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def run_reference(args, cfg):
    """--impl reference: the CPU implementation of the path timed alone."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    try:  # one core, as the reference runs
        os.sched_setaffinity(0, {min(os.sched_getaffinity(0))})
    except (AttributeError, OSError):
        pass
    for _ in range(args.warmup):
        cpu_baseline(cfg, sample_grid=24)
    vals = [cpu_baseline(cfg, sample_grid=24) for _ in range(args.steps)]  # each a bounded sample
    v = statistics.median(x["value"] for x in vals)
    # ms_per_step is the wall time of one timed step (the sample the CPU
    # actually ran); value is the full solve that sample stands for
    measured = statistics.median(x["measured_s"] for x in vals)
    cb = dict(vals[0])
    cb["value"] = v
    line = {"impl": "reference", "metric": metric_name(cfg, None, args.mode), "value": v, "unit": "s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": measured * 1e3, "value_extrapolated": cb["extrapolated"],
            "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": dict(config_block(cfg, args, args.precond or cfg.get("precond", "")),
                           mode="reference (FP64, one core)"),
            "cpu_baseline": cb,
            "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def dist_setup(backend: str = "nccl"):
    """(world, rank, local rank, torch.distributed or None) from the torchrun
    environment; a process group only when there is more than one rank."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group(backend)
    return world, rank, local, dist


def max_over_ranks(value: float, dist, device) -> float:
    """The largest of the ranks' values, on every rank (the job's time with one
    replica per rank); the value itself without a process group."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def metric_name(cfg, res=None, mode="mixed"):
    """The metric as measured: time to k eigenpairs at the configuration's
    residual tolerance -- or, when the timed solve ended without reaching it,
    time to maxit with the residual it reached."""
    arm = "mixed precision; plain FP64 GPU path beside" if mode == "mixed" else \
        "plain FP64 GPU path; mixed precision beside"
    if res is not None and res.flag != 0:
        return (f"time to maxit={res.iterations} WITHOUT reaching resid {cfg['tol']:g} "
                f"(max resid {float(np.max(res.res)):.2e}; {arm})")
    return f"time to k eigenpairs at resid {cfg['tol']:g} ({arm})"


def config_block(cfg, args, precond=""):
    return {"workload": cfg["label"] if precond == cfg.get("precond", "") else
            cfg["label"] + (f" [preconditioner: {precond[3:]} inner CG steps]" if precond
                            else " [preconditioner: Jacobi]"),
            "mode": args.mode, "n": int(np.prod(cfg["grid"])),
            "k": cfg["k"], "maxit": args.maxit or cfg["maxit"], "tol": cfg["tol"],
            "l2": "inputs larger than L2 (X alone is n*k*8 bytes)" if np.prod(cfg["grid"]) *
                  cfg["k"] * 8 > 129e6 else "inputs smaller than L2", "parallelism":
            "replicas"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="c3m", choices=sorted(CONFIGS))
    ap.add_argument("--mode", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--maxit", type=int, default=0, help="override maxit (exploration only)")
    ap.add_argument("--precond", default="",
                    help="'pcgN': precondition with N inner CG steps (Jacobi inside) instead of "
                         "Jacobi alone")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end repetition")
    ap.add_argument("--grid", type=int, default=0,
                    help="override the grid edge (small cases for profiling only)")
    ap.add_argument("--no-full", action="store_true",
                    help="skip the once-measured full-size comparison (config key 'full')")
    ap.add_argument("--no-other-arm", action="store_true",
                    help="skip the other precision's arm (FP64 beside mixed or the reverse)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--no-adjoint", action="store_true",
                    help="skip the derivative configuration measured beside the headline")
    args = ap.parse_args()
    cfg = dict(CONFIGS[args.config])
    if args.maxit:
        cfg["maxit"] = args.maxit
    if args.grid:
        cfg["grid"] = (args.grid,) * 3
        cfg["label"] += f" [profiling case: grid {args.grid}^3]"

    if args.impl == "reference":
        if cfg["kind"] in ("adjoint5", "gen27"):
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no "
                              "derivatives (no adjoint or gradient of its eigenpairs)"}), flush=True)
            return
        run_reference(args, cfg)
        return
    if cfg["kind"] == "adjoint5":
        run_adjoint(args, cfg)
        return
    if cfg["kind"] == "gen27":
        run_generalized(args, cfg)
        return

    import torch
    world, rank, local, dist = dist_setup()
    torch.cuda.set_device(local)

    from blopex_gb300 import solver as S

    def barrier():
        if dist is not None:
            dist.barrier()

    n, op, x0, tdiag = build_problem(cfg)
    k = cfg["k"]
    ctx = S.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", local))
    A = S.CSRMatrix(ctx, *op[1]) if op[0] == "csr" else S.Stencil7(ctx, *op[1])
    T = S.Diagonal(ctx, tdiag) if tdiag is not None else None
    precond = args.precond or cfg.get("precond", "")
    if precond.startswith("pcg"):
        T = S.PCGPreconditioner(ctx, A, T, int(precond[3:]))
    X = S.MultiVector(ctx, n, k)
    if x0 is not None:
        X0 = S.MultiVector.from_host(ctx, x0)
    else:
        X0 = S.MultiVector(ctx, n, k)
        X0.set_random(cfg["seed"])

    def solve(mode, maxit=None, into=None):
        ctx.set_options(precision=S.FP64 if mode == "fp64" else S.MIXED)
        Xs = into or X
        Xs.copy_from(X0)
        return S.lobpcg_solve_double(Xs, A, T=T, atol=cfg["tol"], rtol=1e-50,
                                     maxit=maxit or cfg["maxit"], history=False)

    for _ in range(args.warmup):
        solve(args.mode)

    ctx.profiling(True)
    ctx.reset_kernel_times()
    sampler = ClockSampler(local)
    barrier()
    torch.cuda.synchronize()
    sampler.start()
    launches0 = ctx.lib.gpu_KernelLaunchCount()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    results = [solve(args.mode) for _ in range(args.steps)]
    ev1.record(stream)
    torch.cuda.synchronize()
    launches = ctx.lib.gpu_KernelLaunchCount() - launches0
    clocks = sampler.stop()
    barrier()
    ktimes = ctx.kernel_times()
    ctx.profiling(False)
    secs = max_over_ranks(ev0.elapsed_time(ev1) / 1e3 / args.steps, dist, "cuda")
    res = results[-1]
    stats = res.stats

    # e2e: X0 from pinned host memory, Ritz vectors back, every step, through
    # lobpcg_solve_double
    e2e = None
    if not args.no_e2e:
        if x0 is not None:
            pinned_in = torch.from_numpy(np.asfortranarray(x0).ravel(order="F")).pin_memory()
        else:
            pinned_in = torch.empty(n * k, dtype=torch.float64).pin_memory()
            X0.download_ptr(pinned_in.data_ptr(), n)
        pinned_out = torch.empty(n * k, dtype=torch.float64).pin_memory()
        ctx.set_options(precision=S.FP64 if args.mode == "fp64" else S.MIXED)
        e2e_times = []
        for _ in range(min(max(1, args.steps), 3)):  # median of up to 3 steps
            barrier()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            X.upload_ptr(pinned_in.data_ptr(), n)
            S.lobpcg_solve_double(X, A, T=T, atol=cfg["tol"], rtol=1e-50, maxit=cfg["maxit"],
                                  history=False)
            X.download_ptr(pinned_out.data_ptr(), n)
            e2e_times.append(time.perf_counter() - t0)
        e2e = max_over_ranks(statistics.median(e2e_times), dist, "cuda")
        del pinned_in, pinned_out
    # X holds the timed arm's Ritz vectors again (same solve, deterministic)
    solve(args.mode)

    pk, pk_kind = peaks()
    fp64_peak = fp64_peak_tflops(torch)
    tf32_peak = pk["bf16_tflops"] / 2.0
    traffic = load_traffic(args.config)

    # the other arm on the same problem, one solve with its own kernel
    # breakdown (the plain FP64 GPU path beside the mixed arm, or the mixed
    # arm beside an FP64 timed arm)
    other = None
    other_mode = "fp64" if args.mode == "mixed" else "mixed"
    if not args.no_other_arm:
        Xo = S.MultiVector(ctx, n, k)
        solve(other_mode, maxit=3, into=Xo)  # first launches, workspace growth
        ctx.profiling(True)
        ctx.reset_kernel_times()
        torch.cuda.synchronize()
        eo0 = torch.cuda.Event(enable_timing=True)
        eo1 = torch.cuda.Event(enable_timing=True)
        eo0.record(stream)
        ro = solve(other_mode, into=Xo)
        eo1.record(stream)
        torch.cuda.synchronize()
        to = eo0.elapsed_time(eo1) / 1e3
        kt_o = ctx.kernel_times()
        ctx.profiling(False)
        tot_o = top_level_ms(kt_o)
        other = dict(arm_summary(ro, to), mode=other_mode,
                     kernels={nm: {"share": v["ms"] / tot_o, "launches": v["launches"],
                                   "avg_ms": v["ms"] / v["launches"]}
                              for nm, v in sorted(kt_o.items(), key=lambda kv: -kv[1]["ms"])[:10]})
        Xm, Xf = (X, Xo) if args.mode == "mixed" else (Xo, X)
        rm, rf = (res, ro) if args.mode == "mixed" else (ro, res)
        other["comparison"] = compare_arms(ctx, S, Xm, Xf, rm, rf)
        other["mixed_speedup_over_fp64"] = (to / secs) if args.mode == "mixed" else (secs / to)
        Xo.close()
    orth = orthonormality(ctx, S, X)

    total_ms = top_level_ms(ktimes)
    dom_name, dom = max(((nm, v) for nm, v in ktimes.items() if not nested(nm)),
                        key=lambda kv: kv[1]["ms"])
    roofline = roofline_entry(dom_name, dom, pk["hbm_gbs"], fp64_peak, traffic,
                              fp64_arith=args.mode == "fp64", tf32_peak=tf32_peak)
    if roofline["bound"] == "hbm":
        roofline["peak_kind"] = pk_kind
    roofline["share_of_kernel_time"] = dom["ms"] / total_ms
    roofline["fp64_peak_tflops"] = fp64_peak
    spmm_name = "spmm_csr" if op[0] == "csr" else "stencil7"
    if args.mode == "mixed" and spmm_name + "_fp32" in ktimes:
        spmm_name += "_fp32"  # the FP32 launches (FP64 ones are timed apart)
    spmm = ktimes.get(spmm_name)
    kernels = {nm: {"share": v["ms"] / total_ms, "launches": v["launches"],
                    "nested_in_sygv": nested(nm),
                    "avg_ms": v["ms"] / v["launches"],
                    "gbs": v["bytes"] / (v["ms"] / 1e3) / 1e9,
                    "tflops": v["flops"] / (v["ms"] / 1e3) / 1e12}
               for nm, v in sorted(ktimes.items(), key=lambda kv: -kv[1]["ms"])}
    rooflines = {nm: roofline_entry(nm, ktimes[nm], pk["hbm_gbs"], fp64_peak, traffic,
                                    fp64_arith=args.mode == "fp64", tf32_peak=tf32_peak)
                 for nm in ("tc_gram", "tc_xc_update", "oz_xc_update", "oz_gram",
                            "stencil7_fp32", "spmm_csr_fp32") if nm in ktimes}
    # the split-operand products are FP64-accurate products bound by their
    # digit work: their rate beside the FP64 pipe they replace
    for nm in ("oz_xc_update", "oz_gram"):
        if nm in rooflines:
            v = ktimes[nm]
            eq = v["flops"] / (v["ms"] / 1e3) / 1e12
            rooflines[nm]["fp64_accurate_tflops"] = eq
            rooflines[nm]["over_fp64_pipe"] = eq / fp64_peak

    line = {"metric": metric_name(cfg, res, args.mode), "value": secs, "unit": "s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": secs * 1e3, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f64" if args.mode == "fp64" else "f32/tf32/bf16-split + f64",
            "data": "synthetic", "config": config_block(cfg, args, precond),
            "result": dict(arm_summary(res, secs), mode=args.mode,
                           orthonormality_fro=orth),
            "other_arm": other,
            "roofline": roofline,
            "spmm": None if spmm is None else roofline_entry(spmm_name, spmm, pk["hbm_gbs"],
                                                             fp64_peak, traffic,
                                                             fp64_arith=args.mode == "fp64"),
            "rooflines": rooflines,
            "kernels": kernels,
            "e2e": None if e2e is None else {"value": e2e, "unit": "s",
                                             "h2d_bytes_per_step": n * k * 8,
                                             "d2h_bytes_per_step": n * k * 8 + 2 * k * 8},
            "gpu_launches": int(launches),
            "clocks": clocks}
    full = None
    if cfg.get("full") and not args.no_full:
        X0.close()
        X.close()
        ctx.lib.gpu_ContextTrim(ctx.handle)
        full = run_full(dict(CONFIGS[cfg["full"]]), ctx, S, torch, stream, precond)
        line["full_size"] = full
    if rank == 0 and not args.no_cpu:
        fp64_its = (other["iterations"] if (other and other_mode == "fp64")
                    else (res.iterations if args.mode == "fp64" else None))
        line["cpu_baseline"] = cpu_baseline(cfg, fp64_its)
        if full and full.get("fp64"):
            line["full_size"]["cpu_baseline"] = cpu_baseline(dict(CONFIGS[cfg["full"]]),
                                                             full["fp64"]["iterations"])
    if cfg.get("adjoint") and not args.no_adjoint:
        line["adjoint"] = adjoint_summary(cfg["adjoint"], world, local, dist)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def adjoint_summary(name, world, local, dist):
    """The derivative configuration measured once beside the headline (one
    untimed and one timed forward + backward step): its forward and backward
    times, their ratio and the end-to-end autograd time.  A failure here is
    reported in the record and does not touch the headline."""
    try:
        a = measure_adjoint(dict(CONFIGS[name]), 1, 1, world, local, dist)
    except Exception as e:  # the headline line is printed whatever happens here
        return {"config": name, "error": f"{type(e).__name__}: {e}"}
    return {"config": name, "workload": a["config"]["workload"], "forward_ms": a["forward_ms"],
            "backward_ms": a["backward_ms"], "fwd_plus_bwd_ms": a["value"],
            "fwd_plus_bwd_over_fwd": a["fwd_plus_bwd_over_fwd"],
            "lobpcg_iterations": a["lobpcg_iterations"],
            "adjoint_cg_iterations": a["adjoint_cg_iterations"],
            "adjoint_max_rel_residual": a["adjoint_max_rel_residual"], "e2e_ms": a["e2e"]["value"],
            "gpu_launches": a["gpu_launches"], "steps": 1, "warmup": 1}


def run_full(cfg, ctx, S, torch, stream, precond):
    """The full-size configuration measured once per arm: mixed precision and
    the plain FP64 GPU path, each from the same X0 to the tolerance (after a
    3-iteration warm-up of its kernels), with the eigenvalue error, the
    largest subspace angle between the two blocks and X'X - I."""
    n, op, x0, tdiag = build_problem(cfg)
    k = cfg["k"]
    A = S.Stencil7(ctx, *op[1]) if op[0] == "stencil7" else S.CSRMatrix(ctx, *op[1])
    T = S.Diagonal(ctx, tdiag) if tdiag is not None else None
    if precond.startswith("pcg"):
        T = S.PCGPreconditioner(ctx, A, T, int(precond[3:]))
    X0 = S.MultiVector(ctx, n, k)
    if x0 is not None:
        X0.upload(x0)
    else:
        X0.set_random(cfg["seed"])
    out = {"workload": cfg["label"], "n": n, "k": k, "tol": cfg["tol"], "maxit": cfg["maxit"]}
    blocks, results = {}, {}
    for mode in ("mixed", "fp64"):
        Xm = S.MultiVector(ctx, n, k)
        ctx.set_options(precision=S.FP64 if mode == "fp64" else S.MIXED)
        Xm.copy_from(X0)
        S.lobpcg_solve_double(Xm, A, T=T, atol=cfg["tol"], rtol=1e-50, maxit=3, history=False)
        Xm.copy_from(X0)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        r = S.lobpcg_solve_double(Xm, A, T=T, atol=cfg["tol"], rtol=1e-50, maxit=cfg["maxit"],
                                  history=False)
        e1.record(stream)
        torch.cuda.synchronize()
        out[mode] = dict(arm_summary(r, e0.elapsed_time(e1) / 1e3),
                         orthonormality_fro=orthonormality(ctx, S, Xm))
        blocks[mode], results[mode] = Xm, r
    out["comparison"] = compare_arms(ctx, S, blocks["mixed"], blocks["fp64"], results["mixed"],
                                     results["fp64"])
    out["mixed_speedup_over_fp64"] = out["fp64"]["seconds"] / out["mixed"]["seconds"]
    for b in blocks.values():
        b.close()
    X0.close()
    return out


def arm_summary(r, seconds):
    st = r.stats
    return {"seconds": seconds, "flag": r.flag, "iterations": r.iterations,
            "seconds_per_iteration": seconds / max(r.iterations, 1),
            "max_residual": float(np.max(r.res)),
            "lambda_min": float(r.lam[0]), "lambda_max": float(r.lam[-1]),
            "iterations_explicit": st["iterations_fp32"], "iterations_split": st["iterations_split"],
            "iterations_fp64_loop": st["iterations_fp64"],
            "iterations_compensated": st["iterations_compensated"],
            "explicit_undos": st["explicit_undos"], "explicit_p_drops": st["explicit_p_drops"],
            "handover_reason": st["handover_reason"], "device_errors": st["device_errors"],
            "seconds_explicit_phase": st["seconds_fp32"], "seconds_fp64_loop": st["seconds_fp64"]}


def _gram_host(ctx, S, A_, B_):
    """A_' B_ (FP64 device blocks) through the GPU interpreter, to the host."""
    interp = S._Interp(ctx.lib)
    aa = ctx.lib.mv_MultiVectorWrap(interp.ptr, A_.handle, 0)
    bb = ctx.lib.mv_MultiVectorWrap(interp.ptr, B_.handle, 0)
    h, w = A_.shape[1], B_.shape[1]
    v = np.zeros((h, w), order="F")
    ctx.lib.mv_MultiVectorByMultiVector(aa, bb, h, h, w, v.ctypes.data)
    ctx.lib.mv_MultiVectorDestroy(aa)
    ctx.lib.mv_MultiVectorDestroy(bb)
    return v


def orthonormality(ctx, S, Xb):
    """||X'X - I||_F of a returned block (the reference's -orthchk,
    blopex_hypre/test/ij.c:2626-2643, with B = I)."""
    G = _gram_host(ctx, S, Xb, Xb)
    return float(np.linalg.norm(G - np.eye(G.shape[0])))


def compare_arms(ctx, S, Xm, Xf, rm, rf):
    """Eigenvalue error of the mixed arm against the FP64 arm and the largest
    principal angle between the two k-dimensional eigenvector blocks:
    sin(theta_max) = || Xm - Xf (Xf' Xm) ||_2 with Xf orthonormal (FP64)."""
    C = _gram_host(ctx, S, Xf, Xm)
    n, k = Xm.shape
    D = S.MultiVector(ctx, n, k)
    Cn = np.asfortranarray(-C)
    rc = ctx.lib.gpu_BlockUpdate(Xf.handle, Cn.ctypes.data, k, D.handle, Xm.handle, 0)
    if rc:
        raise RuntimeError(ctx.last_error())
    DD = _gram_host(ctx, S, D, D)
    D.close()
    sin_max = float(np.sqrt(max(np.linalg.eigvalsh(0.5 * (DD + DD.T))[-1], 0.0)))
    return {"max_rel_lambda_error_vs_fp64": float(np.max(np.abs(rm.lam - rf.lam) /
                                                          np.abs(rf.lam))),
            "largest_subspace_angle_rad": float(np.arcsin(min(sin_max, 1.0))),
            "both_converged": bool(rm.flag == 0 and rf.flag == 0)}


if __name__ == "__main__":
    main()
