#!/usr/bin/env python
"""Benchmark of the LOBPCG hot path on GB300 (one JSON line on stdout).

Workload (default, --config c2): the "plain FP64 on GPU" case -- 3D 7-point
Dirichlet Laplacian 128^3 (n = 2,097,152, CSR int32 / FP64, nnz =
14,581,760), block size k = 32, Jacobi preconditioner, X0 = 2*drand48()-1
from seed 1, tolerance 1e-8, at most 300 iterations.  One step = one full
lobpcg_solve_double call from X0 to exit (converged or maxit).  Synthetic
data generated by the seeded builders in blopex_gb300/problems.py.

value  = seconds per solve with X0, the matrix and the preconditioner
         resident in HBM (max over ranks), CUDA events on the solver stream;
e2e    = the same through the C ABI with X0 uploaded from pinned host memory
         and the Ritz vectors + eigenvalues read back, every step;
roofline = the kernel class with the largest share of the timed region,
         from the library's CUDA-event timers (algorithmic bytes per launch /
         event-timed duration), against MEASURED_PEAKS.json;
cpu_baseline = the C restatement of the reference (oracle/, scalar loops,
         one core) on a bounded sample, scaled to the full workload.

--impl reference times that CPU implementation alone (the reference's own
algorithm on the host cores; the compiled reference itself is not available
on the GPU host).  Under torchrun each rank runs an independent replica
(the solver does not shard: replicas only).
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CONFIGS = {
    "c1": dict(kind="csr", grid=(20, 20, 20), k=10, seed=0, tol=1e-6, maxit=100, jacobi=False,
               label="3D 7-point Laplacian 20^3 CSR, k=10, no preconditioner, tol 1e-6, maxit 100"),
    "c2": dict(kind="csr", grid=(128, 128, 128), k=32, seed=1, tol=1e-8, maxit=300, jacobi=True,
               label="3D 7-point Laplacian 128^3 CSR (n=2097152), k=32, Jacobi, tol 1e-8, maxit 300"),
    # matrix-free variable-coefficient stencil; a full solve to 1e-8 takes
    # thousands of iterations, so this case is timed per iteration (maxit 20)
    # differentiation: forward solve + reverse-mode gradient in theta
    "c4": dict(kind="adjoint5", grid=(512, 512), k=8, seed=3, tol=1e-8, maxit=3000,
               jacobi=True, adjoint_tol=1e-8, inner_cg=20,
               label="2D 5-point diffusion 512^2, c = exp(theta), theta GRF (length 0.1, seed 3), "
                     "k=8, loss = sum(lambda) + (x_1'v)^2, d loss / d theta; FP64, tol 1e-8, "
                     "preconditioner 20 Jacobi-CG steps on A"),
    "c3": dict(kind="stencil7", grid=(256, 256, 256), k=64, seed=2, tol=1e-8, maxit=20,
               jacobi=True,
               label="matrix-free variable-coefficient 7-point stencil 256^3 (n=16777216), face "
                     "coefficients exp(N(0,1)) seed 2, k=64, Jacobi, tol 1e-8, 20 iterations"),
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


def cpu_baseline(cfg, budget_s: float = 25.0):
    """The oracle (C restatement of the reference, one core) on a bounded
    sample: a 48^3 grid with the same k / preconditioner, 1 and 3 iterations;
    the per-iteration time is scaled by n to the full grid."""
    from blopex_gb300 import problems as P
    from oracle import oracle as O
    O.build(ref=False)
    nx, ny, nz = cfg["grid"]
    n_full = nx * ny * nz
    s = min(48, nx)
    n, op, x0, tdiag = build_problem(cfg, (s, s, s))
    csr = op[1] if op[0] == "csr" else P.stencil7_to_csr(*op[1])
    A = O.csr(*csr)
    T = O.diag(tdiag) if tdiag is not None else O.NONE
    t0 = time.perf_counter()
    O.solve(A, x0, T=T, atol=cfg["tol"], maxit=1, history=False)
    t1 = time.perf_counter()
    O.solve(A, x0, T=T, atol=cfg["tol"], maxit=3, history=False)
    t2 = time.perf_counter()
    per_it = max((t2 - t1) - (t1 - t0), 1e-9) / 2.0
    setup = max((t1 - t0) - per_it, 0.0)
    scale = n_full / n
    value = (setup + cfg["maxit"] * per_it) * scale
    return {"value": value, "unit": "s", "cores": 1, "kind": "port",
            "sample": f"oracle C restatement, {s}^3 grid k={cfg['k']}, 1 and 3 iterations "
                      f"({t2 - t0:.1f} s), per-iteration {per_it:.3f} s scaled by n x{scale:.1f} "
                      f"to {cfg['maxit']} iterations (extrapolated)",
            "per_iteration_s_full_n": per_it * scale}


def run_adjoint(args, cfg):
    """--config c4: forward LOBPCG solve and reverse-mode gradient of the
    loss through the adjoint module.  value = forward + backward ms per step
    (device-resident coefficients and blocks, CUDA events on the solver
    stream); e2e = the torch.autograd path from a host theta to host
    d loss / d theta."""
    import torch
    from blopex_gb300 import adjoint as AD
    from blopex_gb300 import problems as P
    from blopex_gb300 import solver as S
    world, rank, local, dist = dist_setup()
    torch.cuda.set_device(local)
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

    for _ in range(args.warmup):
        backward(forward())
    ctx.profiling(True)
    ctx.reset_kernel_times()
    sampler = ClockSampler(local)
    if dist is not None:
        dist.barrier()
    sampler.start()
    launches0 = ctx.lib.gpu_KernelLaunchCount()
    fwd, bwd, its, aits, res = [], [], 0, 0, 0.0
    for _ in range(args.steps):
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
    for _ in range(max(1, args.steps)):
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
    total = sum(v_["ms"] for v_ in kt.values()) or 1.0
    e2e_ms = max_over_ranks(statistics.median(e2e), dist, "cuda")
    line = {"metric": "fwd+bwd ms (forward solve + reverse-mode gradient)", "value": tf + tb,
            "unit": "ms", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
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
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def run_reference(args, cfg):
    """--impl reference: the CPU implementation of the path timed alone."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    for _ in range(args.warmup):
        cpu_baseline(cfg)
    vals = [cpu_baseline(cfg) for _ in range(args.steps)]
    v = statistics.median(x["value"] for x in vals)
    cb = dict(vals[0])
    cb["value"] = v
    line = {"impl": "reference", "metric": metric_name(cfg), "value": v, "unit": "s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": v * 1e3, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_block(cfg, args), "cpu_baseline": cb,
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


def metric_name(cfg):
    return ("time to k eigenpairs at resid 1e-8 (FP64 GPU path; mixed reported beside); "
            "SpMM GB/s") if cfg["tol"] <= 1e-8 else "time to k eigenpairs"


def config_block(cfg, args):
    return {"workload": cfg["label"] + (f" [preconditioner: {args.precond[3:]} inner CG steps]"
                                        if args.precond else ""),
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
    ap.add_argument("--config", default="c2", choices=sorted(CONFIGS))
    ap.add_argument("--mode", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--maxit", type=int, default=0, help="override maxit (exploration only)")
    ap.add_argument("--precond", default="",
                    help="'pcgN': precondition with N inner CG steps (Jacobi inside) instead of "
                         "Jacobi alone")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end repetition")
    ap.add_argument("--grid", type=int, default=0,
                    help="override the grid edge (small cases for profiling only)")
    ap.add_argument("--no-mixed", action="store_true", help="skip the mixed-precision arm")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    args = ap.parse_args()
    cfg = dict(CONFIGS[args.config])
    if args.maxit:
        cfg["maxit"] = args.maxit
    if args.grid:
        cfg["grid"] = (args.grid,) * 3
        cfg["label"] += f" [profiling case: grid {args.grid}^3]"

    if args.impl == "reference":
        if cfg["kind"] == "adjoint5":
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no "
                              "derivatives (no adjoint or gradient of its eigenpairs)"}), flush=True)
            return
        run_reference(args, cfg)
        return
    if cfg["kind"] == "adjoint5":
        run_adjoint(args, cfg)
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
    if args.precond.startswith("pcg"):
        T = S.PCGPreconditioner(ctx, A, T, int(args.precond[3:]))
    X = S.MultiVector(ctx, n, k)
    if x0 is not None:
        X0 = S.MultiVector.from_host(ctx, x0)
    else:
        X0 = S.MultiVector(ctx, n, k)
        X0.set_random(cfg["seed"])

    def solve(mode):
        ctx.set_options(precision=S.FP64 if mode == "fp64" else S.MIXED)
        X.copy_from(X0)
        return S.lobpcg_solve_double(X, A, T=T, atol=cfg["tol"], rtol=1e-50,
                                     maxit=cfg["maxit"], history=False)

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

    # e2e: X0 from pinned host memory, Ritz vectors back, every step
    if x0 is not None:
        pinned_in = torch.from_numpy(np.asfortranarray(x0).ravel(order="F")).pin_memory()
    else:
        pinned_in = torch.empty(n * k, dtype=torch.float64).pin_memory()
        X0.download_ptr(pinned_in.data_ptr(), n)
    pinned_out = torch.empty(n * k, dtype=torch.float64).pin_memory()
    ctx.set_options(precision=S.FP64 if args.mode == "fp64" else S.MIXED)
    e2e_times = []
    for _ in range(0 if args.no_e2e else max(1, args.steps)):
        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        X.upload_ptr(pinned_in.data_ptr(), n)
        r2 = S.lobpcg_solve_double(X, A, T=T, atol=cfg["tol"], rtol=1e-50, maxit=cfg["maxit"],
                                   history=False)
        X.download_ptr(pinned_out.data_ptr(), n)
        e2e_times.append(time.perf_counter() - t0)
    e2e = statistics.median(e2e_times) if e2e_times else None
    if e2e is not None:
        e2e = max_over_ranks(e2e, dist, "cuda")

    pk, pk_kind = peaks()
    fp64_peak = fp64_peak_tflops(torch)
    tf32_peak = pk["bf16_tflops"] / 2.0
    traffic = load_traffic(args.config)

    # the mixed-precision arm on the same problem (one solve, timed, with
    # its own kernel breakdown)
    mixed = None
    if args.mode == "fp64" and not args.no_mixed:
        # warm-up of the mixed path (first launches, workspace growth)
        ctx.set_options(precision=S.MIXED)
        X.copy_from(X0)
        S.lobpcg_solve_double(X, A, T=T, atol=cfg["tol"], rtol=1e-50, maxit=3, history=False)
        ctx.profiling(True)
        ctx.reset_kernel_times()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rm = solve("mixed")
        torch.cuda.synchronize()
        tm = time.perf_counter() - t0
        kt_m = ctx.kernel_times()
        ctx.profiling(False)
        tot_m = sum(v["ms"] for v in kt_m.values()) or 1.0
        st = rm.stats
        mixed = {"seconds": tm, "seconds_per_iteration": tm / max(rm.iterations, 1),
                 "seconds_fp32_phase": st["seconds_fp32"],
                 "seconds_per_fp32_iteration": st["seconds_fp32"] / max(st["iterations_fp32"], 1),
                 "seconds_fp64_phase": st["seconds_fp64"],
                 "flag": rm.flag, "iterations": rm.iterations,
                 "iterations_fp32": st["iterations_fp32"],
                 "iterations_compensated": st["iterations_compensated"],
                 "iterations_fp64": st["iterations_fp64"],
                 "explicit_undos": st["explicit_undos"],
                 "max_rel_lambda_diff_vs_fp64": float(np.max(np.abs(rm.lam - res.lam) /
                                                             np.abs(res.lam))),
                 "final_max_residual": float(np.max(rm.res)),
                 "kernels": {nm: {"share": v["ms"] / tot_m, "launches": v["launches"],
                                  "avg_ms": v["ms"] / v["launches"]}
                             for nm, v in sorted(kt_m.items(), key=lambda kv: -kv[1]["ms"])[:10]},
                 "roofline": {nm: roofline_entry(nm, kt_m[nm], pk["hbm_gbs"], fp64_peak, traffic,
                                                 fp64_arith=False, tf32_peak=tf32_peak)
                              for nm in ("tc_gram", "tc_xc_update", "stencil7_fp32",
                                         "spmm_csr_fp32")
                              if nm in kt_m}}
    total_ms = sum(v["ms"] for v in ktimes.values()) or 1.0
    dom_name, dom = max(ktimes.items(), key=lambda kv: kv[1]["ms"])
    roofline = roofline_entry(dom_name, dom, pk["hbm_gbs"], fp64_peak, traffic)
    if roofline["bound"] == "hbm":
        roofline["peak_kind"] = pk_kind
    roofline["share_of_kernel_time"] = dom["ms"] / total_ms
    roofline["fp64_peak_tflops"] = fp64_peak
    spmm_name = "spmm_csr" if op[0] == "csr" else "stencil7"
    if args.mode == "mixed" and spmm_name + "_fp32" in ktimes:
        spmm_name += "_fp32"  # the FP32 phase's launches (FP64 ones are timed apart)
    spmm = ktimes.get(spmm_name)
    kernels = {nm: {"share": v["ms"] / total_ms, "launches": v["launches"],
                    "avg_ms": v["ms"] / v["launches"],
                    "gbs": v["bytes"] / (v["ms"] / 1e3) / 1e9,
                    "tflops": v["flops"] / (v["ms"] / 1e3) / 1e12}
               for nm, v in sorted(ktimes.items(), key=lambda kv: -kv[1]["ms"])}

    line = {"metric": metric_name(cfg), "value": secs, "unit": "s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": secs * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if args.mode == "fp64" else "f32+f64", "data": "synthetic",
            "config": config_block(cfg, args),
            "result": {"flag": res.flag, "iterations": res.iterations,
                       "seconds_per_iteration": secs / max(res.iterations, 1),
                       "lambda_min": float(res.lam[0]), "lambda_max": float(res.lam[-1]),
                       "max_residual": float(np.max(res.res))},
            "roofline": roofline,
            "spmm": None if spmm is None else roofline_entry(spmm_name, spmm, pk["hbm_gbs"],
                                                             fp64_peak, traffic),
            "kernels": kernels,
            "mixed": mixed,
            "e2e": None if e2e is None else {"value": e2e, "unit": "s",
                                             "h2d_bytes_per_step": n * k * 8,
                                             "d2h_bytes_per_step": n * k * 8 + 2 * k * 8},
            "gpu_launches": int(launches),
            "clocks": clocks}
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(cfg)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
