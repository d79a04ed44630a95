"""Generate the golden fixtures in this directory from the UNMODIFIED
reference (test infrastructure).

Runs the reference ``lobpcg_solve_double`` with the serial-double backend
(compiled by ``oracle/Makefile`` into ``oracle/_ref``) on seeded synthetic
inputs and records exit flag, iteration count, eigenvalues, residual norms
and their histories.  Inputs are rebuilt by the tests from the same
generators; a SHA-256 of every input array is stored to pin them.

Run in a container that has the reference checkout (its location in the
environment variable BLOPEX_REFERENCE_DIR):
    python tests/golden/make_golden.py            # the small cases
    python tests/golden/make_golden.py --large    # the 128^3 cases (hours
                                                  # of CPU; the three builds
                                                  # run in parallel processes)
    python tests/golden/make_golden.py --fingerprints  # add the input
                                                  # fingerprints to existing
                                                  # 128^3 fixtures
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from tests.golden import cases as C  # noqa: E402


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def fingerprint(a: np.ndarray) -> list:
    """Two weighted sums of a floating-point input: they pin it to rounding
    where its SHA-256 cannot -- numpy's exp() differs in the last bit between
    x86-64 and aarch64, so exp(N(0,1)) coefficients regenerated on another
    host hash differently while agreeing to ~1e-16."""
    v = np.ascontiguousarray(a, dtype=np.float64).ravel()
    w = (np.arange(v.size) % 97 + 1.0) / 97.0
    return [float(np.sum(v)), float(np.dot(v, w))]


def capture_stdout(fn):
    """Run fn() with the C-level stdout redirected; return (result, text)."""
    sys.stdout.flush()
    fd = os.dup(1)
    with tempfile.TemporaryFile(mode="w+b") as tmp:
        os.dup2(tmp.fileno(), 1)
        try:
            res = fn()
        finally:
            os.dup2(fd, 1)
            os.close(fd)
        tmp.seek(0)
        text = tmp.read().decode()
    return res, text


def run_case(name: str) -> dict:
    case = C.build(name)
    kw = dict(seed=case.seed, x0=case.x0, atol=case.atol, rtol=case.rtol, maxit=case.maxit,
              verbosity=case.verbosity, b_diag=case.b_diag, t_diag=case.t_diag, Y=case.Y,
              potrf_fail_at=case.potrf_fail_at, sygv_fail_at=case.sygv_fail_at)
    if case.csr is not None:
        kw["csr_arrays"] = case.csr
    else:
        kw["dense_a"] = case.dense
    r, text = capture_stdout(lambda: O.ref_solve(case.n, case.k, **kw))
    variants = {}
    for v in ("fma", "x87"):
        rv, _ = capture_stdout(lambda: O.ref_solve(case.n, case.k, variant=v, **kw))
        variants[v] = {"flag": rv.flag, "iterations": rv.iterations, "lambda": rv.lam.tolist(),
                       "resnorm": rv.res.tolist()}
    ncol = r.iterations + 1
    out = {
        "name": name,
        "description": case.description,
        "n": case.n, "k": case.k,
        "atol": case.atol, "rtol": case.rtol, "maxit": case.maxit,
        "flag": r.flag, "iterations": r.iterations,
        "lambda": r.lam.tolist(), "resnorm": r.res.tolist(),
        "lambda_hist": r.lam_hist[:, :ncol].T.tolist() if case.k > 0 else [],
        "res_hist": r.res_hist[:, :ncol].T.tolist() if case.k > 0 else [],
        "inputs_sha256": {key: sha(val) for key, val in case.arrays().items()},
        # the same reference sources built with FMA contraction / x87
        # arithmetic: the reference's own sensitivity to rounding
        "variants": variants,
    }
    if case.verbosity:
        out["stdout"] = text
    if case.n * case.k <= 4000:
        out["x"] = r.x.T.tolist()
    return out


def _large_variant(name: str, variant: str) -> dict:
    """One reference build on one large case (runs in a spawned process)."""
    import time

    case = C.build(name)
    kw = dict(seed=case.seed, atol=case.atol, rtol=case.rtol, maxit=case.maxit,
              t_diag=case.t_diag, b_diag=case.b_diag, csr_arrays=case.csr)
    t0 = time.time()
    r = O.ref_solve(case.n, case.k, variant=variant, **kw)
    ncol = r.iterations + 1
    return {"flag": r.flag, "iterations": r.iterations, "lambda": r.lam.tolist(),
            "resnorm": r.res.tolist(), "lambda_hist": r.lam_hist[:, :ncol].T.tolist(),
            "res_hist": r.res_hist[:, :ncol].T.tolist(), "seconds": time.time() - t0}


def main_large(names):
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor

    jobs = {}
    with ProcessPoolExecutor(max_workers=3 * len(names),
                             mp_context=mp.get_context("spawn")) as ex:
        for name in names:
            for v in ("", "fma", "x87"):
                jobs[(name, v)] = ex.submit(_large_variant, name, v)
        for name in names:
            case = C.build(name)
            plain = jobs[(name, "")].result()
            out = {"name": name, "description": case.description, "n": case.n, "k": case.k,
                   "atol": case.atol, "rtol": case.rtol, "maxit": case.maxit}
            out.update({key: plain[key] for key in ("flag", "iterations", "lambda", "resnorm",
                                                      "lambda_hist", "res_hist")})
            out["reference_seconds_one_core"] = plain["seconds"]
            out["inputs_sha256"] = {key: sha(val) for key, val in case.arrays().items()}
            out["inputs_fingerprint"] = {key: fingerprint(val) for key, val in case.arrays().items()
                                         if np.asarray(val).dtype.kind == "f"}
            out["variants"] = {}
            for v in ("fma", "x87"):
                rv = jobs[(name, v)].result()
                out["variants"][v] = {key: rv[key] for key in
                                      ("flag", "iterations", "lambda", "resnorm",
                                       "lambda_hist", "res_hist")}
            with open(os.path.join(HERE, f"{name}.json"), "w") as f:
                json.dump(out, f, indent=0)
            print(f"{name}: flag {out['flag']} iterations {out['iterations']} "
                  f"({plain['seconds']:.0f} s)", flush=True)


def add_fingerprints(names):
    """Add the input fingerprints to existing large fixtures, after checking
    that the regenerated inputs are those the fixture was made from."""
    for name in names:
        path = os.path.join(HERE, f"{name}.json")
        with open(path) as f:
            g = json.load(f)
        case = C.build(name)
        arrays = case.arrays()
        for key, val in arrays.items():
            if sha(val) != g["inputs_sha256"][key]:
                raise SystemExit(f"{name}: input {key} differs from the fixture's")
        g["inputs_fingerprint"] = {key: fingerprint(val) for key, val in arrays.items()
                                   if np.asarray(val).dtype.kind == "f"}
        with open(path, "w") as f:
            json.dump(g, f, indent=0)
        print(f"{name}: fingerprints added", flush=True)


def main():
    if "--fingerprints" in sys.argv:
        add_fingerprints(C.LARGE_NAMES)
        return
    if not O.have_ref():
        O.build(ref=True)
    O.build_ref_variants()
    if "--large" in sys.argv:
        main_large(C.LARGE_NAMES)
        return
    for name in C.NAMES:
        g = run_case(name)
        with open(os.path.join(HERE, f"{name}.json"), "w") as f:
            json.dump(g, f, indent=0)
        print(f"{name}: flag {g['flag']} iterations {g['iterations']}")


if __name__ == "__main__":
    main()
