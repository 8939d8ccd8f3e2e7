"""The precision check at full size: 1024^2 periodic, lx = ly = 400 um, dt = 5e-4 ps, 1000
steps of rk4-fdm and of split-step-fft (the CPU ordering) with Wigner noise on, each on the GPU
in complex64 and in complex128, compared with the FP64 NumPy oracle on psi, n_R and the norm
trajectory (relative L2 errors; the bar is 1e-10 in FP64 and 1e-4 in FP32).

Physics: the reference's Config defaults with a continuous Gaussian pump P0 = 0.02,
sigma = 12 um, centred, single reservoir, no potential; initial psi complex Gaussian noise of
amplitude 1e-3 from seed 0 (``polarism/simulation_state.py``), n_R = 0; Philox key 42.  An FP32
run is compared with an FP64 oracle run that draws the same noise realisation (the
single-precision normal construction computed in FP64), an FP64 run with the oracle's own
double-precision normals.

The GPU leg and the oracle leg run apart, so the oracle's ~15 minutes of one CPU core per case
need not hold a GPU:

    python -m tests.precision_check gpu --out DIR            # on a GPU: DIR/<case>.npz
    python -m tests.precision_check oracle --gpu DIR --out results.json [--jobs 4]

``tests/test_precision_check_gpu.py`` runs both legs when PG_PRECISION_CHECK=1.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

N = 1024
L = 400.0
DT = 5e-4
STEPS = 1000
P0 = 0.02
SIGMA = 12.0
INIT_SEED = 0
NOISE_KEY = 42
CASES = [("rk4", "single"), ("rk4", "double"), ("split", "single"), ("split", "double")]
BAR = {"single": 1e-4, "double": 1e-10}


def case_name(method, precision):
    return f"{method}_{'fp32' if precision == 'single' else 'fp64'}"


def inputs(n=N):
    """(physics dict, dx, dy, envelope (ny, nx), psi0 (1, 1, ny, nx), k^2) in FP64."""
    from polarism_gb300.host import Config, build_simulation

    cfg = Config()
    cfg.grid.nx = cfg.grid.ny = n
    cfg.grid.lx = cfg.grid.ly = L * n / N
    cfg.laser.P0, cfg.laser.sigma_space = P0, SIGMA
    cfg.solver.dt, cfg.noise.seed = DT, INIT_SEED
    grid, model, state = build_simulation(cfg)
    p = {k: float(getattr(cfg.physics, k)) for k in ("hbar", "m_eff", "g_C", "g_R", "g_I", "R",
                                                     "gamma_C", "gamma_R")}
    env = np.asarray(model.pump.separable_term()[0], dtype=np.float64)
    psi0 = np.asarray(state.field, dtype=np.complex128)
    return p, float(grid.dx), float(grid.dy), env, psi0, np.asarray(grid.k_squared, np.float64)


def fingerprint(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()[:16]


# ----------------------------------------------------------------------------- GPU leg
def gpu_case(method, precision, steps, n):
    from polarism_gb300.engine import Engine, MemberPhysics

    p, dx, dy, env, psi0, _ = inputs(n)
    eng = Engine(n, n, 1, dx, dy, DT, MemberPhysics(**p), precision)
    eng.set_pump(env.astype(eng.real))
    eng.set_noise([NOISE_KEY], p["gamma_C"], p["R"], 1.0, DT / (4 * dx * dy))
    eng.set_state(psi0.astype(eng.complex), np.zeros(psi0.shape, dtype=eng.real))
    norms = np.empty(steps)
    t0 = time.perf_counter()
    for k in range(steps):
        if method == "rk4":
            eng.advance(k, 1, np.full((1, 3, 1), P0), use_graphs=False)
        else:
            eng.split_advance(0, k, 1, np.full((1, 2, 1), P0), use_graphs=False)
        norms[k] = eng.norms()[0]
    psi, res = eng.get_state()
    wall = time.perf_counter() - t0
    eng.close()
    # The envelope travels with the result: NumPy's exp may differ in the last place between
    # the machine that runs the GPU leg and the one that runs the oracle.
    return dict(psi=psi, res=res, norms=norms, wall=wall, env=env,
                inputs=fingerprint(psi0), steps=steps, n=n)


def gpu_leg(out_dir, steps=STEPS, n=N, cases=CASES):
    out = Path(out_dir)
    out.mkdir(parents=True, exist_ok=True)
    for method, precision in cases:
        r = gpu_case(method, precision, steps, n)
        np.savez(out / f"{case_name(method, precision)}.npz", **r)
        print(f"{case_name(method, precision)}: {steps} steps in {r['wall']:.1f} s "
              f"(one step and one norm per call)", flush=True)


# -------------------------------------------------------------------------- oracle leg
def oracle_case(method, precision, steps, n, env=None):
    """The FP64 oracle run an FP32 or FP64 device run is compared with (on the device run's
    pump envelope when given)."""
    from oracle import gpe

    p, dx, dy, own_env, psi0, k2 = inputs(n)
    env = own_env if env is None else np.asarray(env, dtype=np.float64)
    noise = gpe.Noise([NOISE_KEY], [p["gamma_C"]], [p["R"]], [1.0], DT, dx * dy, "double",
                      normals_precision=precision)
    pump = env * P0
    norms = []
    fields = (np.zeros(psi0.shape),)
    if method == "rk4":
        psi, fields = gpe.rk4_advance(psi0.copy(), fields, lambda t: pump, 0.0, p, dx, dy, DT, 0,
                                      steps, noise=noise, norm_trace=norms)
    else:
        psi, fields = gpe.split_advance("cpu", psi0.copy(), fields, lambda t: pump, 0.0, p, k2,
                                        dx, dy, DT, 0, steps, noise=noise, norm_trace=norms)
    return psi, fields[0], np.asarray(norms).ravel(), fingerprint(psi0)


def _rel_l2(a, b):
    a = np.asarray(a, dtype=np.complex128).ravel()
    b = np.asarray(b, dtype=np.complex128).ravel()
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _compare(job):
    gpu_dir, method, precision, keep = job
    name = case_name(method, precision)
    g = np.load(Path(gpu_dir) / f"{name}.npz")
    steps, n = int(g["steps"]), int(g["n"])
    t0 = time.perf_counter()
    psi, res, norms, fp = oracle_case(method, precision, steps, n, env=g["env"])
    if fp != str(g["inputs"]):
        raise RuntimeError(f"{name}: the GPU leg started from a different initial field")
    if keep:
        np.savez(Path(gpu_dir) / f"{name}_oracle.npz", psi=psi, res=res, norms=norms)
    return name, {
        "method": "rk4-fdm" if method == "rk4" else "split-step-fft (CPU ordering)",
        "precision": "complex64" if precision == "single" else "complex128",
        "steps": steps, "grid": [n, n],
        "psi_rel_l2": _rel_l2(g["psi"], psi),
        "n_R_rel_l2": _rel_l2(g["res"], res),
        "norm_trajectory_rel_l2": _rel_l2(g["norms"], norms),
        "norm_max_rel_err": float(np.max(np.abs(g["norms"] - norms) / np.abs(norms))),
        "final_norm": float(norms[-1]),
        "bar": BAR[precision],
        "oracle_seconds": time.perf_counter() - t0,
    }


def oracle_leg(gpu_dir, out_json, jobs=4, cases=CASES, keep=False):
    """Oracle runs for every device file in gpu_dir (``keep``: also save the oracle's final
    state and norms beside it as <case>_oracle.npz)."""
    import multiprocessing as mp

    work = [(str(gpu_dir), m, p, keep) for m, p in cases
            if (Path(gpu_dir) / f"{case_name(m, p)}.npz").exists()]
    if jobs <= 1 or len(work) <= 1:
        results = dict(map(_compare, work))
    else:
        with mp.get_context("spawn").Pool(min(jobs, len(work))) as pool:
            results = dict(pool.map(_compare, work))
    for name, r in results.items():
        r["pass"] = max(r["psi_rel_l2"], r["n_R_rel_l2"], r["norm_trajectory_rel_l2"]) < r["bar"]
    Path(out_json).write_text(json.dumps(results, indent=1) + "\n")
    for name, r in results.items():
        print(f"{name}: psi {r['psi_rel_l2']:.3e}  n_R {r['n_R_rel_l2']:.3e}  "
              f"norms {r['norm_trajectory_rel_l2']:.3e}  (bar {r['bar']:g}) "
              f"{'pass' if r['pass'] else 'FAIL'}", flush=True)
    return results


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    sub = ap.add_subparsers(dest="leg", required=True)
    g = sub.add_parser("gpu")
    g.add_argument("--out", required=True)
    g.add_argument("--steps", type=int, default=STEPS)
    g.add_argument("--grid", type=int, default=N)
    g.add_argument("--cases", nargs="+", default=[case_name(m, p) for m, p in CASES],
                   help="subset of " + " ".join(case_name(m, p) for m, p in CASES))
    o = sub.add_parser("oracle")
    o.add_argument("--gpu", required=True)
    o.add_argument("--out", required=True)
    o.add_argument("--jobs", type=int, default=int(os.environ.get("PG_ORACLE_JOBS", "4")))
    o.add_argument("--cases", nargs="+", default=[case_name(m, p) for m, p in CASES])
    o.add_argument("--keep", action="store_true", help="save the oracle states too")
    a = ap.parse_args(argv)
    if a.leg == "gpu":
        gpu_leg(a.out, a.steps, a.grid, [c for c in CASES if case_name(*c) in a.cases])
    else:
        oracle_leg(a.gpu, a.out, a.jobs, [c for c in CASES if case_name(*c) in a.cases], a.keep)


if __name__ == "__main__":
    main()
