"""Writes the oracle side of the full-size precision check as small fixtures.

For each case (rk4-fdm and split-step-fft in its CPU ordering; the FP32 device run's noise
realisation and the FP64 one) the FP64 oracle steps the 1024^2, 1000-step workload of
``tests/precision_check.py`` and ``tests/golden/precision_<case>.npz`` keeps:

* ``norms``: the 1000-entry norm trajectory (sum |psi|^2 dx dy after every step);
* ``psi`` and ``res``: the final psi and n_R on every 8th row and column (128^2 sites);
* ``stride``, ``steps``, ``n`` and ``inputs``: the sampling stride, the run's size and a
  fingerprint of the initial field, so a device run can check that it started from the same
  field.

The oracle takes about a quarter of an hour of one CPU core per case, which is why its results
are kept: the ``-m gpu`` test runs only the device leg and compares with these files.

    python tests/golden/make_precision_golden.py [--jobs 4] [--cases rk4_fp32 ...]
"""
from __future__ import annotations

import argparse
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

HERE = Path(__file__).resolve().parent
STRIDE = 8


def _one(case):
    from tests import precision_check as pc

    method, precision = case
    t0 = time.perf_counter()
    psi, res, norms, fp = pc.oracle_case(method, precision, pc.STEPS, pc.N)
    out = HERE / f"precision_{pc.case_name(method, precision)}.npz"
    np.savez_compressed(out, norms=np.asarray(norms, np.float64),
                        psi=np.ascontiguousarray(psi[0, 0, ::STRIDE, ::STRIDE]),
                        res=np.ascontiguousarray(res[0, 0, ::STRIDE, ::STRIDE]),
                        stride=STRIDE, steps=pc.STEPS, n=pc.N, inputs=fp)
    return f"{out.name}: {time.perf_counter() - t0:.0f} s, final norm {norms[-1]:.17g}"


def main(argv=None):
    from tests import precision_check as pc

    names = [pc.case_name(m, p) for m, p in pc.CASES]
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--jobs", type=int, default=4)
    ap.add_argument("--cases", nargs="+", default=names, choices=names)
    a = ap.parse_args(argv)
    work = [c for c in pc.CASES if pc.case_name(*c) in a.cases]
    if a.jobs <= 1:
        lines = list(map(_one, work))
    else:
        import multiprocessing as mp

        with mp.get_context("spawn").Pool(min(a.jobs, len(work))) as pool:
            lines = pool.map(_one, work)
    for line in lines:
        print(line, flush=True)


if __name__ == "__main__":
    main()
