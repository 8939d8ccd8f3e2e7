"""CUDA graph capture failures fall back to plain launches (GPU).

The reference re-runs a chunk with plain launches after restoring the pre-chunk state when its
graph capture fails (``polarism/solver/rk4_cuda_solver.py:3591-3602``;
``ifrk_fft_cuda_solver.py:1101-1109``).  Here capture only records, so a failed capture or
instantiation has run nothing of the chunk; the chunk then runs as plain launches.  The failure
is made on the host by the library's test hook (the capture or instantiation call reports an
error as a failing CUDA call would), so no GPU fault is involved.  Results must equal a run whose
graphs were built normally, bit for bit, and the fallback must be counted.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _engine(precision, nx=64, ny=32, members=2):
    from polarism_gb300.engine import MemberPhysics, RK4Engine

    rng = np.random.default_rng(21)
    eng = RK4Engine(nx, ny, members, 0.5, 0.5, 1e-3, MemberPhysics(), precision)
    x = (np.arange(nx) - nx / 2) * 0.5
    y = (np.arange(ny) - ny / 2) * 0.5
    eng.set_pump(np.exp(-0.5 * (x[None, :] ** 2 + y[:, None] ** 2) / 4.0 ** 2).astype(eng.real))
    eng.set_noise([5, 6], 0.083, 0.02, 1.0, 1e-3 / (4 * 0.25))
    psi = 0.1 * (rng.standard_normal((members, 1, ny, nx)) + 1j * rng.standard_normal((members, 1, ny, nx)))
    eng.set_state(psi.astype(eng.complex), np.full((members, 1, ny, nx), 0.2, eng.real))
    return eng


@pytest.mark.parametrize("what", [1, 2], ids=["capture", "instantiate"])
@pytest.mark.parametrize("path", ["rk4", "split-cpu", "split-kouter"])
def test_failed_graph_runs_as_plain_launches_with_equal_results(cuda_lib, path, what):
    steps = 20
    scales = np.full((steps, 3, 2), 0.05) if path == "rk4" else np.full((steps, 2, 2), 0.05)

    def run(fail):
        eng = _engine("single")
        if fail:
            eng.fail_next_graph(fail)
        if path == "rk4":
            eng.advance(0, steps, scales)
        else:
            eng.split_advance(0 if path == "split-cpu" else 1, 0, steps, scales)
        psi, res = eng.get_state()
        return psi, res, eng.graph_fallbacks

    psi_g, res_g, fb_g = run(0)
    psi_f, res_f, fb_f = run(what)
    assert fb_g == 0 and fb_f == 1
    assert np.array_equal(psi_f, psi_g)
    assert np.array_equal(res_f, res_g)
