"""Failure detection of the TMA-fed kernels on the GPU, without a fault.

Every mbarrier wait of the full-width RK4 kernel (two and four sites a thread, the cluster
form) and of the uneven-sweep kernel is bounded (100000 polls, compiled in).  The give-up
setting (wait limit 0) withholds each block's first row copy, so that on a healthy GPU every
thread's first wait runs out; the thread that feeds the ring then completes the remaining ring
slots without copies, the kernel ends in about the time of one full wait, and the next
synchronising call reports PG_ERR_TIMEOUT.  The test then restores the default and checks
that the same solver steps correctly again (bitwise equal to a fresh solver), so the context
and the solver stay usable.
"""
from __future__ import annotations

import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rk4(nx, ny, kind, members=1):
    from polarism_gb300.engine import MemberPhysics, RK4Engine

    dx = 400.0 / 1024
    eng = RK4Engine(nx, ny, members, dx, dx, 5e-4, MemberPhysics(), "single")
    x = (np.arange(nx) - nx / 2) * dx
    y = (np.arange(ny) - ny / 2) * dx
    eng.set_pump(np.exp(-0.5 * (x[None, :] ** 2 + y[:, None] ** 2) / 12.0 ** 2).astype(np.float32))
    eng.set_noise([42 + m for m in range(members)], 0.083, 0.02, 1.0, 5e-4 / (4 * dx * dx))
    eng.set_kernel(kind)
    rng = np.random.default_rng(nx + ny + kind)
    psi = (1e-2 * (rng.standard_normal((members, 1, ny, nx)) +
                   1j * rng.standard_normal((members, 1, ny, nx)))).astype(np.complex64)
    res = np.full((members, 1, ny, nx), 0.1, dtype=np.float32)
    return eng, psi, res


@pytest.mark.parametrize("nx,ny,kind", [(1024, 64, 2), (256, 64, 2), (1024, 64, 3), (2048, 32, 2)],
                         ids=["full-width-1024", "full-width-256", "four-sites-1024", "cluster-2048"])
def test_zero_poll_limit_reports_timeout_and_solver_recovers(cuda_lib, nx, ny, kind):
    from polarism_gb300 import _lib

    steps = 6
    scales = np.full((steps, 3, 1), 0.05)
    eng, psi, res = _rk4(nx, ny, kind)
    assert eng.kernel() == kind
    eng.set_state(psi, res)
    eng.set_wait_limit(0)
    t0 = time.perf_counter()
    eng.advance(0, steps, scales)
    status = eng.lib.pg_synchronize(eng.handle)
    elapsed = time.perf_counter() - t0
    assert status == _lib.PG_ERR_TIMEOUT, (status, eng.lib.pg_last_error())
    assert b"timed out" in eng.lib.pg_last_error()
    assert elapsed < 10.0, f"the failed advance took {elapsed:.1f} s"

    with pytest.raises(RuntimeError, match="or 100000"):
        eng.set_wait_limit(5)
    eng.set_wait_limit(100000)
    eng.set_state(psi, res)
    eng.advance(0, steps, scales)
    got_psi, got_res = eng.get_state()
    ref, _, _ = _rk4(nx, ny, kind)
    ref.set_state(psi, res)
    ref.advance(0, steps, scales)
    exp_psi, exp_res = ref.get_state()
    assert np.array_equal(got_psi, exp_psi)
    assert np.array_equal(got_res, exp_res)


def test_sweep_zero_poll_limit_reports_timeout_and_recovers(cuda_lib):
    from polarism_gb300 import _lib
    from polarism_gb300.engine import MemberPhysics
    from polarism_gb300.sweep import SweepEngine

    grids = [(64, 64, 0.5, 0.5), (128, 128, 0.5, 0.5), (64, 64, 0.5, 0.5)]
    rng = np.random.default_rng(3)
    psi = [(1e-2 * (rng.standard_normal((g[1], g[0])) + 1j * rng.standard_normal((g[1], g[0]))))
           .astype(np.complex64) for g in grids]
    res = [np.full((g[1], g[0]), 0.1, dtype=np.float32) for g in grids]
    env = [np.ones((g[1], g[0]), dtype=np.float32) for g in grids]
    steps = 4
    scales = np.full((steps, 3, len(grids)), 0.05)

    def make():
        eng = SweepEngine(grids, [MemberPhysics()] * len(grids), 1e-3)
        eng.set_pump(env)
        eng.set_noise([7, 8, 9], [0.083] * 3, [0.02] * 3, [1.0] * 3)
        eng.set_state(psi, res)
        return eng

    eng = make()
    eng.set_wait_limit(0)
    eng.advance(0, steps, scales)
    status = eng._lib.pg_sweep_synchronize(eng._h)
    assert status == _lib.PG_ERR_TIMEOUT, (status, eng._lib.pg_last_error())
    eng.set_wait_limit(100000)
    eng.set_state(psi, res)
    eng.advance(0, steps, scales)
    got = eng.get_state()
    ref = make()
    ref.advance(0, steps, scales)
    exp = ref.get_state()
    for a, b in zip(got, exp):
        for x, y in zip(a, b):
            assert np.array_equal(x, y)
