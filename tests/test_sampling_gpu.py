"""The device-resident steady-state monitor on the GPU (``pg_steady_update`` / ``_poll`` /
``_results``, driven by ``polarism_gb300.sampling.run_to_steady``).

Mirrors the sampling path of ``SimulationController.run`` (``polarism/simulation_controller.py:
1063-1130``, ``_check_steady_state`` :710-734, ``_record_stops`` :698-708): uniform condensates
relaxing to the fixed point of a uniform pump at three pump strengths, so members stop at
different checks.  Checks: the device loop stops every member on the same step as a loop that
reads every check back to the host and decides there (bitwise equal final state, FP32 and FP64);
FP64 stop steps equal the FP64 oracle's; a halted engine resumes from the halt step.
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import gpe
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

P = dict(hbar=0.6582119514, m_eff=0.284, g_C=0.001, g_R=0.002, g_I=0.0, R=0.02, gamma_C=0.083,
         gamma_R=0.5)
N, DX, DT, INTERVAL, RTOL, STEPS = 16, 1.0, 0.05, 20, 5e-3, 4000
P0 = np.array([4.0, 8.0, 16.0])


def _initial():
    x = (np.arange(N) - N / 2) * DX
    psi = np.broadcast_to((1.0 + 0.02 * np.cos(2 * np.pi * x / (N * DX)))[None, :], (N, N))
    psi = np.broadcast_to(psi.astype(np.complex128), (3, 1, N, N)).copy()
    return psi, np.full((3, 1, N, N), 4.0)


def _engine(precision):
    from polarism_gb300.engine import MemberPhysics, RK4Engine

    eng = RK4Engine(N, N, 3, DX, DX, DT, MemberPhysics(**P), precision)
    eng.set_pump(np.ones((N, N), dtype=eng.real))
    psi, n0 = _initial()
    eng.set_state(psi.astype(eng.complex), n0.astype(eng.real))
    return eng


def _scales(a, b):
    return np.broadcast_to(P0, (b - a, 3, 3))


def _host_loop(eng, min_time=0.0):
    """The reference's loop with every check read back and decided on the host."""
    stop = np.full(3, -1)
    step = 0
    first = True
    while step < STEPS and not (stop >= 0).all():
        eng.advance(step, INTERVAL, _scales(step, step + INTERVAL))
        step += INTERVAL
        rd, rn, norms = eng.steady_check()
        if not first and step * DT >= min_time:
            reached = (norms < 1e-30) | ((rn < RTOL) & (rd < RTOL))
            stop[reached & (stop < 0)] = step
        first = False
    return stop, step


@pytest.mark.parametrize("precision", ["single", "double"])
@pytest.mark.parametrize("min_time", [0.0, 70.0])
def test_device_loop_matches_host_decisions(cuda_lib, precision, min_time):
    from polarism_gb300 import sampling

    dev = _engine(precision)
    run = sampling.run_to_steady(dev, 0, STEPS, _scales, DT, INTERVAL, RTOL, min_time=min_time)
    ref = _engine(precision)
    ref.steady_reset()
    stop, final = _host_loop(ref, min_time)
    assert run.halted and (run.stop_steps >= 0).all()
    if min_time == 0.0:
        assert len(set(run.stop_steps.tolist())) == 3  # staggered stops
    else:
        assert (run.stop_steps * DT >= min_time).all() and min(run.stop_steps) * DT == min_time
    assert run.stop_steps.tolist() == stop.tolist() and run.final_step == final
    np.testing.assert_allclose(run.stop_times, stop * DT)
    p1, n1 = dev.get_state()
    p2, n2 = ref.get_state()
    assert np.array_equal(p1, p2) and np.array_equal(n1, n2)
    stopped, done = dev.steady_poll()
    assert stopped == 3 and done == final // INTERVAL
    dev.close()
    ref.close()


def test_fp64_stop_steps_match_the_oracle(cuda_lib):
    from polarism_gb300 import sampling

    eng = _engine("double")
    run = sampling.run_to_steady(eng, 0, STEPS, _scales, DT, INTERVAL, RTOL)
    psi, n0 = _initial()
    fields = (n0,)
    p0 = P0[:, None, None, None]
    stop = np.full(3, -1)
    old = old_norm = None
    step = 0
    margin = np.inf
    while not (stop >= 0).all():
        psi, fields = gpe.rk4_advance(psi, fields, lambda t: p0, 0.0, P, DX, DX, DT, step, INTERVAL)
        step += INTERVAL
        rho = np.abs(psi) ** 2
        norms = rho.sum(axis=(1, 2, 3)) * DX * DX
        if old is not None:
            rd = np.sqrt(((rho - old) ** 2).sum(axis=(1, 2, 3))) / np.sqrt((old ** 2).sum(axis=(1, 2, 3)))
            rn = np.abs(norms - old_norm) / old_norm
            margin = min(margin, np.min(np.abs(np.concatenate([rd, rn]) / RTOL - 1)))
            stop[((rn < RTOL) & (rd < RTOL)) & (stop < 0)] = step
        old, old_norm = rho, norms
    assert margin > 1e-8  # no decision sits on the threshold
    assert run.stop_steps.tolist() == stop.tolist() and run.final_step == step
    p_gpu, n_gpu = eng.get_state()
    assert rel_l2(p_gpu, psi) < 1e-10 and rel_l2(n_gpu, fields[0]) < 1e-10
    eng.close()


def test_halted_engine_resumes_from_the_halt_step(cuda_lib):
    from polarism_gb300 import sampling

    dev = _engine("single")
    run = sampling.run_to_steady(dev, 0, STEPS, _scales, DT, INTERVAL, RTOL, poll_every=1000)
    assert run.halted and run.checks > run.final_step // INTERVAL  # work was queued past the halt
    dev.advance(run.final_step, 30, _scales(0, 30))
    ref = _engine("single")
    ref.advance(0, run.final_step, _scales(0, run.final_step))
    ref.advance(run.final_step, 30, _scales(0, 30))
    p1, n1 = dev.get_state()
    p2, n2 = ref.get_state()
    assert np.array_equal(p1, p2) and np.array_equal(n1, n2)
    dev.close()
    ref.close()
