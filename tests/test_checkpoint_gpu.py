"""Checkpoint format 2 of the GPU-resident state (``polarism/simulation_controller.py:736-923``):
a run interrupted, written to disk, read back into a fresh engine and continued equals the run
that was never interrupted -- field, both reservoir fields, the device steady-state monitor
(reference density, norms, stop steps) and the FP64 accumulator sums, bit for bit."""
from __future__ import annotations

import numpy as np
import pytest

from polarism_gb300 import checkpoint

pytestmark = pytest.mark.gpu

P = dict(hbar=0.6582119514, m_eff=0.284, g_C=0.001, g_R=0.002, g_I=0.0, R=0.02, gamma_C=0.083,
         gamma_R=0.005, gamma_I=0.001, gamma_A=0.005, R_IA=0.05, R_AI=0.0025)
N, M, DX, DT, CHUNK = 128, 3, 0.8, 2e-3, 16


def _engine(precision):
    from polarism_gb300.engine import MemberPhysics, RK4Engine

    eng = RK4Engine(N, N, M, DX, DX, DT, MemberPhysics(**P), precision, reservoir="double")
    x = (np.arange(N) - N / 2) * DX
    eng.set_pump(np.exp(-0.5 * (x[None, :] ** 2 + x[:, None] ** 2) / 400.0).astype(eng.real))
    eng.set_noise([7, 8, 9], P["gamma_C"], P["R"], 1.0, DT / (4 * DX * DX))
    rng = np.random.default_rng(2)
    psi = 0.1 * (rng.standard_normal((M, 1, N, N)) + 1j * rng.standard_normal((M, 1, N, N)))
    eng.set_state(psi.astype(eng.complex), np.zeros((2, M, 1, N, N), dtype=eng.real))
    eng.steady_reset()
    return eng


def _chunks(eng, start, count, rtol):
    step = start
    for _ in range(count):
        eng.advance(step, CHUNK, np.full((CHUNK, 3, M), 2.0))
        step += CHUNK
        eng.steady_update(step, record=True, rtol=rtol)
        eng.accumulate(density=True, momentum=True)
    return step


@pytest.mark.parametrize("precision", ["single", "double"])
def test_resume_from_checkpoint_equals_uninterrupted_run(cuda_lib, tmp_path, precision):
    rtol = 0.3  # loose enough that some members stop within the run
    whole = _engine(precision)
    _chunks(whole, 0, 8, rtol)
    first = _engine(precision)
    step = _chunks(first, 0, 4, rtol)
    ck = checkpoint.capture(first, step=step, t0=0.0, dt=DT, reservoir_names=("nA", "nI"),
                            reservoir_type="double", steady_last_step=step,
                            accumulators={"g2": {"t_first": DT * CHUNK, "t_last": DT * step},
                                          "momentum-distribution": {"t_first": DT * CHUNK,
                                                                    "t_last": DT * step}})
    path = checkpoint.save(tmp_path / "ck.npz", ck)
    first.close()
    resumed = _engine(precision)
    back = checkpoint.load(path)
    assert back["attrs"]["step"] == step and back["data"]["steady_density"].shape == (M, N, N)
    assert checkpoint.restore(resumed, back) == step
    _chunks(resumed, step, 4, rtol)
    for a, b in zip(whole.get_state(), resumed.get_state()):
        assert np.array_equal(a, b)
    r_whole, r_res = whole.steady_results(), resumed.steady_results()
    for a, b in zip(r_whole[:4], r_res[:4]):
        assert np.array_equal(a, b)
    assert (r_whole[3] >= 0).any()  # the monitor's stop steps crossed the checkpoint
    for kind in ("rho", "rho2", "k"):
        s1, n1 = whole.accumulator_sums(kind)
        s2, n2 = resumed.accumulator_sums(kind)
        assert n1 == n2 == 8 and np.array_equal(s1, s2)
    whole.close()
    resumed.close()
