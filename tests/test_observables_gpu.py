"""FP64 device observables against NumPy on the same fields.

Mirrors ``tests/unit/test_accumulators.py:41-97`` (plane-wave sum rule, batched equals
single) and the steady-state criterion of ``polarism/simulation_controller.py:710-734``.
The sums are FP64 on the device; the comparison is at 1e-12 (FP64 state) and 1e-6 (FP32
state, spectra through the FP32 FFT).
"""
from __future__ import annotations

import numpy as np
import pytest

from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


def _engine(precision, members=2, nx=64, ny=32):
    from polarism_gb300.engine import Engine, MemberPhysics

    rng = np.random.default_rng(4)
    eng = Engine(nx, ny, members, 0.5, 0.7, 1e-3, MemberPhysics(), precision)
    eng.set_pump(np.abs(rng.standard_normal((ny, nx))).astype(eng.real))
    psi = (rng.standard_normal((members, 1, ny, nx)) + 1j * rng.standard_normal((members, 1, ny, nx)))
    eng.set_state(psi.astype(eng.complex), np.zeros((members, 1, ny, nx), eng.real))
    return eng


@pytest.mark.parametrize("precision,tol", [("double", 1e-12), ("single", 1e-6)])
def test_accumulators_match_numpy(cuda_lib, precision, tol):
    eng = _engine(precision)
    rho_sum = rho2_sum = k_sum = 0
    for k in range(3):
        psi, _ = eng.get_state()
        p = psi.astype(np.complex128)
        rho = p.real ** 2 + p.imag ** 2
        rho_sum = rho_sum + rho
        rho2_sum = rho2_sum + rho * rho
        fk = np.fft.fft2(p, axes=(-2, -1))
        k_sum = k_sum + fk.real ** 2 + fk.imag ** 2
        eng.accumulate(density=True, momentum=True)
        eng.advance(k, 2, np.full((2, 3, eng.members), 0.1))
    s_rho, n_rho = eng.accumulator_sums("rho")
    s_rho2, _ = eng.accumulator_sums("rho2")
    s_k, n_k = eng.accumulator_sums("k")
    assert n_rho == 3 and n_k == 3
    assert rel_l2(s_rho, rho_sum) < 1e-14
    assert rel_l2(s_rho2, rho2_sum) < 1e-14
    assert rel_l2(s_k, k_sum) < tol
    eng.accumulator_reset()
    eng.accumulate(density=True)
    assert eng.accumulator_sums("rho")[1] == 1


def test_plane_wave_sum_rule(cuda_lib):
    """A plane wave puts all of |FFT psi|^2 = N^2 |A|^2 in one mode."""
    from polarism_gb300.engine import Engine, MemberPhysics

    nx, ny = 32, 16
    eng = Engine(nx, ny, 1, 1.0, 1.0, 1e-3, MemberPhysics(), "double")
    x = np.arange(nx)
    psi = np.broadcast_to(0.5 * np.exp(2j * np.pi * 3 * x / nx), (1, 1, ny, nx)).copy()
    eng.set_pump(np.zeros((ny, nx)))
    eng.set_state(psi, np.zeros((1, 1, ny, nx)))
    eng.accumulate(density=False, momentum=True)
    s_k, _ = eng.accumulator_sums("k")
    expected = np.zeros((ny, nx))
    expected[0, 3] = (nx * ny * 0.5) ** 2
    assert np.allclose(s_k[0, 0], expected, atol=1e-9 * expected.max())


@pytest.mark.parametrize("precision", ["double", "single"])
def test_norms_and_steady_state(cuda_lib, precision):
    eng = _engine(precision)
    psi0, _ = eng.get_state()
    rd, rn, n0 = eng.steady_check()
    assert np.all(np.isinf(rd)) and np.all(np.isinf(rn))
    cell = 0.5 * 0.7
    rho0 = np.abs(psi0.astype(np.complex128)) ** 2
    expect = rho0.reshape(eng.members, -1).sum(axis=1) * cell
    tol = 1e-12 if precision == "double" else 1e-6
    assert np.allclose(n0, expect, rtol=tol)
    assert np.allclose(eng.norms(), expect, rtol=tol)
    eng.advance(0, 3, np.full((3, 3, eng.members), 0.1))
    psi1, _ = eng.get_state()
    rd, rn, n1 = eng.steady_check()
    rho1 = np.abs(psi1.astype(np.complex128)) ** 2
    if precision == "single":
        rho0 = (np.abs(psi0) ** 2).astype(np.float64)
        rho1 = (psi1.real * psi1.real + psi1.imag * psi1.imag).astype(np.float64)
    for m in range(eng.members):
        d = np.sqrt(((rho1[m] - rho0[m]) ** 2).sum()) / np.sqrt((rho0[m] ** 2).sum())
        assert abs(rd[m] - d) <= 1e-6 * d + 1e-12
        assert abs(rn[m] - abs(n1[m] - n0[m]) / n0[m]) < 1e-9


def test_field_norms_on_caller_device_arrays(cuda_lib):
    import torch

    from polarism_gb300 import _lib

    lib = _lib.load()
    rng = np.random.default_rng(9)
    for dtype, prec in ((torch.complex64, _lib.PG_SINGLE), (torch.complex128, _lib.PG_DOUBLE)):
        host = rng.standard_normal((3, 1, 40, 24)) + 1j * rng.standard_normal((3, 1, 40, 24))
        dev = torch.as_tensor(host, dtype=dtype, device="cuda")
        out = torch.zeros(3, dtype=torch.float64, device="cuda")
        _lib.check(lib.pg_field_norms(dev.data_ptr(), prec, 3, 40 * 24, 0.25, out.data_ptr(), None),
                   "pg_field_norms")
        expect = (np.abs(dev.cpu().numpy().astype(np.complex128)) ** 2).reshape(3, -1).sum(1) * 0.25
        assert np.allclose(out.cpu().numpy(), expect, rtol=1e-12)


def test_device_sums_finalise_to_the_reference_accumulators(cuda_lib):
    """The sampled fields of ``tests/golden/accumulators.npz`` through the device's FP64
    accumulation (``pg_accumulate``), finalised on the host, against the reference's own
    MomentumDistribution / G2Accumulator results at 1e-12."""
    from polarism_gb300 import observables as obs
    from polarism_gb300.engine import Engine, MemberPhysics
    from tests.conftest import load_golden

    g = load_golden("accumulators")
    fields = g["fields"]  # (samples, members, 1, ny, nx) complex128
    members, ny, nx = fields.shape[1], fields.shape[-2], fields.shape[-1]
    eng = Engine(nx, ny, members, 1.25, 0.75, 1e-3, MemberPhysics(), "double")
    res = np.zeros((members, 1, ny, nx))
    for f in fields:
        eng.set_state(np.ascontiguousarray(f), res)
        eng.accumulate(density=True, momentum=True)
    (s_rho, n), (s_rho2, _), (s_k, _) = (eng.accumulator_sums(k) for k in ("rho", "rho2", "k"))
    assert n == int(g["samples"])
    n_k = obs.momentum_distribution(s_k[:, 0], n, float(g["cell"]), int(g["cells"]), g["strength"])
    mean, squared = obs.density_moments(s_rho[:, 0], s_rho2[:, 0], n, g["delta"])
    for name, value in (("momentum_distribution", n_k), ("g1", obs.g1(n_k)),
                        ("density_mean", mean), ("density_squared_mean", squared),
                        ("g2", obs.g2(mean, squared))):
        assert rel_l2(value, g[name]) < 1e-12, name
