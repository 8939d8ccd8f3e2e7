"""Host finalisation of the accumulated observables (no GPU needed).

Mirrors ``tests/unit/test_accumulators.py`` (complex-Gaussian g2 = 2, Wigner vacuum
subtraction, g1 of a single mode) on the reference formulas restated in
``polarism_gb300.observables``.
"""
from __future__ import annotations

import numpy as np

from polarism_gb300 import observables as obs


def test_complex_gaussian_g2_is_two():
    rng = np.random.default_rng(0)
    samples = 4000
    psi = (rng.standard_normal((samples, 8, 8)) + 1j * rng.standard_normal((samples, 8, 8))) / np.sqrt(2)
    rho = np.abs(psi) ** 2
    mean, squared = obs.density_moments(rho.sum(0), (rho ** 2).sum(0), samples)
    g = obs.g2(mean, squared)
    assert abs(g.mean() - 2.0) < 0.05


def test_wigner_vacuum_subtraction_removes_vacuum():
    """A pure vacuum field (variance delta/2 per quadrature sum) has <n> = 0, <n^2> = 0."""
    rng = np.random.default_rng(1)
    samples, delta = 20000, 3.0
    psi = np.sqrt(delta / 2) * (rng.standard_normal((samples, 4, 4))
                                + 1j * rng.standard_normal((samples, 4, 4))) / np.sqrt(2)
    rho = np.abs(psi) ** 2
    mean, squared = obs.density_moments(rho.sum(0)[None], (rho ** 2).sum(0)[None], samples,
                                        delta=np.asarray([delta]))
    assert abs(mean.mean()) < 0.02 * delta and abs(squared.mean()) < 0.05 * delta ** 2


def test_single_mode_g1_is_one():
    n_k = np.zeros((1, 8, 8))
    n_k[0, 4, 5] = 7.0
    g = obs.g1(n_k)
    assert np.allclose(np.abs(g), 1.0)


def test_momentum_distribution_normalisation():
    sum_k = np.full((1, 4, 4), 8.0)
    value = obs.momentum_distribution(sum_k, 2, cell=0.5, cells=16, strength=np.asarray([1.0]))
    assert np.allclose(value, 8.0 * 0.5 / (16 * 2) - 0.5)


def test_finalisation_matches_the_reference_accumulators():
    """The reference's own MomentumDistribution and G2Accumulator results
    (``polarism/results/accumulators.py:95-172``; two members with Wigner strengths 1 and 0.5,
    cell 0.9375, six samples of a noisy rk4-fdm run, ``tests/golden/accumulators.npz``):
    the sums formed again from the sampled fields, then n(k), g1, the corrected density
    moments and g2 from this module, agree to 1e-12."""
    from polarism_gb300 import observables as obs
    from tests.conftest import load_golden

    g = load_golden("accumulators")
    fields = g["fields"][:, :, 0]  # (samples, members, ny, nx)
    samples = int(g["samples"])
    rho = np.abs(fields) ** 2
    fk = np.fft.fft2(fields, axes=(-2, -1))
    sums = {"sum_density": rho.sum(0), "sum_density_squared": (rho * rho).sum(0),
            "sum_k": (fk.real ** 2 + fk.imag ** 2).sum(0)}
    for name, value in sums.items():
        np.testing.assert_allclose(value, g[name], rtol=1e-13, atol=0)
    n_k = obs.momentum_distribution(sums["sum_k"], samples, float(g["cell"]), int(g["cells"]),
                                    g["strength"])
    mean, squared = obs.density_moments(sums["sum_density"], sums["sum_density_squared"], samples,
                                        g["delta"])
    for name, value in (("momentum_distribution", n_k), ("g1", obs.g1(n_k)),
                        ("density_mean", mean), ("density_squared_mean", squared),
                        ("g2", obs.g2(mean, squared))):
        ref = g[name]
        assert np.linalg.norm(value - ref) <= 1e-12 * np.linalg.norm(ref), name
