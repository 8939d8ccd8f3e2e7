"""Finalisation of the FP64 device accumulators into Polarism's observables.

The sums are accumulated on the GPU in FP64 (``pg_accumulate``); these host functions turn
them into the reference's results, with the same normalisation and truncated-Wigner vacuum
subtraction:

* ``momentum_distribution`` / ``g1`` -- ``polarism/results/accumulators.py:119-131`` and
  ``polarism/analysis/correlations.py:11-21``
* ``density_moments`` / ``g2``       -- ``polarism/results/accumulators.py:156-172`` and
  ``polarism/analysis/correlations.py:24-29``
"""
from __future__ import annotations

import numpy as np


def momentum_distribution(sum_k, samples, cell, cells, strength=None):
    """Mean particles per mode, centred (fftshift); minus s/2 per mode when Wigner noise ran."""
    value = np.fft.fftshift(np.asarray(sum_k) * (cell / (cells * samples)), axes=(-2, -1))
    if strength is not None:
        value = value - np.asarray(strength).reshape((-1,) + (1,) * (value.ndim - 1)) / 2
    return value


def g1(n_k):
    """Normalised, centred first-order spatial correlation of a centred n(k)."""
    n_k = np.asarray(n_k)
    axes = (-2, -1)
    correlation = np.fft.ifftn(np.fft.ifftshift(n_k, axes=axes), axes=axes)
    origin = correlation[..., 0, 0]
    denominator = np.where(np.abs(origin) > 1e-30, origin, 1)
    normalised = np.where(np.abs(origin)[..., None, None] > 1e-30,
                          correlation / denominator[..., None, None], 0)
    return np.fft.fftshift(normalised, axes=axes)


def density_moments(sum_rho, sum_rho2, samples, delta=None):
    """(mean density, mean squared density) with the Wigner vacuum subtraction
    <n^2> - 2 delta <n> + delta^2 / 2 and <n> - delta / 2, delta = s / dV."""
    mean = np.asarray(sum_rho) / samples
    squared = np.asarray(sum_rho2) / samples
    if delta is not None:
        d = np.asarray(delta).reshape((-1,) + (1,) * (mean.ndim - 1))
        squared = squared - 2 * d * mean + d * d / 2
        mean = mean - d / 2
    return mean, squared


def g2(mean, squared_mean):
    """Second-order correlation, zero where the density is negligible."""
    mean = np.asarray(mean)
    squared_mean = np.asarray(squared_mean)
    return np.where(mean > 1e-30, squared_mean / np.maximum(mean * mean, 1e-60), 0)
