"""Philox-4x32-10 and the truncated-Wigner increment (oracle; test infrastructure).

Restates ``polarism/noise/philox.py`` and ``polarism/noise/stochastic.py``:

* ``philox4x32``     -- ``polarism/noise/philox.py:7-27`` (Random123 Philox-4x32,
  10 rounds, multipliers 0xD2511F53 / 0xCD9E8D57, Weyl keys 0x9E3779B9 /
  0xBB67AE85).
* ``counter_words``  -- ``polarism/noise/philox.py:30-38``
  (counter = (cell, step_lo, step_hi, stream)).
* ``normal_pair``    -- ``polarism/noise/philox.py:41-56`` (24-bit uniforms in
  single precision, 53-bit uniforms from two words in double precision,
  Box-Muller).
* ``wigner_increment`` -- ``polarism/noise/stochastic.py:40-96``
  (sigma**2 = s (gamma_C + R n_A) dt / (4 dV)).
"""
from __future__ import annotations

import numpy as np

_M0 = np.uint64(0xD2511F53)
_M1 = np.uint64(0xCD9E8D57)
_W0 = 0x9E3779B9
_W1 = 0xBB67AE85
_MASK32 = np.uint64(0xFFFFFFFF)
_SHIFT32 = np.uint64(32)


def philox4x32(counter, key: int) -> np.ndarray:
    """Return the four output words for every four-word counter (``(..., 4)`` uint32)."""
    words = np.asarray(counter, dtype=np.uint32)
    if words.shape[-1] != 4:
        raise ValueError("Philox counters must have four uint32 words")
    x = [words[..., i].astype(np.uint64) for i in range(4)]
    k0 = int(key) & 0xFFFFFFFF
    k1 = (int(key) >> 32) & 0xFFFFFFFF
    for r in range(10):
        lo_hi0 = x[0] * _M0            # exact 64-bit products of two 32-bit words
        lo_hi1 = x[2] * _M1
        hi0, lo0 = lo_hi0 >> _SHIFT32, lo_hi0 & _MASK32
        hi1, lo1 = lo_hi1 >> _SHIFT32, lo_hi1 & _MASK32
        x = [hi1 ^ x[1] ^ np.uint64(k0), lo1, hi0 ^ x[3] ^ np.uint64(k1), lo0]
        if r < 9:
            k0 = (k0 + _W0) & 0xFFFFFFFF
            k1 = (k1 + _W1) & 0xFFFFFFFF
    return np.stack([w.astype(np.uint32) for w in x], axis=-1)


def counter_words(cells, step: int, stream: int = 1) -> np.ndarray:
    """Counters (cell, step low word, step high word, stream) for each cell index."""
    cells = np.asarray(cells, dtype=np.uint32)
    out = np.empty((*cells.shape, 4), dtype=np.uint32)
    out[..., 0] = cells
    out[..., 1] = np.uint32(int(step) & 0xFFFFFFFF)
    out[..., 2] = np.uint32((int(step) >> 32) & 0xFFFFFFFF)
    out[..., 3] = np.uint32(stream)
    return out


def normal_pair(words, precision: str):
    """Two standard normals per word quadruple, in the precision's own arithmetic."""
    w = np.asarray(words, dtype=np.uint32)
    if precision == "single":
        f = np.float32
        u1 = ((w[..., 0] >> 8).astype(f) + f(1)) * f(2.0 ** -24)
        u2 = ((w[..., 1] >> 8).astype(f) + f(1)) * f(2.0 ** -24)
        r = np.sqrt(f(-2) * np.log(u1))
        theta = f(2.0 * np.pi) * u2
        return r * np.cos(theta), r * np.sin(theta)
    if precision != "double":
        raise ValueError(f"unknown precision {precision!r}")
    u1 = ((w[..., 0] >> 5).astype(np.float64) * 67108864.0
          + (w[..., 1] >> 6).astype(np.float64) + 1.0) * 2.0 ** -53
    u2 = ((w[..., 2] >> 5).astype(np.float64) * 67108864.0
          + (w[..., 3] >> 6).astype(np.float64) + 1.0) * 2.0 ** -53
    r = np.sqrt(-2.0 * np.log(u1))
    theta = 2.0 * np.pi * u2
    return r * np.cos(theta), r * np.sin(theta)


def wigner_increment(field, active, step: int, seeds, gamma, scattering, strength,
                     dt: float, cell_volume: float, precision: str,
                     normals_precision: str | None = None) -> None:
    """Add one Wigner increment in place to a canonical ``(B, C, ny, nx)`` field.

    ``active`` is the active reservoir density ``(B, 1 or C, ny, nx)`` (or a scalar 0).
    ``normals_precision`` chooses which uniform construction draws the normals;
    by default it equals ``precision`` as in the reference.  The FP64 oracle run
    that an FP32 device run is compared with passes ``"single"`` here so that
    both see the same noise realisation (the two constructions use different
    counter words for the angle).
    """
    normals_precision = normals_precision or precision
    rdt = np.float32 if precision == "single" else np.float64
    members, comps = field.shape[:2]
    spatial = int(np.prod(field.shape[2:]))
    for m in range(members):
        if float(strength[m]) == 0.0:
            continue
        for c in range(comps):
            words = philox4x32(counter_words(np.arange(spatial), step, 1 + c), int(seeds[m]))
            re, im = normal_pair(words, normals_precision)
            re = re.astype(rdt)
            im = im.astype(rdt)
            if np.ndim(active) == 0:
                dens = rdt(0)
            else:
                dens = np.asarray(active[m, c if active.shape[1] == comps else 0],
                                  dtype=rdt).reshape(-1)
            sigma = np.sqrt(rdt(strength[m]) * (rdt(gamma[m]) + rdt(scattering[m]) * dens)
                            * rdt(dt / (4.0 * cell_volume)))
            field[m, c] += (sigma * (re + 1j * im)).reshape(field.shape[2:]).astype(field.dtype)
