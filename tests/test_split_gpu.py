"""GPU parity of the split-step Fourier passes (both Strang orderings), through the C ABI.

Mirrors ``tests/crosscheck/test_split_step_fft_cuda.py:46-129`` (the GPU ordering
against an independent NumPy composition at 1e-10 FP64 / 1e-5 FP32, bitwise repeat)
and the reference CPU ordering's own output (``split-step-fft``).  Tolerances: FP64
1e-10 and FP32 1e-4 relative L2 against the FP64 oracle; graph and plain launches
and batch members are compared bitwise.
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import gpe
from tests.conftest import load_golden, rel_l2

pytestmark = pytest.mark.gpu

P = dict(hbar=0.6582119514, m_eff=0.284, g_C=0.001, g_R=0.002, g_I=0.0, R=0.02, gamma_C=0.083,
         gamma_R=0.005)


def _grid(nx, ny, dx, dy):
    kx = 2 * np.pi * np.fft.fftfreq(nx, d=dx)
    ky = 2 * np.pi * np.fft.fftfreq(ny, d=dy)
    KX, KY = np.meshgrid(kx, ky, indexing="xy")
    return KX ** 2 + KY ** 2


def _case(nx=32, ny=16, seed=3, potential=True):
    rng = np.random.default_rng(seed)
    dx, dy, dt = 1.25, 0.9, 4e-3
    psi0 = 0.2 * (rng.standard_normal((1, 1, ny, nx)) + 1j * rng.standard_normal((1, 1, ny, nx)))
    res0 = np.abs(rng.standard_normal((1, 1, ny, nx))) * 0.05
    env = np.exp(-0.5 * (((np.arange(nx) - nx / 2) * dx) ** 2)[None, :] / 16.0
                 - 0.5 * (((np.arange(ny) - ny / 2) * dy) ** 2)[:, None] / 9.0)
    pot = None
    if potential:
        pot = 0.01 * np.cos(np.arange(nx) * 2 * np.pi / nx)[None, :] - 0.002j * (
            1 + np.sin(np.arange(ny) * 2 * np.pi / ny))[:, None]
    return dict(dx=dx, dy=dy, dt=dt, psi0=psi0, res0=res0, env=env, pot=pot,
                k2=_grid(nx, ny, dx, dy))


def _coeff(t):
    return 0.3 * (1.0 + 0.5 * np.sin(20.0 * t))


def _engine(c, precision, members=1, seed=77, noise=True):
    from polarism_gb300 import _lib
    from polarism_gb300.engine import Engine, MemberPhysics

    ny, nx = c["psi0"].shape[-2:]
    eng = Engine(nx, ny, members, c["dx"], c["dy"], c["dt"], MemberPhysics(**P), precision,
                 potential=_lib.PG_POT_NONE if c["pot"] is None else _lib.PG_POT_COMPLEX)
    eng.set_pump(c["env"].astype(eng.real))
    if c["pot"] is not None:
        eng.set_potential(c["pot"].astype(eng.complex))
    if noise:
        eng.set_noise([seed] * members, P["gamma_C"], P["R"], 1.0,
                      c["dt"] / (4 * c["dx"] * c["dy"]))
    eng.set_state(np.repeat(c["psi0"], members, 0).astype(eng.complex),
                  np.repeat(c["res0"], members, 0).astype(eng.real))
    return eng


def _half_scales(dt, start, steps, members=1):
    out = np.empty((steps, 2, members))
    for k in range(steps):
        t = (start + k) * dt
        out[k, 0] = _coeff(t + dt / 4)
        out[k, 1] = _coeff(t + 3 * dt / 4)
    return out


def _oracle(c, ordering, steps, normals, noise=True, seed=77):
    dx, dy, dt = c["dx"], c["dy"], c["dt"]
    nz = gpe.Noise([seed], [P["gamma_C"]], [P["R"]], [1.0], dt, dx * dy, "double",
                   normals_precision=normals) if noise else None
    pot = 0.0 if c["pot"] is None else c["pot"]
    return gpe.split_advance(ordering, c["psi0"].copy(), (c["res0"].copy(),),
                             lambda t: c["env"] * _coeff(t), pot, P, c["k2"], dx, dy, dt, 0,
                             steps, noise=nz)


@pytest.mark.parametrize("precision,tol", [("double", 1e-10), ("single", 1e-4)])
@pytest.mark.parametrize("ordering", ["cpu", "kouter"])
def test_split_matches_oracle(cuda_lib, precision, tol, ordering):
    c = _case()
    steps = 10
    eng = _engine(c, precision)
    eng.split_advance(0 if ordering == "cpu" else 1, 0, steps, _half_scales(c["dt"], 0, steps))
    psi, res = eng.get_state()
    if ordering == "kouter":
        assert eng.state_kind()
        psi = np.fft.ifft2(psi.astype(np.complex128), axes=(-2, -1))
    psi_o, f_o = _oracle(c, ordering, steps, precision)
    assert rel_l2(psi, psi_o) < tol
    assert rel_l2(res, f_o[0]) < tol


@pytest.mark.parametrize("potential", [False, True])
@pytest.mark.parametrize("ordering", ["cpu", "kouter"])
@pytest.mark.parametrize("ny,nx", [(1024, 16), (16, 1024)])
def test_split_1024_site_passes_match_oracle(cuda_lib, ny, nx, ordering, potential):
    """FP32 rows and columns of 1024 sites run the register-resident four-step passes; the
    column pass's local step runs in batches of sites (one reservoir, one laser, no potential)
    or a site at a time (with a potential).  Against the FP64 oracle at 1e-4."""
    c = _case(nx=nx, ny=ny, seed=11, potential=potential)
    steps = 6
    eng = _engine(c, "single")
    eng.split_advance(0 if ordering == "cpu" else 1, 0, steps, _half_scales(c["dt"], 0, steps))
    psi, res = eng.get_state()
    eng.close()
    if ordering == "kouter":
        psi = np.fft.ifft2(psi.astype(np.complex128), axes=(-2, -1))
    psi_o, f_o = _oracle(c, ordering, steps, "single")
    assert rel_l2(psi, psi_o) < 1e-4
    assert rel_l2(res, f_o[0]) < 1e-4


def test_split_cpu_ordering_matches_reference_output(cuda_lib):
    """The reference's own split-step-fft trajectory (FP64, Wigner on, 32x16)."""
    from polarism_gb300.engine import Engine, MemberPhysics

    g = load_golden("split_cpu_p2")
    p = g["physics"]
    ny, nx = g["psi0"].shape[-2:]
    dx, dy, dt = float(g["dx"]), float(g["dy"]), float(g["dt"])
    eng = Engine(nx, ny, 1, dx, dy, dt, MemberPhysics.from_object(p), "double")
    eng.set_pump(g["envelope"])
    eng.set_noise([int(g["seed"])], p["gamma_C"], p["R"], 1.0, dt / (4 * dx * dy))
    eng.set_state(g["psi0"], g["res0"][0])
    steps = int(g["steps"])
    norms = []
    for k in range(steps):
        eng.split_advance(0, k, 1, np.full((1, 2, 1), float(g["p0"])), use_graphs=False)
        psi, res = eng.get_state()
        norms.append(gpe.norm(psi, dx, dy)[0])
    assert rel_l2(psi, g["psi"]) < 1e-10
    assert rel_l2(res, g["res"][0]) < 1e-10
    assert rel_l2(np.asarray(norms), g["norms"]) < 1e-10


@pytest.mark.parametrize("ordering", [0, 1])
def test_split_graphs_members_and_chunks_bitwise(cuda_lib, ordering):
    c = _case(nx=64, ny=32, seed=5)
    steps = 70  # crosses a 64-step chunk boundary
    scales = _half_scales(c["dt"], 0, steps)
    plain = _engine(c, "single")
    plain.split_advance(ordering, 0, steps, scales, use_graphs=False)
    ref_psi, ref_res = plain.get_state()
    graph = _engine(c, "single", members=3)
    graph.split_advance(ordering, 0, steps, np.repeat(scales, 3, axis=2), use_graphs=True)
    psi, res = graph.get_state()
    for m in range(3):
        assert np.array_equal(psi[m], ref_psi[0]) and np.array_equal(res[m], ref_res[0])


def test_kouter_spectral_state_continues(cuda_lib):
    """Two advances of 5 steps equal one of 10 (spectrum carried between calls)."""
    c = _case(potential=False)
    one = _engine(c, "double")
    one.split_advance(1, 0, 10, _half_scales(c["dt"], 0, 10))
    a, ra = one.get_state()
    two = _engine(c, "double")
    two.split_advance(1, 0, 5, _half_scales(c["dt"], 0, 5))
    two.split_advance(1, 5, 5, _half_scales(c["dt"], 5, 5))
    b, rb = two.get_state()
    assert rel_l2(b, a) < 1e-13 and rel_l2(rb, ra) < 1e-13


@pytest.mark.parametrize("n", [4, 8, 128, 512, 2048])
def test_fft_sizes_against_numpy(cuda_lib, n):
    """Pure kinetic evolution (g = R = gamma = 0) is one FFT round trip per step."""
    from polarism_gb300.engine import Engine, MemberPhysics

    ny = 16 if n >= 512 else n
    rng = np.random.default_rng(n)
    psi0 = rng.standard_normal((1, 1, ny, n)) + 1j * rng.standard_normal((1, 1, ny, n))
    dx, dy, dt = 0.7, 1.3, 0.01
    phys = MemberPhysics(g_C=0.0, g_R=0.0, R=0.0, gamma_C=0.0, gamma_R=0.0)
    eng = Engine(n, ny, 1, dx, dy, dt, phys, "double")
    eng.set_pump(np.zeros((ny, n)))
    eng.set_state(psi0, np.zeros((1, 1, ny, n)))
    eng.split_advance(1, 0, 3, np.zeros((3, 2, 1)))
    spec, _ = eng.get_state()
    k2 = _grid(n, ny, dx, dy)
    expect = np.fft.fft2(psi0, axes=(-2, -1)) * np.exp(-1j * P["hbar"] * k2 * 3 * dt / (2 * P["m_eff"]))
    assert rel_l2(spec, expect) < 1e-12
