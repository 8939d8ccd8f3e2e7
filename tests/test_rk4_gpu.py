"""GPU parity of the fused RK4 kernel and the Philox stream, through the C ABI.

Mirrors the reference's own checks: ``tests/unit/test_noise.py:56-118`` (Philox
words bit-exact, one-step Wigner variance), ``tests/crosscheck/test_rk4_cuda_agreement.py:90-152``
(rk4-cuda vs rk4-fdm at 1e-10 FP64 / 1e-5 FP32, bitwise determinism) and
``tests/crosscheck/test_rk4_cuda_tiled.py:125-133,233-289`` (tiled and staged
paths agree, odd grid sizes).  Tolerances: FP64 1e-10 relative L2 and FP32 1e-4
relative L2 against the FP64 oracle (the spec bar); tile geometries, graph
and plain launches, and batch members are compared bitwise.
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import gpe
from oracle.philox import counter_words, philox4x32
from tests.conftest import load_golden, rel_l2

pytestmark = pytest.mark.gpu


def _engine(g, precision, members=1, noise=True):
    from polarism_gb300.engine import MemberPhysics, RK4Engine

    p = g["physics"]
    ny, nx = g["psi0"].shape[-2:]
    eng = RK4Engine(nx, ny, members, float(g["dx"]), float(g["dy"]), float(g["dt"]),
                    MemberPhysics.from_object(p), precision)
    real = eng.real
    eng.set_pump(np.ascontiguousarray(g["envelope"], dtype=real))
    if noise and bool(g["wigner"]):
        dv = float(g["dx"]) * float(g["dy"])
        eng.set_noise([int(g["seed"])] * members, p["gamma_C"], p["R"], 1.0,
                      float(g["dt"]) / (4 * dv))
    psi0 = np.repeat(g["psi0"], members, axis=0)
    res0 = np.repeat(g["res0"][0], members, axis=0)
    eng.set_state(psi0.astype(eng.complex), res0.astype(real))
    return eng


def _scales(g, steps, members=1):
    return np.full((steps, 3, members), float(g["p0"]))


def test_philox_words_bit_exact(cuda_lib):
    from polarism_gb300.engine import philox_words

    g = load_golden("philox")
    for key, ctr, exp in zip(g["kat_keys"], g["kat_counters"], g["kat_expected"]):
        assert np.array_equal(philox_words(ctr[None], int(key))[0], exp)
    counters = counter_words(np.arange(4096), int(g["batch_step"]))
    assert np.array_equal(philox_words(counters, int(g["batch_key"])), g["batch_words"])
    rng = np.random.default_rng(1)
    random_ctr = rng.integers(0, 2 ** 32, size=(1000, 4), dtype=np.uint64).astype(np.uint32)
    key = int(rng.integers(0, 2 ** 63))
    assert np.array_equal(philox_words(random_ctr, key), philox4x32(random_ctr, key))


@pytest.mark.parametrize("case", ["rk4_fdm", "rk4_fdm_quiet"])
def test_fp64_matches_reference_rk4_fdm(cuda_lib, case):
    """FP64 device run vs the reference's own rk4-fdm output (1e-10)."""
    g = load_golden(case)
    steps = int(g["steps"])
    eng = _engine(g, "double")
    norms = []
    for k in range(steps):
        eng.advance(k, 1, _scales(g, 1), use_graphs=False)
        psi, res = eng.get_state()
        norms.append(gpe.norm(psi, float(g["dx"]), float(g["dy"]))[0])
    assert rel_l2(psi, g["psi"]) < 1e-10
    assert rel_l2(res, g["res"][0]) < 1e-10
    assert rel_l2(np.asarray(norms), g["norms"]) < 1e-10


def _oracle_single_noise(g, steps):
    """FP64 oracle on the same noise realisation an FP32 run draws."""
    p = g["physics"]
    dx, dy, dt = float(g["dx"]), float(g["dy"]), float(g["dt"])
    noise = None
    if bool(g["wigner"]):
        noise = gpe.Noise([int(g["seed"])], [p["gamma_C"]], [p["R"]], [1.0], dt, dx * dy,
                          "double", normals_precision="single")
    pump = g["envelope"] * g["p0"]
    norms = []
    psi, fields = gpe.rk4_advance(g["psi0"].copy(), (g["res0"][0],), lambda t: pump, 0.0, p, dx,
                                  dy, dt, 0, steps, noise=noise, norm_trace=norms)
    return psi, fields[0], np.asarray(norms).ravel()


@pytest.mark.parametrize("case", ["rk4_fdm", "rk4_fdm_quiet"])
def test_fp32_within_1e4_of_fp64_oracle(cuda_lib, case):
    g = load_golden(case)
    steps = int(g["steps"])
    psi_ref, res_ref, norms_ref = _oracle_single_noise(g, steps)
    eng = _engine(g, "single")
    norms = []
    for k in range(steps):
        eng.advance(k, 1, _scales(g, 1))
        psi, res = eng.get_state()
        norms.append(gpe.norm(psi.astype(np.complex128), float(g["dx"]), float(g["dy"]))[0])
    assert psi.dtype == np.complex64 and res.dtype == np.float32
    assert rel_l2(psi, psi_ref) < 1e-4
    assert rel_l2(res, res_ref) < 1e-4
    assert rel_l2(np.asarray(norms), norms_ref) < 1e-4


@pytest.mark.parametrize("precision", ["single", "double"])
def test_geometries_graphs_and_members_are_bitwise_identical(cuda_lib, precision):
    g = load_golden("rk4_fdm")
    steps = 10
    ref = _engine(g, precision)
    ref.advance(0, steps, _scales(g, steps), use_graphs=False)
    psi_ref, res_ref = ref.get_state()
    variants = [(8, 8), (16, 4), (24, 12), (g["psi0"].shape[-1], 8)]
    for tile_w, strip_h in variants:
        eng = _engine(g, precision)
        eng.set_geometry(tile_w, strip_h)
        eng.advance(0, steps, _scales(g, steps), use_graphs=True)
        psi, res = eng.get_state()
        assert np.array_equal(psi, psi_ref), (tile_w, strip_h)
        assert np.array_equal(res, res_ref), (tile_w, strip_h)
    batch = _engine(g, precision, members=3)
    batch.advance(0, steps, _scales(g, steps, 3), use_graphs=True)
    psi_b, res_b = batch.get_state()
    for m in range(3):
        assert np.array_equal(psi_b[m], psi_ref[0]) and np.array_equal(res_b[m], res_ref[0])


@pytest.mark.parametrize("shape", [(9, 6), (53, 37), (24, 600)])
def test_ragged_grids_match_oracle(cuda_lib, shape):
    """Odd sizes exercise partial strips, partial tiles and idle lanes."""
    from polarism_gb300.engine import MemberPhysics, RK4Engine

    ny, nx = shape
    rng = np.random.default_rng(7)
    p = dict(hbar=0.6582119514, m_eff=0.284, g_C=0.001, g_R=0.002, g_I=0.0, R=0.02,
             gamma_C=0.083, gamma_R=0.005)
    dx, dy, dt = 0.9, 1.1, 2e-3
    psi0 = (0.1 * (rng.standard_normal((1, 1, ny, nx)) + 1j * rng.standard_normal((1, 1, ny, nx))))
    res0 = np.abs(rng.standard_normal((1, 1, ny, nx))) * 0.01
    env = np.exp(-((np.arange(nx) - nx / 2) ** 2)[None, :] / 50.0
                 - ((np.arange(ny) - ny / 2) ** 2)[:, None] / 30.0)
    eng = RK4Engine(nx, ny, 1, dx, dy, dt, MemberPhysics(**p), "double")
    eng.set_pump(env)
    eng.set_noise([99], p["gamma_C"], p["R"], 1.0, dt / (4 * dx * dy))
    eng.set_state(psi0, res0)
    steps = 6
    eng.advance(0, steps, np.full((steps, 3, 1), 0.03))
    psi, res = eng.get_state()
    noise = gpe.Noise([99], [p["gamma_C"]], [p["R"]], [1.0], dt, dx * dy)
    psi_o, f_o = gpe.rk4_advance(psi0, (res0,), lambda t: env * 0.03, 0.0, p, dx, dy, dt, 0, steps,
                                 noise=noise)
    assert rel_l2(psi, psi_o) < 1e-10
    assert rel_l2(res, f_o[0]) < 1e-10


def test_potential_and_relaxation_general_path(cuda_lib):
    """Complex potential, kinetic relaxation and a time-dependent pump coefficient."""
    from polarism_gb300 import _lib
    from polarism_gb300.engine import MemberPhysics, RK4Engine

    ny, nx = 20, 28
    rng = np.random.default_rng(11)
    p = dict(hbar=0.6582119514, m_eff=0.284, g_C=0.003, g_R=0.002, g_I=0.0, R=0.02,
             gamma_C=0.083, gamma_R=0.005, kinetic_relaxation_eta=0.05)
    dx, dy, dt = 0.7, 0.8, 3e-3
    psi0 = 0.2 * (rng.standard_normal((1, 1, ny, nx)) + 1j * rng.standard_normal((1, 1, ny, nx)))
    res0 = np.abs(rng.standard_normal((1, 1, ny, nx))) * 0.05
    env = np.abs(rng.standard_normal((ny, nx)))
    pot = 0.01 * rng.standard_normal((ny, nx)) - 0.002j * np.abs(rng.standard_normal((ny, nx)))
    eng = RK4Engine(nx, ny, 1, dx, dy, dt, MemberPhysics(**p), "double",
                    potential=_lib.PG_POT_COMPLEX)
    eng.set_pump(env)
    eng.set_potential(pot)
    eng.set_state(psi0, res0)
    steps = 8
    coeff = lambda t: 0.05 * (1.0 + np.sin(30.0 * t))  # noqa: E731
    scales = np.asarray([[[coeff(k * dt)], [coeff(k * dt + dt / 2)], [coeff(k * dt + dt)]]
                         for k in range(steps)])
    eng.advance(0, steps, scales)
    psi, res = eng.get_state()
    psi_o, f_o = gpe.rk4_advance(psi0, (res0,), lambda t: env * coeff(t), pot, p, dx, dy, dt, 0,
                                 steps)
    assert rel_l2(psi, psi_o) < 1e-10
    assert rel_l2(res, f_o[0]) < 1e-10


def test_one_step_wigner_variance(cuda_lib):
    """Mean |psi|^2 after one noisy step from zero is s gamma_C dt / 2 (+-6%)."""
    from polarism_gb300.engine import MemberPhysics, RK4Engine

    n = 64
    p = dict(hbar=0.6582119514, m_eff=0.284, g_C=0.0, g_R=0.0, g_I=0.0, R=0.0, gamma_C=0.083,
             gamma_R=0.005)
    dx = dy = 1.0
    dt = 0.01
    for strength in (1.0, 2.0):
        eng = RK4Engine(n, n, 1, dx, dy, dt, MemberPhysics(**p), "single")
        eng.set_pump(np.zeros((n, n), dtype=np.float32))
        eng.set_noise([123456], p["gamma_C"], 0.0, strength, dt / (4 * dx * dy))
        eng.set_state(np.zeros((1, 1, n, n), np.complex64), np.zeros((1, 1, n, n), np.float32))
        eng.advance(0, 1, np.zeros((1, 3, 1)))
        psi, _ = eng.get_state()
        expected = strength * p["gamma_C"] * dt / 2.0
        assert abs(np.mean(np.abs(psi) ** 2) - expected) / expected < 0.06


def test_deterministic_repeat(cuda_lib):
    g = load_golden("rk4_fdm")
    outs = []
    for _ in range(2):
        eng = _engine(g, "single")
        eng.advance(0, 12, _scales(g, 12))
        outs.append(eng.get_state())
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])


def test_launch_count_and_error_status(cuda_lib):
    g = load_golden("rk4_fdm")
    eng = _engine(g, "single")
    eng.advance(0, 70, _scales(g, 70))
    assert eng.last_launch_count == 70
    with pytest.raises(RuntimeError, match="strip height"):
        eng.set_geometry(8, 6)


@pytest.mark.parametrize("nx,ny,members", [(128, 48, 3), (256, 20, 2), (512, 12, 2), (1024, 8, 1),
                                            (2048, 40, 1), (3072, 10, 1), (4096, 6, 2), (8192, 4, 1),
                                            (9216, 6, 1)])
def test_full_width_kernel_matches_oracle_and_tiled(cuda_lib, nx, ny, members):
    """The TMA full-width FP32 kernel against the oracle (1e-4) and the tiled kernel (1e-5).

    Rows of 2048 to 8192 sites run as clusters of 1024-site bands exchanging edge columns
    through distributed shared memory (clusters of 2, 3, 4 and 8 here, with row ranges that
    cross members); wider rows (9216) as independent bands with four recomputed halo columns on each
    side, whose row ranges cross from one band into the next.  Both cover the periodic wrap
    of the first and last band."""
    from polarism_gb300.engine import MemberPhysics, RK4Engine

    rng = np.random.default_rng(nx + ny)
    p = dict(hbar=0.6582119514, m_eff=0.284, g_C=0.001, g_R=0.002, g_I=0.0, R=0.02,
             gamma_C=0.083, gamma_R=0.005)
    dx, dy, dt = 0.5, 0.6, 1e-3
    psi0 = 0.05 * (rng.standard_normal((members, 1, ny, nx))
                   + 1j * rng.standard_normal((members, 1, ny, nx)))
    res0 = np.abs(rng.standard_normal((members, 1, ny, nx))) * 0.02
    env = np.abs(rng.standard_normal((members, 1, ny, nx)))
    seeds = [5 + m for m in range(members)]
    steps = 7
    outs = {}
    for kernel in (2, 1):
        eng = RK4Engine(nx, ny, members, dx, dy, dt, MemberPhysics(**p), "single",
                        pump_per_member=True)
        eng.set_kernel(kernel)
        assert eng.kernel() == kernel
        eng.set_pump(env.astype(np.float32))
        eng.set_noise(seeds, p["gamma_C"], p["R"], 1.0, dt / (4 * dx * dy))
        eng.set_state(psi0.astype(np.complex64), res0.astype(np.float32))
        eng.advance(0, steps, np.full((steps, 3, members), 0.04))
        outs[kernel] = eng.get_state()
    noise = gpe.Noise(seeds, [p["gamma_C"]] * members, [p["R"]] * members, [1.0] * members, dt,
                      dx * dy, "double", normals_precision="single")
    psi_o, f_o = gpe.rk4_advance(psi0.copy(), (res0.copy(),), lambda t: env * 0.04, 0.0, p, dx,
                                 dy, dt, 0, steps, noise=noise)
    psi_w, res_w = outs[2]
    psi_t, res_t = outs[1]
    assert rel_l2(psi_w, psi_o) < 1e-4 and rel_l2(res_w, f_o[0]) < 1e-4
    assert rel_l2(psi_w, psi_t) < 1e-5 and rel_l2(res_w, res_t) < 1e-5


@pytest.mark.parametrize("precision", ["single", "double"])
def test_device_normals_within_error_bound(cuda_lib, precision):
    """Device Box-Muller normals against the reference's normal_pair on the same words.

    FP64 uses correctly rounded library functions (2e-14, the reference's own bound).  FP32
    uses SFU approximations: |error| <= 4e-6 (1 + r) plus 3e-7 / r for the radius term."""
    from oracle.philox import normal_pair
    from polarism_gb300.engine import wigner_normals

    counters = counter_words(np.arange(1 << 18), 987654321)
    key = 0xDEADBEEF12345
    got = wigner_normals(counters, key, precision)
    words = philox4x32(counters, key)
    if precision == "double":
        re, im = normal_pair(words, "double")
    else:
        # The single-precision uniforms of normal_pair, transformed exactly (in FP64).
        u1 = ((words[..., 0] >> 8).astype(np.float64) + 1.0) * 2.0 ** -24
        u2 = ((words[..., 1] >> 8).astype(np.float64) + 1.0) * 2.0 ** -24
        rr = np.sqrt(-2.0 * np.log(u1))
        re, im = rr * np.cos(2 * np.pi * u2), rr * np.sin(2 * np.pi * u2)
        ref32 = normal_pair(words, "single")
        assert rel_l2(ref32[0], re) < 1e-6  # the reference's own FP32 path, same realisation
    r = np.hypot(re, im)
    if precision == "double":
        np.testing.assert_allclose(got[0], re, rtol=2e-14, atol=2e-14)
        np.testing.assert_allclose(got[1], im, rtol=2e-14, atol=2e-14)
        return
    bound = 4e-6 * (1 + r) + 3e-7 / np.maximum(r, 1e-30)
    assert np.all(np.abs(got[0] - re) <= bound)
    assert np.all(np.abs(got[1] - im) <= bound)
    assert rel_l2(got[0], re) < 1e-6 and rel_l2(got[1], im) < 1e-6


@pytest.mark.parametrize("pot_kind,per_member", [("complex", True), ("real", False), ("none", False)])
@pytest.mark.parametrize("nx,ny,members", [(256, 24, 2), (1024, 12, 1), (2048, 12, 2), (4096, 6, 1)])
def test_full_width_general_variant_matches_oracle_and_tiled(cuda_lib, pot_kind, per_member, nx, ny,
                                                             members):
    """The full-width kernel's general variant (potential and kinetic relaxation, Wigner noise
    on): within 1e-4 of the FP64 oracle on the same noise and 1e-5 of the tiled kernel."""
    from polarism_gb300 import _lib
    from polarism_gb300.engine import MemberPhysics, RK4Engine

    rng = np.random.default_rng(nx + members)
    p = dict(hbar=0.6582119514, m_eff=0.284, g_C=0.003, g_R=0.002, g_I=0.0, R=0.02,
             gamma_C=0.083, gamma_R=0.005, kinetic_relaxation_eta=0.05)
    dx, dy, dt = 0.5, 0.6, 1e-3
    psi0 = 0.1 * (rng.standard_normal((members, 1, ny, nx)) + 1j * rng.standard_normal((members, 1, ny, nx)))
    res0 = np.abs(rng.standard_normal((members, 1, ny, nx))) * 0.05
    env = np.abs(rng.standard_normal((members, 1, ny, nx)))
    shape = (members, 1, ny, nx) if per_member else (ny, nx)
    kind = {"complex": _lib.PG_POT_COMPLEX, "real": _lib.PG_POT_REAL, "none": _lib.PG_POT_NONE}[pot_kind]
    pot = 0.02 * rng.standard_normal(shape)
    if pot_kind == "complex":
        pot = pot - 0.003j * np.abs(rng.standard_normal(shape))
    seeds = [9 + m for m in range(members)]
    steps = 6
    outs = {}
    for kernel in (2, 1):
        eng = RK4Engine(nx, ny, members, dx, dy, dt, MemberPhysics(**p), "single", pump_per_member=True,
                        potential=kind, potential_per_member=per_member)
        eng.set_kernel(kernel)
        assert eng.kernel() == kernel
        eng.set_pump(env.astype(np.float32))
        if pot_kind != "none":
            eng.set_potential(pot.astype(np.complex64 if pot_kind == "complex" else np.float32))
        eng.set_noise(seeds, p["gamma_C"], p["R"], 1.0, dt / (4 * dx * dy))
        eng.set_state(psi0.astype(np.complex64), res0.astype(np.float32))
        eng.advance(0, steps, np.full((steps, 3, members), 0.05))
        outs[kernel] = eng.get_state()
        eng.close()
    noise = gpe.Noise(seeds, [p["gamma_C"]] * members, [p["R"]] * members, [1.0] * members, dt,
                      dx * dy, "double", normals_precision="single")
    psi_o, f_o = gpe.rk4_advance(psi0.copy(), (res0.copy(),), lambda t: env * 0.05,
                                 0.0 if pot_kind == "none" else pot, p, dx, dy, dt, 0, steps, noise=noise)
    (psi_w, res_w), (psi_t, res_t) = outs[2], outs[1]
    assert rel_l2(psi_w, psi_o) < 1e-4 and rel_l2(res_w, f_o[0]) < 1e-4
    assert rel_l2(psi_w, psi_t) < 1e-5 and rel_l2(res_w, res_t) < 1e-5


@pytest.mark.parametrize("nx,ny,members,noise", [(1024, 40, 3, True), (1024, 8, 1, False),
                                                  (512, 36, 5, True), (512, 12, 2, False)])
def test_four_site_form_is_bitwise_the_two_site_form(cuda_lib, nx, ny, members, noise):
    """The full-width kernel's four-sites-a-thread form (kernel kind 3) does the same operations
    site by site as the default two-site form (kind 2), so the results are identical bit for
    bit -- over member boundaries inside a block's row range, the periodic seams and several
    graph-captured steps -- and within 1e-4 of the oracle."""
    from polarism_gb300.engine import MemberPhysics, RK4Engine

    rng = np.random.default_rng(nx * 7 + ny)
    p = dict(hbar=0.6582119514, m_eff=0.284, g_C=0.001, g_R=0.002, g_I=0.0, R=0.02,
             gamma_C=0.083, gamma_R=0.005)
    dx, dy, dt, steps = 0.45, 0.55, 1e-3, 9
    psi0 = 0.05 * (rng.standard_normal((members, 1, ny, nx))
                   + 1j * rng.standard_normal((members, 1, ny, nx)))
    res0 = np.abs(rng.standard_normal((members, 1, ny, nx))) * 0.02
    env = np.abs(rng.standard_normal((members, 1, ny, nx)))
    seeds = [11 + m for m in range(members)]
    # Coefficients at every half step (a time-dependent pump): step k's stages read samples
    # 2k, 2k + 1 and 2k + 2.
    samples = 0.03 + 0.01 * rng.random((2 * steps + 1, members))
    scales = np.stack([samples[2 * k:2 * k + 3] for k in range(steps)])
    outs = {}
    for kernel in (2, 3):
        eng = RK4Engine(nx, ny, members, dx, dy, dt, MemberPhysics(**p), "single",
                        pump_per_member=True)
        eng.set_kernel(kernel)
        assert eng.kernel() == kernel
        eng.set_pump(env.astype(np.float32))
        if noise:
            eng.set_noise(seeds, p["gamma_C"], p["R"], 1.0, dt / (4 * dx * dy))
        eng.set_state(psi0.astype(np.complex64), res0.astype(np.float32))
        eng.advance(0, steps, scales)
        outs[kernel] = eng.get_state()
        eng.close()
    assert np.array_equal(outs[2][0].view(np.uint32), outs[3][0].view(np.uint32))
    assert np.array_equal(outs[2][1].view(np.uint32), outs[3][1].view(np.uint32))
    nz = (gpe.Noise(seeds, [p["gamma_C"]] * members, [p["R"]] * members, [1.0] * members, dt,
                    dx * dy, "double", normals_precision="single") if noise else None)
    def pump_at(t):  # the oracle's pump at stage time t (a half-step sample)
        return env * samples[int(round(2 * t / dt))][:, None, None, None]

    psi_o, fields = gpe.rk4_advance(psi0.copy(), (res0.copy(),), pump_at, 0.0, p, dx, dy, dt, 0,
                                    steps, noise=nz)
    assert rel_l2(outs[2][0], psi_o) < 1e-4 and rel_l2(outs[2][1], fields[0]) < 1e-4
