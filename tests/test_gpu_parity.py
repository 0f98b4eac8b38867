"""CUDA engine vs the CPU oracle, through the C ABI (GPU only).

Tolerances: complex64 results are compared with the FP64 oracle at relative
L2 <= 1e-5 per the propagation-path contract (complex128 at 1e-11); potential
geometry without transcendental functions is compared bit for bit.
"""
import math

import numpy as np
import pytest

from oracle import wfs_oracle as orc

pytestmark = pytest.mark.gpu

C64_TOL = 1e-5
C128_TOL = 1e-11


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.complex128) - np.asarray(b, np.complex128)) /
                 np.linalg.norm(np.asarray(b, np.complex128)))


@pytest.fixture(scope="module")
def Engine():
    from wavefunctionsimpython_gb300 import Engine as E

    return E


def packet_args(n, L):
    return dict(sigma=(0.12 * L[0], 0.11 * L[1], 0.1 * L[2]), r0=(-0.1 * L[0], 0.05 * L[1], 0.0),
                k0=(2.0, 0.0, -0.5))


@pytest.mark.parametrize("dbl", [False, True])
@pytest.mark.parametrize("n", [(32, 32, 32), (16, 24, 48), (64, 32, 96)])
def test_gaussian_packet(Engine, n, dbl):
    L = tuple(0.5 * x for x in n)
    e = Engine(n, L, double_precision=dbl)
    p = packet_args(n, L)
    e.init_gaussian(p["sigma"], p["r0"], p["k0"])
    ref = orc.gaussian_wave_packet(n, orc.delta_x(L, n), p["sigma"], p["r0"], p["k0"], dbl)
    assert rel(e.get_psi(), ref) < (1e-14 if dbl else 1e-6)


@pytest.mark.parametrize("slits,rot", [(0, 0.0), (1, 0.0), (2, math.pi / 2), (3, 0.3), (4, math.pi / 2)])
def test_wall_bit_exact(Engine, slits, rot):
    n, L = (32, 48, 24), (20.0, 30.0, 15.0)
    e = Engine(n, L)
    w = orc.Wall(potential_hartree=7.0, center_bohr_radii_3=(0.5, -1.0, 0.0), normal_vector_3=(1.0, 0.2, 0.0),
                 plateau_thickness_bohr_radii=2.0, slope_thickness_bohr_radii=0.0, slit_count=slits,
                 slit_spacing_bohr_radii=5.0, slit_width_bohr_radii=2.0, slit_rotation_radian=rot)
    e.add_wall(w.potential_hartree, w.center_bohr_radii_3, w.normal_vector_3, w.plateau_thickness_bohr_radii,
               0.0, 1.0, slits, 5.0, 2.0, rot)
    ref = orc.add_potential_wall(np.zeros(n, np.complex64), orc.delta_x(L, n), w)
    assert np.array_equal(e.get_potential(), ref)


def test_wall_slope(Engine):
    n, L = (48, 16, 16), (24.0, 8.0, 8.0)
    e = Engine(n, L)
    w = orc.Wall(potential_hartree=7.0, plateau_thickness_bohr_radii=2.0, slope_thickness_bohr_radii=2.0,
                 slope_exponent=1.5)
    e.add_wall(7.0, (0, 0, 0), (1, 0, 0), 2.0, 2.0, 1.5)
    ref = orc.add_potential_wall(np.zeros(n, np.complex64), orc.delta_x(L, n), w)
    np.testing.assert_allclose(e.get_potential().real, ref.real, rtol=2e-6, atol=1e-6)


@pytest.mark.parametrize("offset,exps", [(0.0, (2.0, 2.0, 2.0)), (1.0, (3.0, 2.0, 1.5))])
def test_absorbing(Engine, offset, exps):
    n, L = (40, 32, 48), (40.0, 32.0, 48.0)
    e = Engine(n, L)
    ab = orc.Absorbing(bottom=(-12.0, -9.0, -15.0), top=(12.0, 10.0, 14.0), offset=offset,
                       potential_pos=(-50.0, -10.0, -20.0), potential_neg=(-40.0, -10.0, -30.0),
                       exponent_pos=exps, exponent_neg=exps[::-1])
    e.add_absorbing(ab.bottom, ab.top, ab.offset, ab.potential_pos, ab.potential_neg, ab.exponent_pos, ab.exponent_neg)
    ref = orc.absorbing_potential_imag(n, orc.delta_x(L, n), ab)
    got = e.get_potential()
    assert np.all(got.real == 0)
    np.testing.assert_allclose(got.imag, ref, rtol=1e-5, atol=1e-4)


def scenario(n, L, dbl, absorber=True):
    dx = orc.delta_x(L, n)
    p = packet_args(n, L)
    V = np.zeros(n, np.complex64)
    w = orc.Wall(potential_hartree=3.0, plateau_thickness_bohr_radii=0.1 * L[0], slit_count=2,
                 slit_spacing_bohr_radii=0.2 * L[1], slit_width_bohr_radii=0.08 * L[1],
                 slit_rotation_radian=math.pi / 2)
    orc.add_potential_wall(V, dx, w)
    if absorber:
        inner = tuple(0.35 * x for x in L)
        V += (1j * orc.absorbing_potential_imag(n, dx, orc.Absorbing(
            bottom=tuple(-x for x in inner), top=inner, offset=0.0, potential_pos=(-20.0,) * 3,
            potential_neg=(-20.0,) * 3, exponent_pos=(2.0,) * 3, exponent_neg=(2.0,) * 3))).astype(np.complex64)
    psi0 = orc.gaussian_wave_packet(n, dx, p["sigma"], p["r0"], p["k0"], dbl)
    return dx, V, psi0


@pytest.mark.parametrize("schedule", ["auto", "axis"])
@pytest.mark.parametrize("dbl", [False, True])
@pytest.mark.parametrize("n", [(32, 32, 32), (64, 64, 64), (16, 48, 32), (48, 48, 48), (96, 32, 64), (8, 128, 16),
                               (16, 96, 96), (8, 128, 128), (4, 256, 256), (384, 64, 6)])
def test_split_step(Engine, n, dbl, schedule):
    # (384, 64, 6): the y passes have 384 tiles of 32 columns with 6 in the grid, so the
    # copy-staged strided pass runs with zero-filled columns past the edge
    L = tuple(0.4 * x for x in n)
    dx, V, psi0 = scenario(n, L, dbl)
    e = Engine(n, L, double_precision=dbl)
    e.set_schedule(schedule)
    e.set_potential(V)
    e.set_psi(psi0)
    e.step_split(7, 0.01, 1.0)
    ref = orc.split_step(psi0.astype(np.complex128), V, dx, 0.01, 1.0, nsteps=7, double_precision=True)
    assert rel(e.get_psi(), ref) < (C128_TOL if dbl else C64_TOL)


def test_split_step_chunking_and_mass(Engine):
    """Repeated calls (lazy Strang merging), a dt change and a non-unit mass."""
    n, L = (32, 32, 32), (16.0, 16.0, 16.0)
    dx, V, psi0 = scenario(n, L, True)
    e = Engine(n, L, double_precision=True)
    e.set_potential(V)
    e.set_psi(psi0)
    e.step_split(3, 0.01, 2.0)
    e.step_split(2, 0.01, 2.0)
    e.step_split(4, 0.02, 2.0)
    ref = orc.split_step(psi0, V, dx, 0.01, 2.0, nsteps=5)
    ref = orc.split_step(ref, V, dx, 0.02, 2.0, nsteps=4)
    assert rel(e.get_psi(), ref) < C128_TOL


@pytest.mark.parametrize("dbl", [False, True])
@pytest.mark.parametrize("stencil", [2, 4])
@pytest.mark.parametrize("n", [(32, 32, 32), (24, 40, 16), (64, 64, 64)])
def test_taylor(Engine, n, stencil, dbl):
    L = tuple(0.5 * x for x in n)
    dx, V, psi0 = scenario(n, L, dbl)
    e = Engine(n, L, double_precision=dbl)
    e.set_potential(V)
    e.set_psi(psi0)
    e.step_taylor(3, 0.005, 1.0, order=10, stencil_order=stencil)
    ref = orc.taylor_step(psi0.astype(np.complex128), V, dx, 0.005, 1.0, order=10, stencil_order=stencil, nsteps=3)
    assert rel(e.get_psi(), ref) < (C128_TOL if dbl else C64_TOL)


@pytest.mark.parametrize("dbl", [False, True])
def test_observables(Engine, dbl):
    n, L = (48, 32, 64), (24.0, 16.0, 32.0)
    dx, V, psi0 = scenario(n, L, dbl, absorber=False)
    e = Engine(n, L, double_precision=dbl)
    e.set_psi(psi0)
    boxes = [((0, 0, 0), (47, 31, 63)), ((24, 1, 3), (23, 29, 57)), ((5, 7, 9), (1, 1, 1)), ((10, 0, 0), (3, 31, 63))]
    loc = ((2, 1, 4), (43, 29, 57))
    for stage in range(3):
        probs, er, er2 = e.observe(boxes, loc)
        psi = e.get_psi()
        for (b, c), p in zip(boxes, probs):
            assert abs(p - orc.volume_probability(psi, dx, b, c)) <= 1e-6 * max(1.0, abs(p))
        rr, rr2 = orc.expected_location(psi, dx, *loc)
        np.testing.assert_allclose(er, rr, rtol=1e-6, atol=1e-7)
        np.testing.assert_allclose(er2, rr2, rtol=1e-6, atol=1e-7)
        e.step_split(3, 0.02, 1.0)  # observation from the pending split-step state next time


@pytest.mark.parametrize("interval", [1, 4])
def test_run_split_series(Engine, interval):
    n, L = (32, 32, 32), (20.0, 20.0, 20.0)
    dx, V, psi0 = scenario(n, L, True)
    e = Engine(n, L, double_precision=True)
    e.set_potential(V)
    e.set_psi(psi0)
    boxes = [((0, 0, 0), (31, 31, 31)), ((16, 0, 0), (15, 31, 31))]
    loc = ((1, 1, 1), (29, 29, 29))
    nsteps = 10
    ps, ls = e.run_split(nsteps, 0.01, 1.0, interval, boxes, loc)
    assert ps.shape == (-(-nsteps // interval), 2)
    psi = psi0.copy()
    for k, i in enumerate(range(0, nsteps, interval)):
        for j, (b, c) in enumerate(boxes):
            assert abs(ps[k, j] - orc.volume_probability(psi, dx, b, c)) < 1e-9
        rr, rr2 = orc.expected_location(psi, dx, *loc)
        np.testing.assert_allclose(ls[k, :3], rr, rtol=1e-9, atol=1e-11)
        np.testing.assert_allclose(ls[k, 3:], rr2, rtol=1e-9, atol=1e-11)
        psi = orc.split_step(psi, V, dx, 0.01, 1.0, nsteps=min(interval, nsteps - i))
    assert rel(e.get_psi(), psi) < C128_TOL


def test_norm_and_nonfinite(Engine):
    from wavefunctionsimpython_gb300._lib import WFS_ERR_NONFINITE, WfsError

    n, L = (16, 16, 16), (12.0, 12.0, 12.0)
    e = Engine(n, L, double_precision=True)
    e.init_gaussian((1.5,) * 3, (0, 0, 0), (0, 0, 0))
    ref = orc.gaussian_wave_packet(n, orc.delta_x(L, n), (1.5,) * 3, (0, 0, 0), (0, 0, 0), True)
    assert abs(e.norm() - np.sum(np.abs(ref) ** 2) * np.prod(orc.delta_x(L, n))) < 1e-12
    bad = e.get_psi()
    bad[3, 4, 5] = np.nan
    e.set_psi(bad)
    with pytest.raises(WfsError) as ei:
        e.norm()
    assert ei.value.code == WFS_ERR_NONFINITE


def test_operators_module(Engine):
    from wavefunctionsimpython_gb300 import operators

    n, dx = (16, 8, 32), (0.5, 0.25, 0.75)
    K = operators.init_kinetic_operator(dx, 0.01, 1.0, n, double_precision=True)
    ref = orc.kinetic_phase(n, dx, 0.01, 1.0, True)
    assert np.max(np.abs(K - ref)) < 1e-14
    V = (np.random.default_rng(0).standard_normal(n) + 1j * np.minimum(0, np.random.default_rng(1).standard_normal(n))).astype(np.complex64)
    P = np.ones(n, np.complex128)
    got = operators.init_potential_operator(P, V, 0.05, dx)
    assert np.max(np.abs(got - orc.potential_phase(V, 0.05, True))) < 1e-14


def test_unsupported_length_rejected_by_split_step_only(Engine):
    """Any axis length is accepted; the split step refuses lengths its FFT does not
    cover, the power series runs on them."""
    from wavefunctionsimpython_gb300._lib import WFS_ERR_UNSUPPORTED, WfsError

    n, L = (20, 16, 18), (10.0, 8.0, 9.0)
    e = Engine(n, L, double_precision=True)
    e.init_gaussian((1.5,) * 3, (0, 0, 0), (0.5, 0, 0))
    with pytest.raises(WfsError) as ei:
        e.step_split(1, 0.01, 1.0)
    assert ei.value.code == WFS_ERR_UNSUPPORTED
    psi0 = e.get_psi()
    e.step_taylor(2, 0.002, 1.0, order=8, stencil_order=2)
    ref = orc.taylor_step(psi0, np.zeros(n, np.complex64), orc.delta_x(L, n), 0.002, 1.0, order=8, stencil_order=2, nsteps=2)
    assert rel(e.get_psi(), ref) < C128_TOL
