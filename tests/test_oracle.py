"""Pins the CPU oracle against the reference's known answers (CPU only).

Known answers used (paths relative to the reference project root):
* free-packet <x>(t) = x0 + v t and sigma(t) = sqrt(a^2 + 4 t^2/(m^2 a^2))/2,
  a = 2 sigma0 (sources/math_utils.py:237-267);
* unit norm of the Gaussian packet (sources/cuda_kernels/common.cu:569-605);
* norm="ortho" transforms are unitary: a split step with real V conserves the norm;
* harmonic oscillator V = 1/2 w^2 r^2 (sources/potential.py:414-423): <x>(t) = x0 cos(w t);
* Simpson weights integrate polynomials up to degree 3 exactly.
"""
import math

import numpy as np
import pytest

from oracle import wfs_oracle as orc


def test_gaussian_unit_norm():
    n, L = (48, 48, 48), (24.0, 24.0, 24.0)
    dx = orc.delta_x(L, n)
    psi = orc.gaussian_wave_packet(n, dx, (1.5, 2.0, 1.7), (-1.0, 0.5, 0.0), (1.0, 0.0, -0.5), True)
    norm = np.sum(np.abs(psi) ** 2) * np.prod(dx)
    assert abs(norm - 1.0) < 1e-7   # tails beyond the box edge (6 sigma) are cut


def test_ortho_round_trip_is_identity():
    rng = np.random.default_rng(1)
    a = rng.standard_normal((8, 12, 16)) + 1j * rng.standard_normal((8, 12, 16))
    b = np.fft.ifftn(np.fft.fftn(a, norm="ortho"), norm="ortho")
    assert np.max(np.abs(a - b)) < 1e-12


def test_split_step_unitary_for_real_potential():
    sc = orc.config1_barrier_64()
    sc.n = (32, 32, 32)
    sc.extent = (30.0, 30.0, 30.0)
    psi0 = sc.psi0()
    V = sc.potential()
    assert np.all(V.imag == 0)
    psi = orc.split_step(psi0, V, sc.dx, sc.dt, 1.0, nsteps=20)
    n0 = np.sum(np.abs(psi0) ** 2)
    n1 = np.sum(np.abs(psi) ** 2)
    assert abs(n1 / n0 - 1.0) < 1e-12


def test_free_packet_matches_reference_predictions():
    """Oracle split step with V = 0 against math_utils.predict_free_space_* (c128)."""
    n, L = (64, 64, 64), (48.0, 48.0, 48.0)
    dx = orc.delta_x(L, n)
    sigma0, x0, v = 2.0, -6.0, 2.0
    psi = orc.gaussian_wave_packet(n, dx, (sigma0,) * 3, (x0, 0.0, 0.0), (v, 0.0, 0.0), True)
    V = np.zeros(n, np.complex64)
    dt, steps, every = 0.02, 100, 25
    box = (np.zeros(3, np.int64), np.array([63, 63, 63]))
    xs, ss = [], []
    for i in range(0, steps + 1, every):
        er, er2 = orc.expected_location(psi, dx, *box)
        norm = orc.volume_probability(psi, dx, *box)
        xs.append(er[0] / norm)
        ss.append(math.sqrt(er2[0] / norm - (er[0] / norm) ** 2))
        if i < steps:
            psi = orc.split_step(psi, V, dx, dt, 1.0, nsteps=every)
    t_idx = np.arange(0, steps + 1, every)
    px = orc.predict_free_space_expected_location(dt, x0, v, steps + 1)[t_idx]
    ps = orc.predict_free_space_standard_deviation(dt, sigma0, 1.0, steps + 1)[t_idx]
    assert np.max(np.abs(np.array(xs) - px)) < 2e-3
    assert np.max(np.abs(np.array(ss) - ps)) < 2e-3


def test_harmonic_oscillator_coherent_state():
    """HO with w = 0.5, packet displaced to x0 = 3: <x>(t) = x0 cos(w t)."""
    n, L = (48, 48, 48), (24.0, 24.0, 24.0)
    dx = orc.delta_x(L, n)
    w, x0 = 0.5, 3.0
    sigma = math.sqrt(1.0 / (2.0 * w))  # ground-state width of the oscillator
    psi = orc.gaussian_wave_packet(n, dx, (sigma,) * 3, (x0, 0.0, 0.0), (0.0, 0.0, 0.0), True)
    V = orc.harmonic_oscillator(n, dx, w)
    box = (np.zeros(3, np.int64), np.array([47, 47, 47]))
    dt = 0.05
    for k in range(4):
        er, _ = orc.expected_location(psi, dx, *box)
        norm = orc.volume_probability(psi, dx, *box)
        t = k * 20 * dt
        assert abs(er[0] / norm - x0 * math.cos(w * t)) < 5e-3
        psi = orc.split_step(psi, V, dx, dt, 1.0, nsteps=20)


def test_taylor_agrees_with_split_step_small_dt():
    n, L = (32, 32, 32), (20.0, 20.0, 20.0)
    dx = orc.delta_x(L, n)
    psi = orc.gaussian_wave_packet(n, dx, (2.0,) * 3, (0.0, 0.0, 0.0), (0.5, 0.0, 0.0), True)
    V = orc.harmonic_oscillator(n, dx, 0.5)
    a = orc.taylor_step(psi, V, dx, 0.002, 1.0, order=10, stencil_order=4, nsteps=25)
    b = orc.split_step(psi, V, dx, 0.002, 1.0, nsteps=25)
    assert np.linalg.norm(a - b) / np.linalg.norm(b) < 5e-3


def test_simpson_weights_exact_for_cubics():
    n, L = (33, 9, 9), (8.0, 8.0, 8.0)
    dx = orc.delta_x(L, n)
    x = (np.arange(33) * dx[0])
    f = (x ** 3 + 2 * x + 1.0)
    psi = np.sqrt(np.broadcast_to(f[:, None, None], n).astype(np.complex128))
    p = orc.volume_probability(psi, dx, (0, 0, 0), (33, 9, 9))
    exact = ((32 * dx[0]) ** 4 / 4 + (32 * dx[0]) ** 2 + 32 * dx[0]) * (8 * dx[1]) * (8 * dx[2])
    assert abs(p - exact) / exact < 1e-12


def test_indefinite_simpson_integral_polynomial():
    t = np.arange(21) * 0.1
    f = 3 * t ** 2
    I = orc.indefinite_simpson_integral(f, 0.1)
    assert abs(I[-1] - 2.0 ** 3) < 1e-9
    assert I[0] == 0.0


@pytest.mark.parametrize("slits", [0, 1, 2, 3, 4])
def test_wall_geometry(slits):
    n, L = (16, 32, 24), (16.0, 32.0, 24.0)
    dx = orc.delta_x(L, n)
    w = orc.Wall(potential_hartree=5.0, plateau_thickness_bohr_radii=2.0, slope_thickness_bohr_radii=1.0,
                 slope_exponent=2.0, slit_count=slits, slit_spacing_bohr_radii=6.0, slit_width_bohr_radii=2.0,
                 slit_rotation_radian=math.pi / 2)
    V = orc.add_potential_wall(np.zeros(n, np.complex64), dx, w)
    assert V.real.max() == pytest.approx(5.0)
    # slab: |x| <= 1 plateau, slope to 2
    x = dx[0] * (np.arange(n[0]) - n[0] / 2)
    assert np.all(V.real[np.abs(x) > 2.0 + 1e-6] == 0)
    if slits == 0:
        assert np.all(V.real[np.abs(x) <= 1.0] == 5.0)


def test_absorbing_ramp_zero_inside_box_and_negative_outside():
    n, L = (32, 32, 32), (32.0, 32.0, 32.0)
    dx = orc.delta_x(L, n)
    ab = orc.Absorbing(bottom=(-10.0,) * 3, top=(10.0,) * 3, offset=0.0, potential_pos=(-50.0,) * 3,
                       potential_neg=(-50.0,) * 3, exponent_pos=(2.0,) * 3, exponent_neg=(2.0,) * 3)
    U = orc.absorbing_potential_imag(n, dx, ab)
    r = dx[0] * (np.arange(32) - 16)
    inside = (np.abs(r) < 10.0)
    assert np.all(U[np.ix_(inside, inside, inside)] == 0)
    assert U.min() < -10.0 and U.max() <= 0.0
    # face value at the outer boundary: ((d - off)/maxD)^2 * U
    i = 0
    d = -10.0 - r[i]   # -dB.x, with dB.x = r - bottom < 0
    expect = (d / (16.0 - 10.0)) ** 2 * -50.0
    assert U[i, 16, 16] == pytest.approx(expect, rel=1e-5)


def test_dynamic_rebuild_matches_initial_build_and_clamps():
    """generate_potential_from_walls_and_drain (walls, then the ramp, from zero) gives the
    initial potential back when nothing moved, and advection clamps the x centre at 0."""
    n, L = (16, 16, 16), (8.0, 8.0, 8.0)
    dx = orc.delta_x(L, n)
    walls = [orc.Wall(potential_hartree=3.0, center_bohr_radii_3=(0.1, 0.0, 0.0), plateau_thickness_bohr_radii=1.0,
                      slope_thickness_bohr_radii=0.5, slit_count=1, slit_width_bohr_radii=1.0)]
    ab = orc.Absorbing(bottom=(-3.0,) * 3, top=(3.0,) * 3, offset=0.2, potential_pos=(-10.0,) * 3,
                       potential_neg=(-10.0,) * 3, exponent_pos=(2.0,) * 3, exponent_neg=(2.0,) * 3)
    sc = orc.Scenario(n=n, extent=L, sigma=(1.0,) * 3, r0=(0.0,) * 3, k0=(0.0,) * 3, dt=0.02, walls=walls,
                      absorbing=ab)
    assert np.array_equal(orc.rebuild_potential(n, dx, walls, ab), sc.potential())
    moved = orc.advect_walls(walls, [(-3.0, 1.0, 0.0)], 0.05)
    assert moved[0].center_bohr_radii_3 == (0.0, 0.05, 0.0)
    assert not np.array_equal(orc.rebuild_potential(n, dx, moved, ab), sc.potential())
