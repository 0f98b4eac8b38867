"""Dynamic potential mode on the device (GPU only).

The reference advects its walls and rebuilds V after every step
(sources/sim_state.py:466-509, sources/potential.py:508-522). The engine does the
same inside its step loop: the first update rebuilds V whole, later ones rewrite only
the voxels a moving wall reaches, with their phase-table entries. These tests run
trajectories with two walls (one sliding into the x = 0 clamp, one tilted) and an
absorbing ramp against the oracle, which rebuilds V from scratch every step.
"""
import math
import time

import numpy as np
import pytest

from oracle import wfs_oracle as orc

pytestmark = pytest.mark.gpu

C64_TOL, C128_TOL = 1e-5, 1e-11


def rel(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def scenario(n, L, dbl):
    """Two walls and an absorbing ramp. The second wall starts at x = -3: the reference's
    update clamps every wall's x centre at 0 (sources/sim_state.py:472), so it jumps to
    x = 0 at the first update, moving or not."""
    dx = orc.delta_x(L, n)
    walls = [orc.Wall(potential_hartree=4.0, center_bohr_radii_3=(0.2, 0.0, 0.0), normal_vector_3=(1.0, 0.0, 0.0),
                      plateau_thickness_bohr_radii=1.0, slope_thickness_bohr_radii=0.6, slope_exponent=1.0,
                      slit_count=2, slit_spacing_bohr_radii=3.1, slit_width_bohr_radii=1.05,
                      slit_rotation_radian=math.pi / 2),
             orc.Wall(potential_hartree=2.0, center_bohr_radii_3=(-3.0, 1.0, 0.0), normal_vector_3=(0.6, 0.8, 0.0),
                      plateau_thickness_bohr_radii=0.8, slope_thickness_bohr_radii=0.0, slit_count=1,
                      slit_width_bohr_radii=2.1, slit_rotation_radian=0.3)]
    # slit edges placed off the grid's float32 coordinates, so the oracle's correctly rounded
    # cos/sin and the device's cosf/sinf decide every voxel alike; a linear slope, so powf is
    # exact (the device's powf and numpy's float32 power differ by an ulp at some arguments,
    # the reference's kernels use powf as the engine does: tests/test_gpu_refpath.py)
    vel = [(-2.0, 0.37, 0.0), (1.5, 0.0, -0.45)]
    inner = tuple(0.5 * x - 3 * d for x, d in zip(L, dx))
    ab = orc.Absorbing(bottom=tuple(-v for v in inner), top=inner, offset=0.3, potential_pos=(-20.0,) * 3,
                       potential_neg=(-15.0,) * 3, exponent_pos=(2.0,) * 3, exponent_neg=(2.0,) * 3)
    sc = orc.Scenario(n=n, extent=L, sigma=(1.5, 1.5, 1.5), r0=(-4.0, 0.5, 0.0), k0=(2.0, 0.0, 0.3), dt=0.02,
                      double_precision=dbl, walls=walls, absorbing=ab)
    return sc, vel


def wall_args(w):
    return (w.potential_hartree, w.center_bohr_radii_3, w.normal_vector_3, w.plateau_thickness_bohr_radii,
            w.slope_thickness_bohr_radii, w.slope_exponent, w.slit_count, w.slit_spacing_bohr_radii,
            w.slit_width_bohr_radii, w.slit_rotation_radian)


def abs_args(a):
    return (a.bottom, a.top, a.offset, a.potential_pos, a.potential_neg, a.exponent_pos, a.exponent_neg)


def engine_for(sc, vel):
    from wavefunctionsimpython_gb300 import Engine

    e = Engine(sc.n, sc.extent, double_precision=sc.double_precision)
    e.add_absorbing(*abs_args(sc.absorbing))
    for w in sc.walls:
        e.add_wall(*wall_args(w))
    e.init_gaussian(sc.sigma, sc.r0, sc.k0)
    e.set_dynamic_walls([wall_args(w) for w in sc.walls], vel, abs_args(sc.absorbing))
    return e


def oracle_run(e, sc, vel, psi, V, walls, nsteps, taylor=False):
    """The oracle's dynamic loop, with the absorbing ramp taken from the engine (it does
    not move): the ramp's float32 atan and pow round differently on the host by up to two
    ulps, which would otherwise show in complex128 at 1e-10."""
    ramp = e.get_potential().imag.astype(np.float32)
    for _ in range(nsteps):
        if taylor:
            psi = orc.taylor_step(psi, V, sc.dx, 0.005, 1.0, order=10, stencil_order=4, nsteps=1)
        else:
            psi = orc.split_step(psi, V, sc.dx, sc.dt, 1.0, nsteps=1, double_precision=True)
        walls = orc.advect_walls(walls, vel, 0.005 if taylor else sc.dt)
        V = (orc.rebuild_potential(sc.n, sc.dx, walls, None).real + 1j * ramp).astype(np.complex64)
    return psi, V, walls


@pytest.mark.parametrize("dbl", [False, True])
def test_moving_walls_match_oracle(dbl):
    """25 steps: psi against the FP64 oracle, V against its rebuild (the wall part bit for
    bit; the absorbing ramp to the float32 rounding of atan and pow) and the centres."""
    n, L = (32, 32, 32), (16.0, 16.0, 16.0)
    sc, vel = scenario(n, L, dbl)
    e = engine_for(sc, vel)
    psi0 = e.get_psi()
    V0 = e.get_potential()
    np.testing.assert_allclose(V0.imag, sc.potential().imag, rtol=1e-6, atol=0)
    psi, V, walls = oracle_run(e, sc, vel, psi0.astype(np.complex128), V0, sc.walls, 25)
    e.step_split(25, sc.dt, 1.0)
    got_v = e.get_potential()
    assert np.array_equal(got_v.real, V.real)
    assert np.array_equal(got_v.imag, V.imag)
    np.testing.assert_array_equal(e.get_dynamic_walls(), np.array([w.center_bohr_radii_3 for w in walls]))
    assert walls[0].center_bohr_radii_3[0] == 0.0  # the first wall reached the x = 0 clamp
    assert rel(e.get_psi(), psi) < (C128_TOL if dbl else C64_TOL)
    e.close()


def test_moving_walls_device_loop_series():
    """run_split with moving walls records the same series as observing before each
    chunk of steps in the oracle's trajectory."""
    n, L = (32, 32, 32), (16.0, 16.0, 16.0)
    sc, vel = scenario(n, L, True)
    e = engine_for(sc, vel)
    psi = e.get_psi().astype(np.complex128)
    V, walls = e.get_potential(), sc.walls
    box = ((2, 2, 2), (27, 27, 27))
    series = []
    for k in range(4):
        series.append((orc.volume_probability(psi, sc.dx, *box), orc.expected_location(psi, sc.dx, *box)[0]))
        psi, V, walls = oracle_run(e, sc, vel, psi, V, walls, 5)
    ps, ls = e.run_split(20, sc.dt, 1.0, 5, [box], box)
    for k in range(4):
        assert abs(ps[k, 0] - series[k][0]) < 1e-10
        np.testing.assert_allclose(ls[k, :3], series[k][1], rtol=1e-9, atol=1e-11)
    assert rel(e.get_psi(), psi) < C128_TOL
    e.close()


def test_moving_walls_power_series():
    """The same update after each power-series step (V read directly by the term kernel)."""
    n, L = (32, 32, 32), (16.0, 16.0, 16.0)
    sc, vel = scenario(n, L, True)
    e = engine_for(sc, vel)
    psi = e.get_psi().astype(np.complex128)
    psi, V, walls = oracle_run(e, sc, vel, psi, e.get_potential(), sc.walls, 6, taylor=True)
    e.step_taylor(6, 0.005, 1.0, 10, 4)
    assert np.array_equal(e.get_potential().real, V.real)
    assert rel(e.get_psi(), psi) < C128_TOL
    e.close()


def test_moving_wall_step_cost_256():
    """At 256^3 (config 3's double slit with the wall sliding at 0.5 Bohr per unit time)
    a step with the update costs little more than a static step: only the band of voxels
    the wall sweeps is rewritten."""
    import torch

    from wavefunctionsimpython_gb300 import Engine

    sc = orc.config3_double_slit(256, 80.0)
    w = sc.walls[0]
    times = {}
    for moving in (False, True, False, True):
        e = Engine(sc.n, sc.extent)
        a = sc.absorbing
        e.add_absorbing(*abs_args(a))
        e.add_wall(*wall_args(w))
        e.init_gaussian(sc.sigma, sc.r0, sc.k0)
        if moving:
            e.set_dynamic_walls([wall_args(w)], [(0.5, 0.0, 0.0)], abs_args(a))
        e.step_split(3, sc.dt, 1.0)  # warm-up, includes the first (whole) rebuild
        e.synchronize()
        t0 = time.perf_counter()
        e.step_split(100, sc.dt, 1.0)
        e.synchronize()
        times.setdefault(moving, []).append(time.perf_counter() - t0)
        assert np.isfinite(e.norm())
        e.close()
        torch.cuda.empty_cache()
    ratio = min(times[True]) / min(times[False])
    print(f"moving / static step time at 256^3: {ratio:.3f} ({min(times[True]) * 10:.4f} vs "
          f"{min(times[False]) * 10:.4f} ms per step)")
    assert ratio < 1.2
