"""Checks at the workloads' own sizes (GPU only): the 64^3 complex128 barrier series
against the FP64 oracle, the 128^3 power-series oscillator against the analytic
<x>(t) and the split step, the 256^3 double slit against the FP64 oracle plus
size-independent properties (unitarity, time reversal, linearity), and every
instance of the 256-instance batched sweep."""
import math
import os

import numpy as np
import pytest

from oracle import wfs_oracle as orc

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def scipy_fft():
    import scipy.fft as sf

    w = os.cpu_count() or 1
    return (lambda a, norm: sf.fftn(a, norm=norm, workers=w), lambda a, norm: sf.ifftn(a, norm=norm, workers=w))


def engine_for(sc, V=None):
    from wavefunctionsimpython_gb300 import Engine

    e = Engine(sc.n, sc.extent, double_precision=sc.double_precision)
    e.set_potential(sc.potential() if V is None else V)
    e.init_gaussian(sc.sigma, sc.r0, sc.k0)
    return e


def test_barrier_64_c128_series_matches_fp64_oracle():
    """64^3 over 60 Bohr, complex128, 1 Ha barrier, dt 0.01, 200 steps, norm / <r> / <r^2> every 10."""
    sc = orc.config1_barrier_64()
    e = engine_for(sc)
    box = ((0, 0, 0), (63, 63, 63))
    ps, ls = e.run_split(200, sc.dt, 1.0, 10, [box], box)
    V = sc.potential()
    psi = sc.psi0()
    for k in range(20):
        assert abs(ps[k, 0] - orc.volume_probability(psi, sc.dx, *box)) < 1e-9
        rr, rr2 = orc.expected_location(psi, sc.dx, *box)
        np.testing.assert_allclose(ls[k, :3], rr, rtol=1e-9, atol=1e-10)
        np.testing.assert_allclose(ls[k, 3:], rr2, rtol=1e-9, atol=1e-10)
        psi = orc.split_step(psi, V, sc.dx, sc.dt, 1.0, nsteps=10)
    assert rel(e.get_psi(), psi) < 1e-11


def test_oscillator_128_power_series_follows_ehrenfest():
    """128^3 over 40 Bohr, complex64, omega 0.5, Taylor p=10 with the 4th-order Laplacian,
    dt 0.005, 1000 steps: <x>(t) = x0 cos(omega t) exactly for a harmonic potential, which
    the spectral split step follows to 2e-2 Bohr; the power series' finite-difference
    Laplacian (dispersion error ~(k dx)^4 / 90 at the packet's k dx ~ 0.8) stays within
    0.1 Bohr of both; the norm is kept."""
    sc = orc.config2_ho_128()
    box = ((0, 0, 0), (127, 127, 127))
    taylor, split = engine_for(sc), engine_for(sc)
    n0 = taylor.norm()
    taylor.step_taylor(1000, sc.dt, 1.0, 10, 4)
    split.step_split(1000, sc.dt, 1.0)
    x_t = taylor.observe((), box)[1][0]
    x_s = split.observe((), box)[1][0]
    x_exact = sc.r0[0] * math.cos(0.5 * 1000 * sc.dt)
    assert abs(x_s - x_exact) < 2e-2, (x_s, x_exact)
    assert abs(x_t - x_exact) < 0.1, (x_t, x_exact)
    assert abs(x_t - x_s) < 0.1
    assert abs(taylor.norm() / n0 - 1.0) < 1e-4


@pytest.fixture(scope="module")
def slit():
    return orc.config3_double_slit(256, 80.0)


def test_double_slit_256_two_steps_match_fp64_oracle(slit):
    e = engine_for(slit)
    e.step_split(2, slit.dt, 1.0)
    ref = orc.split_step(slit.psi0().astype(np.complex128), slit.potential().astype(np.complex128), slit.dx, slit.dt,
                         1.0, nsteps=2, double_precision=True, fft=scipy_fft())
    assert rel(e.get_psi(), ref) < 1e-5


def test_double_slit_256_unitarity_and_time_reversal(slit):
    """Without the absorber V is real: the step is unitary and dt -> -dt undoes it
    (measured: norm +1.4e-5 over 200 steps, reversal 2.8e-5)."""
    V = np.zeros(slit.n, np.complex64)
    orc.add_potential_wall(V, slit.dx, slit.walls[0])
    e = engine_for(slit, V)
    psi0 = e.get_psi()
    n0 = e.norm()
    e.step_split(200, slit.dt, 1.0)
    assert abs(e.norm() / n0 - 1.0) < 5e-5
    e.step_split(200, -slit.dt, 1.0)
    assert rel(e.get_psi(), psi0) < 1e-4


def test_double_slit_256_2000_step_trajectory_vs_complex128(slit):
    """The whole double-slit run of the benchmark (2000 steps, absorber on, P(x > 1) every
    20 steps) in complex64 against the same run in complex128, whose single steps match
    the FP64 oracle to 1e-11. An FFT-based oracle run of 2000 steps at 256^3 would take
    hours on the host, so the complex128 engine stands in for it here.

    Rounded butterfly constants shrink every complex64 transform by a fixed fraction
    (-3.2e-7 of the norm per step at 256^3, -5.6e-4 over this run). The engine folds the
    inverse of that gain into its kinetic tables, which leaves 9.6e-5 relative L2 on psi
    and 2.4e-5 on the P(x > 1) series after 2000 steps. The bounds below sit at about
    twice the measured values and below what the run gives without the compensation
    (2.9e-4 on psi, 1.9e-4 on the series)."""
    from wavefunctionsimpython_gb300 import Engine

    dx = 80.0 / 256
    inner = 40.0 - 16 * dx
    b = np.array([1.0, -inner, -inner])
    t = np.array([inner, inner, inner])
    bv = ((b + 40.0) / dx).astype(np.int64)
    tv = ((t + 40.0) / dx).astype(np.int64) + 1
    cnt = np.minimum(tv - bv, 256 - bv)
    cnt = np.where(cnt % 2 == 0, cnt - 1, cnt)  # Simpson needs an odd sample count
    box = (tuple(int(v) for v in bv), tuple(int(v) for v in cnt))
    runs = {}
    for dbl in (False, True):
        e = Engine(slit.n, slit.extent, double_precision=dbl)
        e.set_potential(slit.potential())
        e.init_gaussian(slit.sigma, slit.r0, slit.k0)
        probs, _ = e.run_split(2000, slit.dt, 1.0, 20, [box], None)
        runs[dbl] = (np.asarray(probs, np.float64).ravel(), e.get_psi().astype(np.complex128), e.norm())
        e.close()
    (p64, psi64, n64), (p128, psi128, n128) = runs[False], runs[True]
    assert p128.size == 100 and p128.max() > 0.3  # a third of the packet has passed the slits
    assert rel(psi64, psi128) < 2e-4
    assert np.max(np.abs(p64 - p128)) < 6e-5
    assert abs(n64 / n128 - 1.0) < 2e-4


def test_double_slit_256_linearity(slit):
    from wavefunctionsimpython_gb300 import Engine

    V = slit.potential()
    p1 = slit.psi0()
    p2 = orc.gaussian_wave_packet(slit.n, slit.dx, (2.0,) * 3, (-15.0, 4.0, 0.0), (1.5, -0.5, 0.0), False)
    a, b = 0.6, 0.8j
    outs = []
    for p in (p1, p2, (a * p1 + b * p2).astype(np.complex64)):
        e = Engine(slit.n, slit.extent)
        e.set_potential(V)
        e.set_psi(p)
        e.step_split(20, slit.dt, 1.0)
        outs.append(e.get_psi())
        e.close()
    assert rel(outs[2], a * outs[0].astype(np.complex128) + b * outs[1]) < 1e-5


def test_batched_sweep_full_mix():
    """The 256-instance sweep (128x32^3, 64x48^3, 48x64^3, 16x96^3) for 500 steps. Every
    instance keeps its norm (barriers only, no absorber) to 2e-4 (measured at most 8.7e-5),
    and two instances of every size agree with the single-grid engine to 2e-5 (measured
    6.5e-6) and with the complex128 engine to 1e-4 (measured 3.8e-5). Over 500 steps
    complex64 rounding accumulates past the 1e-5 that short runs meet against the FP64
    oracle."""
    from wavefunctionsimpython_gb300 import Engine
    from wavefunctionsimpython_gb300._lib import Batch

    mix = [(32, 128), (48, 64), (64, 48), (96, 16)]
    sizes = [n for n, c in mix for _ in range(c)]
    rng = np.random.default_rng(2024)
    L = 40.0
    b = Batch(sizes, [L] * len(sizes))
    params = []
    for i, n in enumerate(sizes):
        U, w = rng.uniform(0.2, 2.0), rng.uniform(1.0, 4.0)
        k0, sig, x0 = rng.uniform(0.5, 3.0), rng.uniform(1.0, 3.0), rng.uniform(-12.0, -6.0)
        b.add_wall(i, U, (0, 0, 0), (1, 0, 0), w)
        b.init_gaussian(i, (sig,) * 3, (x0, 0, 0), (k0, 0, 0))
        params.append((U, w, k0, sig, x0))
    norms0 = [float(np.sum(np.abs(b.get_psi(i).astype(np.complex128)) ** 2)) for i in range(len(sizes))]
    b.run(500, 0.01, 1.0, graph=True)
    b.synchronize()
    for i in range(len(sizes)):
        n1 = float(np.sum(np.abs(b.get_psi(i).astype(np.complex128)) ** 2))
        assert abs(n1 / norms0[i] - 1.0) < 2e-4, i
    first = {}
    for i, n in enumerate(sizes):
        first.setdefault(n, []).append(i)
    for n, idx in first.items():
        for i in (idx[0], idx[-1]):
            U, w, k0, sig, x0 = params[i]
            single = {}
            for dbl in (False, True):
                e = Engine((n,) * 3, (L,) * 3, double_precision=dbl)
                e.add_wall(U, (0, 0, 0), (1, 0, 0), w)
                e.init_gaussian((sig,) * 3, (x0, 0, 0), (k0, 0, 0))
                e.step_split(500, 0.01, 1.0)
                single[dbl] = e.get_psi()
                e.close()
            psi_b = b.get_psi(i)
            assert rel(psi_b, single[False]) < 2e-5, (n, i)
            assert rel(psi_b, single[True]) < 1e-4, (n, i)


@pytest.mark.parametrize("n", [512, 1024])
def test_maximum_sizes_keep_norm_and_reverse(n):
    """The largest grids: 512^3 (fused plane pass) and 1024^3 (per-axis passes, 8 GiB psi
    plus V and the phase table) keep the norm with a real barrier and return to the
    initial <r>, <r^2> after dt -> -dt; everything stays on the device."""
    from wavefunctionsimpython_gb300 import Engine

    L = 80.0
    e = Engine((n,) * 3, (L,) * 3)
    e.add_wall(5.0, (0.0, 0.0, 0.0), (1.0, 0.0, 0.0), 1.0)
    e.init_gaussian((3.0,) * 3, (-10.0, 1.0, 0.0), (2.0, 0.0, 0.5))
    box = ((1, 1, 1), (n - 3, n - 3, n - 3))
    n0 = e.norm()
    _, r0, q0 = e.observe((), box)
    e.step_split(10, 0.01, 1.0)
    _, r1, _ = e.observe((), box)
    assert abs(r1[0] - r0[0]) > 0.1          # the packet moved
    assert abs(e.norm() / n0 - 1.0) < 1e-5
    e.step_split(10, -0.01, 1.0)
    _, r2, q2 = e.observe((), box)
    np.testing.assert_allclose(r2, r0, atol=1e-4)
    np.testing.assert_allclose(q2, q0, rtol=1e-4)
    e.close()


def test_observables_at_256_accurate_to_1e9(slit):
    """Compensated (float-float) thread and warp sums with FP64 CTA and grid sums: at 256^3
    complex64 the volume probabilities and <r>, <r^2> from both observation paths (the
    fused transform after split steps and the real-space kernel) agree with FP64 sums
    of the same psi to 1e-9."""
    e = engine_for(slit)
    e.step_split(10, slit.dt, 1.0)
    inner = 40.0 - 16 * slit.dx[0]
    trans = orc.simpson_box_from_corners((1.0, -inner, -inner), (inner, inner, inner), slit.extent, slit.n)
    obsb = orc.simpson_box_from_corners((-inner,) * 3, (inner,) * 3, slit.extent, slit.n)
    left = orc.simpson_box_from_corners((-inner,) * 3, (0.0, inner, inner), slit.extent, slit.n)
    boxes = [tuple(map(tuple, b)) for b in (trans, obsb, left)]
    fused = e.observe(boxes, boxes[1])  # from the split step's frequency-space state
    psi = e.get_psi()
    real = e.observe(boxes, boxes[1])   # from real-space psi
    ref_p = [orc.volume_probability(psi, slit.dx, *b) for b in boxes]
    ref_r, ref_r2 = orc.expected_location(psi, slit.dx, *boxes[1])
    scale_r = float(np.sqrt(np.max(ref_r2)))
    for name, (probs, r, r2) in (("fused", fused), ("real", real)):
        print(name, "probabilities", np.abs(np.asarray(probs) / np.asarray(ref_p) - 1.0),
              "<r>", np.abs(r - ref_r) / scale_r, "<r^2>", np.abs(r2 / ref_r2 - 1.0))
        np.testing.assert_allclose(probs[1:], ref_p[1:], rtol=1e-9)
        assert abs(probs[0] - ref_p[0]) < 1e-9 * ref_p[1]  # P(x > 1) is still ~0 after 10 steps
        np.testing.assert_allclose(r, ref_r, rtol=0, atol=1e-9 * scale_r)
        np.testing.assert_allclose(r2, ref_r2, rtol=1e-9)
    e.close()
