"""The engine against the reference project's own CUDA kernels (GPU only).

Two sources of reference results, both produced by the reference's kernel files
compiled unchanged (oracle/build_ref.py) and driven on the reference's own call
sequence with cuFFT for its transforms (oracle/ref_gpu.py):

* tests/golden/reference_gpu.npz, committed, made by
  tests/golden/make_ref_gpu_golden.py on a GB300: always checked;
* the live reference path, when oracle/_ref/ holds the compiled kernels: full
  fields at full sizes (config 3's 2000-step double slit, config 1's series).

Tolerances: complex64 results within 1e-5 relative L2 of the reference's
complex64 results over short runs (the workload's stated bar); complex128 within
1e-10 over the whole 2000-step run; observables within the reference's own FP32
atomic-sum rounding (2e-6 relative) in single precision. Over the 2000-step run
the reference's own complex64 path drifts 1e-3 from its complex128 path, so long
complex64 runs are bounded against the reference's complex128 run (see
test_config3_2000_steps_match_reference).
"""
import os

import numpy as np
import pytest

from oracle import wfs_oracle as orc

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "reference_gpu.npz")


def rel(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLDEN)


@pytest.fixture(scope="module")
def mk():
    import importlib.util

    spec = importlib.util.spec_from_file_location("make_ref_gpu_golden", os.path.join(HERE, "golden",
                                                                                      "make_ref_gpu_golden.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def engine(sc, dp=None):
    from wavefunctionsimpython_gb300 import Engine

    return Engine(sc.n, sc.extent, double_precision=sc.double_precision if dp is None else dp)


def build_potential(e, sc):
    if sc.ho_omega is not None:
        e.add_raw_potential(orc.harmonic_oscillator(sc.n, sc.dx, sc.ho_omega, sc.mass))
    if sc.absorbing is not None:
        a = sc.absorbing
        e.add_absorbing(a.bottom, a.top, a.offset, a.potential_pos, a.potential_neg, a.exponent_pos, a.exponent_neg)
    for w in sc.walls:
        e.add_wall(w.potential_hartree, w.center_bohr_radii_3, w.normal_vector_3, w.plateau_thickness_bohr_radii,
                   w.slope_thickness_bohr_radii, w.slope_exponent, w.slit_count, w.slit_spacing_bohr_radii,
                   w.slit_width_bohr_radii, w.slit_rotation_radian)


@pytest.mark.parametrize("dp", [False, True])
def test_packet_matches_reference(gold, mk, dp):
    sc = mk.grid_scenario(dp)
    e = engine(sc)
    e.init_gaussian(sc.sigma, sc.r0, sc.k0)
    got = e.get_psi()
    ref = gold["grid_psi0_f64" if dp else "grid_psi0_f32"]
    assert rel(got, ref) < (1e-13 if dp else 1e-6)
    e.close()


def test_potential_matches_reference(gold, mk):
    """Walls and absorbing ramp, built by the engine's kernels, against the reference's V."""
    sc = mk.grid_scenario(False)
    e = engine(sc)
    build_potential(e, sc)
    got = e.get_potential()
    ref = gold["grid_V"]
    d_re = got.real != ref.real
    d_im = np.abs(got.imag - ref.imag) / np.spacing(np.abs(ref.imag).astype(np.float32))
    print("real voxels differing:", int(d_re.sum()), "imag max ulp:", float(np.max(d_im)))
    assert np.array_equal(got.real, ref.real)
    assert np.array_equal(got.imag, ref.imag)
    e.close()


@pytest.mark.parametrize("dp", [False, True])
def test_split_steps_match_reference(gold, mk, dp):
    """10 split steps from the reference's own packet and potential."""
    sc = mk.grid_scenario(dp)
    tag = "f64" if dp else "f32"
    e = engine(sc)
    e.set_potential(gold["grid_V"])
    e.set_psi(gold[f"grid_psi0_{tag}"])
    e.step_split(mk.GRID_STEPS, sc.dt, 1.0)
    err = rel(e.get_psi(), gold[f"grid_psi_{tag}"])
    print(f"{tag}: 10 steps vs reference {err:.3e}")
    assert err < (1e-11 if dp else 1e-5)
    e.close()


@pytest.mark.parametrize("dp", [False, True])
def test_observables_match_reference(gold, mk, dp):
    sc = mk.grid_scenario(dp)
    tag = "f64" if dp else "f32"
    e = engine(sc)
    e.set_psi(gold[f"grid_psi_{tag}"])
    probs, r, r2 = e.observe(mk.GRID_BOXES, mk.GRID_BOXES[1])
    tol = 1e-12 if dp else 2e-6
    np.testing.assert_allclose(probs, gold[f"grid_vp_{tag}"], rtol=tol)
    np.testing.assert_allclose(r, gold[f"grid_el_{tag}"][:3], rtol=tol, atol=tol)
    np.testing.assert_allclose(r2, gold[f"grid_el_{tag}"][3:], rtol=tol)
    e.close()


def test_power_series_matches_reference(gold, mk):
    """Two order-10 steps with the reference's 2nd-order stencil (Δx-only division,
    clamped neighbours at the faces) on a 64^3 oscillator plus wall."""
    sc = mk.taylor_scenario()
    e = engine(sc)
    build_potential(e, sc)
    assert np.array_equal(e.get_potential()[mk.TAYLOR_PLANES], gold["taylor_V_planes"])
    e.init_gaussian(sc.sigma, sc.r0, sc.k0)
    e.step_taylor(mk.TAYLOR_STEPS, sc.dt, 1.0, 10, 2)
    psi = e.get_psi()
    err = rel(psi[mk.TAYLOR_PLANES], gold["taylor_psi_planes"])
    print(f"power series planes vs reference {err:.3e}")
    assert err < 1e-5
    np.testing.assert_allclose(mk.grid_sums(psi, sc.dx), gold["taylor_sums"], rtol=1e-5, atol=1e-6)
    e.close()


def test_config1_series_matches_reference(gold, mk):
    """64^3 complex128 barrier, 200 steps, norm and <r> every 10 steps on the whole grid."""
    sc = orc.config1_barrier_64()
    e = engine(sc)
    build_potential(e, sc)
    e.init_gaussian(sc.sigma, sc.r0, sc.k0)
    box = ((0, 0, 0), (63, 63, 63))
    ps, ls = e.run_split(200, sc.dt, 1.0, 10, [box], box)
    np.testing.assert_allclose(ps[:, 0], gold["cfg1_norm_series"], rtol=1e-11)
    np.testing.assert_allclose(ls[:, :3], gold["cfg1_loc_series"], rtol=1e-9, atol=1e-11)
    psi = e.get_psi()
    assert rel(psi[32], gold["cfg1_psi_plane32"]) < 1e-11
    np.testing.assert_allclose(mk.grid_sums(psi, sc.dx), gold["cfg1_sums"], rtol=1e-11)
    e.close()


def _cfg3(dp=False):
    sc = orc.config3_double_slit(256, 80.0)
    sc.double_precision = dp
    from wavefunctionsimpython_gb300 import Engine

    e = Engine(sc.n, sc.extent, double_precision=dp)
    build_potential(e, sc)
    e.init_gaussian(sc.sigma, sc.r0, sc.k0)
    return sc, e


def test_config3_two_steps_match_reference(gold):
    sc, e = _cfg3()
    e.step_split(2, sc.dt, 1.0)
    psi = e.get_psi()
    err = rel(psi[::8, ::8, ::8], gold["cfg3_psi2_sub8"])
    print(f"256^3 double slit, 2 steps, vs reference (every 8th site): {err:.3e}")
    assert err < 1e-5
    e.close()


def test_config3_2000_steps_match_reference(gold, mk):
    """The benchmark's whole run (2000 steps, P(x > 1) every 20 steps) against the
    reference's own runs of it (its kernels, cuFFT transforms).

    complex128: the engine follows the reference's complex128 run to round-off
    (measured 1.7e-12 on psi, 2.1e-12 on the series). complex64: the reference's
    complex64 run is itself 9.7e-4 (psi) and 1.3e-3 (series) away from its complex128
    run, because its cuFFT complex64 transforms lose 9e-7 of the norm per step; the
    engine's complex64 run is 9.6e-5 and 6.3e-5 away, ten times closer. Two complex64
    FFT implementations cannot agree to 1e-5 over this run when the reference alone
    drifts 1e-3, so the complex64 bounds are against the reference's complex128 run,
    with the distance to its complex64 run bounded by that run's own drift."""
    from wavefunctionsimpython_gb300 import Engine

    sc = orc.config3_double_slit(256, 80.0)
    box = mk.cfg3_box()
    runs = {}
    for dp in (False, True):
        e = Engine(sc.n, sc.extent, double_precision=dp)
        build_potential(e, sc)
        e.init_gaussian(sc.sigma, sc.r0, sc.k0)
        probs, _ = e.run_split(2000, sc.dt, 1.0, 20, [box], None)
        runs[dp] = (probs[:, 0].copy(), e.get_psi()[::16, ::16, ::16])
        e.close()

    def srel(a, b):
        return float(np.linalg.norm(np.asarray(a) - b) / np.linalg.norm(b))

    ref64_p, ref64_psi = gold["cfg3_p_series"], gold["cfg3_psi2000_sub16"]
    ref128_p, ref128_psi = gold["cfg3d_p_series"], gold["cfg3d_psi2000_sub16"]
    (p64, psi64), (p128, psi128) = runs[False], runs[True]
    own_drift = (rel(ref64_psi, ref128_psi), srel(ref64_p, ref128_p))
    print(f"complex128 vs reference complex128: psi {rel(psi128, ref128_psi):.3e}, series {srel(p128, ref128_p):.3e}")
    print(f"complex64 vs reference complex128: psi {rel(psi64, ref128_psi):.3e}, series {srel(p64, ref128_p):.3e}")
    print(f"reference complex64 vs its complex128: psi {own_drift[0]:.3e}, series {own_drift[1]:.3e}")
    print(f"complex64 vs reference complex64: psi {rel(psi64, ref64_psi):.3e}, series {srel(p64, ref64_p):.3e}")
    assert rel(psi128, ref128_psi) < 1e-10
    assert srel(p128, ref128_p) < 1e-10
    assert rel(psi64, ref128_psi) < 2e-4
    assert srel(p64, ref128_p) < 1.5e-4
    assert rel(psi64, ref128_psi) < 0.25 * own_drift[0]
    assert srel(p64, ref128_p) < 0.25 * own_drift[1]
    assert rel(psi64, ref64_psi) < 1.5 * own_drift[0]
    assert srel(p64, ref64_p) < 1.5 * own_drift[1]


@pytest.fixture(scope="module")
def live():
    from oracle import ref_gpu

    if not ref_gpu.available():
        pytest.skip("reference kernels not compiled (oracle/_ref/ is built where the reference sources are)")
    return ref_gpu


def test_config3_2000_steps_full_field_vs_live_reference(live):
    """Full 256^3 fields after the 2000-step run, complex128 against the reference's
    complex128 run of its own kernels (the reference's complex64 run drifts 1e-3 from
    both, see the fixture test)."""
    sc, e = _cfg3(True)
    e.step_split(2000, sc.dt, 1.0)
    got = e.get_psi()
    e.close()
    sim = live.RefSim(sc.n, sc.extent, True)
    sim.build_scenario(sc)
    sim.split_step(sc.dt, 1.0, 2000)
    ref = sim.get_psi()
    err = rel(got, ref)
    print(f"256^3 double slit, 2000 steps, complex128 full field vs live reference: {err:.3e}")
    assert err < 1e-10


def test_config3_potential_vs_live_reference(live):
    sc, e = _cfg3()
    got = e.get_potential()
    e.close()
    sim = live.RefSim(sc.n, sc.extent, False)
    sim.build_scenario(sc)
    ref = sim.get_potential()
    print("256^3 potential: real voxels differing", int(np.sum(got.real != ref.real)),
          "imag voxels differing", int(np.sum(got.imag != ref.imag)))
    assert np.array_equal(got, ref)
