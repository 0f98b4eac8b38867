"""The CPU oracle against outputs of the reference project's own CUDA kernels.

tests/golden/reference_gpu.npz holds results of the reference's kernel files,
compiled unchanged and run on a GB300 on the reference's own call sequence with
cuFFT for its transforms (tests/golden/make_ref_gpu_golden.py, oracle/ref_gpu.py).
These tests pin the NumPy restatement in oracle/wfs_oracle.py to them: the
geometry of the potential, the packet, the split step in both precisions, the
power series with the reference's 2nd-order stencil, and the Simpson
observables. They run on the CPU only.
"""
import importlib.util
import os

import numpy as np
import pytest

from oracle import wfs_oracle as orc

HERE = os.path.dirname(os.path.abspath(__file__))


def rel(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def gold():
    return np.load(os.path.join(HERE, "golden", "reference_gpu.npz"))


@pytest.fixture(scope="module")
def mk():
    spec = importlib.util.spec_from_file_location("make_ref_gpu_golden",
                                                  os.path.join(HERE, "golden", "make_ref_gpu_golden.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def test_walls_bit_exact_and_ramp_within_ulps(gold, mk):
    """Two walls (one tilted so that 27 voxels lie exactly on its plateau edge, where the
    reference compiler's fused multiply-adds decide) are bit-exact; the absorbing ramp is
    within a few float32 ulps (the reference's atanf/powf are not correctly rounded at
    every argument, the oracle's are)."""
    V = mk.grid_scenario(False).potential()
    ref = gold["grid_V"]
    assert np.array_equal(V.real, ref.real)
    np.testing.assert_allclose(V.imag, ref.imag, rtol=5e-7, atol=0)


@pytest.mark.parametrize("dp", [False, True])
def test_packet(gold, mk, dp):
    sc = mk.grid_scenario(dp)
    tag = "f64" if dp else "f32"
    assert rel(sc.psi0(), gold[f"grid_psi0_{tag}"]) < (1e-14 if dp else 1e-6)


def test_split_step_fp64_matches_reference_fp64(gold, mk):
    """Ten double-precision steps from the reference's own packet and potential."""
    sc = mk.grid_scenario(True)
    ref = orc.split_step(gold["grid_psi0_f64"], gold["grid_V"], sc.dx, sc.dt, 1.0, nsteps=mk.GRID_STEPS,
                         double_precision=True)
    assert rel(ref, gold["grid_psi_f64"]) < 1e-13


def test_split_step_reference_fp32_error(gold, mk):
    """The reference's single-precision path is within 1e-5 of the FP64 oracle after ten
    steps (its own complex64 rounding)."""
    sc = mk.grid_scenario(False)
    ref = orc.split_step(gold["grid_psi0_f32"].astype(np.complex128), gold["grid_V"], sc.dx, sc.dt, 1.0,
                         nsteps=mk.GRID_STEPS, double_precision=True)
    assert rel(gold["grid_psi_f32"], ref) < 1e-5


@pytest.mark.parametrize("dp", [False, True])
def test_observables(gold, mk, dp):
    """Simpson volume probabilities of three boxes and the expected location of one;
    single precision carries the reference's FP32 atomic sums."""
    sc = mk.grid_scenario(dp)
    tag = "f64" if dp else "f32"
    psi = gold[f"grid_psi_{tag}"]
    tol = 1e-13 if dp else 2e-6
    got = [orc.volume_probability(psi, sc.dx, b, c) for b, c in mk.GRID_BOXES]
    np.testing.assert_allclose(got, gold[f"grid_vp_{tag}"], rtol=tol)
    er, er2 = orc.expected_location(psi, sc.dx, *mk.GRID_BOXES[1])
    np.testing.assert_allclose(er, gold[f"grid_el_{tag}"][:3], rtol=tol, atol=tol)
    np.testing.assert_allclose(er2, gold[f"grid_el_{tag}"][3:], rtol=tol)


def test_power_series_reference_stencil(gold, mk):
    """Two order-10 power-series steps with the reference's 2nd-order stencil (its Δx-only
    division and clamped face neighbours) in FP64 against the reference's complex64 run."""
    sc = mk.taylor_scenario()
    V = sc.potential()
    assert np.array_equal(V[mk.TAYLOR_PLANES], gold["taylor_V_planes"])
    psi = orc.taylor_step(sc.psi0().astype(np.complex128), V, sc.dx, sc.dt, 1.0, order=10, stencil_order=2,
                          nsteps=mk.TAYLOR_STEPS)
    assert rel(psi[mk.TAYLOR_PLANES], gold["taylor_psi_planes"]) < 1e-5
    np.testing.assert_allclose(mk.grid_sums(psi, sc.dx), gold["taylor_sums"], rtol=1e-5, atol=1e-6)


def test_config1_series(gold):
    """64^3 complex128 barrier over 200 steps: norm and <r> every 10 steps, the final field."""
    sc = orc.config1_barrier_64()
    V = sc.potential()
    psi = sc.psi0()
    box = ((0, 0, 0), (63, 63, 63))
    norms, locs = [], []
    for _ in range(20):
        norms.append(orc.volume_probability(psi, sc.dx, *box))
        locs.append(orc.expected_location(psi, sc.dx, *box)[0])
        psi = orc.split_step(psi, V, sc.dx, sc.dt, 1.0, nsteps=10, double_precision=True)
    np.testing.assert_allclose(norms, gold["cfg1_norm_series"], rtol=1e-12)
    np.testing.assert_allclose(np.array(locs), gold["cfg1_loc_series"], rtol=1e-10, atol=1e-12)
    assert rel(psi[32], gold["cfg1_psi_plane32"]) < 1e-11
    np.testing.assert_allclose(mk_sums(psi, sc.dx), gold["cfg1_sums"], rtol=1e-11)


def mk_sums(psi, dx):
    p = np.asarray(psi, np.complex128)
    a2 = np.abs(p) ** 2
    x = (np.arange(p.shape[0]) - p.shape[0] // 2) * dx[0]
    return np.array([a2.sum(), p.sum().real, p.sum().imag, (a2 * x[:, None, None]).sum()])
