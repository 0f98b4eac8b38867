"""Generates tests/golden/reference_gpu.npz: outputs of the reference project's own CUDA
kernels, run on a GPU through oracle/ref_gpu.py on the reference's own call sequence.

Run on a machine with a GPU after ``python oracle/build_ref.py`` has compiled the
reference kernels into oracle/_ref/:

    python tests/golden/make_ref_gpu_golden.py OUT.npz

Cases (all inputs seeded or analytic; every array small):

* ``grid_*``: a (32, 24, 16) grid over (24, 18, 12) Bohr with two walls (one with
  a slope and two slits, one tilted with one slit) and an absorbing ramp with
  per-axis heights and exponents; the packet in complex64 and complex128, the
  potential, 10 split steps of dt 0.02 in both precisions, then volume
  probabilities of three boxes and the expected location of one.
* ``taylor_*``: 64^3 over 16 Bohr, harmonic oscillator plus a wall, 2 power-series
  steps (order 10, dt 0.002) with the reference's 2nd-order stencil; the planes
  x = 28..35 of psi and whole-grid sums.
* ``cfg1_*``: 64^3 complex128 barrier (60 Bohr, dt 0.01), 200 steps; norm and <r>
  every 10 steps on the whole grid, the plane x = 32 of the final psi.
* ``cfg3_*``: 256^3 complex64 double slit (80 Bohr, dt 0.01); psi after 2 steps
  sampled every 8th site per axis; the 2000-step run's P(x > 1) every 20 steps and
  its final psi sampled every 16th site; ``cfg3d_*`` the same 2000-step run in
  complex128.
"""
from __future__ import annotations

import math
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import ref_gpu  # noqa: E402
from oracle import wfs_oracle as orc  # noqa: E402

GRID_N = (32, 24, 16)
GRID_L = (24.0, 18.0, 12.0)
GRID_DT = 0.02
GRID_STEPS = 10
GRID_BOXES = [((4, 4, 2), (21, 15, 11)), ((1, 1, 1), (29, 21, 13)), ((0, 0, 0), (31, 23, 15))]


def grid_scenario(double_precision):
    dxv = GRID_L[0] / GRID_N[0]
    inner = tuple(0.5 * GRID_L[a] - 3 * dxv for a in range(3))
    return orc.Scenario(
        n=GRID_N, extent=GRID_L, sigma=(1.5, 1.2, 1.0), r0=(-4.0, 0.5, -0.25), k0=(1.5, 0.3, -0.2), dt=GRID_DT,
        double_precision=double_precision,
        walls=[orc.Wall(potential_hartree=3.0, center_bohr_radii_3=(1.0, 0.0, 0.0), normal_vector_3=(1.0, 0.0, 0.0),
                        plateau_thickness_bohr_radii=1.0, slope_thickness_bohr_radii=0.75, slope_exponent=1.5,
                        slit_count=2, slit_spacing_bohr_radii=3.0, slit_width_bohr_radii=1.0,
                        slit_rotation_radian=math.pi / 2),
               orc.Wall(potential_hartree=1.0, center_bohr_radii_3=(-1.0, 0.5, 0.0), normal_vector_3=(0.6, 0.8, 0.0),
                        plateau_thickness_bohr_radii=0.5, slope_thickness_bohr_radii=0.0, slit_count=1,
                        slit_width_bohr_radii=2.0, slit_rotation_radian=0.3)],
        absorbing=orc.Absorbing(bottom=tuple(-v for v in inner), top=inner, offset=0.5,
                                potential_pos=(-20.0, -15.0, -10.0), potential_neg=(-25.0, -20.0, -5.0),
                                exponent_pos=(2.0, 1.5, 3.0), exponent_neg=(2.0, 2.0, 1.0)))


TAYLOR_N = (64, 64, 64)
TAYLOR_L = (16.0, 16.0, 16.0)
TAYLOR_DT = 0.002
TAYLOR_STEPS = 2
TAYLOR_PLANES = slice(28, 36)


def taylor_scenario():
    return orc.Scenario(n=TAYLOR_N, extent=TAYLOR_L, sigma=(1.0, 1.0, 1.0), r0=(-1.5, 0.3, 0.0), k0=(2.0, 0.0, 0.5),
                        dt=TAYLOR_DT, ho_omega=1.0,
                        walls=[orc.Wall(potential_hartree=5.0, plateau_thickness_bohr_radii=0.5,
                                        slope_thickness_bohr_radii=0.0)])


def grid_sums(psi, dx):
    """Whole-grid sums used to pin a field without storing it: norm, sum psi, <x>-like moment."""
    p = np.asarray(psi, np.complex128)
    a2 = np.abs(p) ** 2
    x = (np.arange(p.shape[0]) - p.shape[0] // 2) * dx[0]
    return np.array([a2.sum(), p.sum().real, p.sum().imag, (a2 * x[:, None, None]).sum()])


def cfg3_box():
    inner = 40.0 - 16 * (80.0 / 256)
    bv, cnt = orc.simpson_box_from_corners((1.0, -inner, -inner), (inner, inner, inner), (80.0,) * 3, (256,) * 3)
    return tuple(int(v) for v in bv), tuple(int(v) for v in cnt)


def main(out):
    import torch

    torch.cuda.init()
    torch.zeros(1, device="cuda")
    res = {}

    # -- fixture grid: packet, potential, 10 split steps, observables -------------
    for dp, tag in ((False, "f32"), (True, "f64")):
        sc = grid_scenario(dp)
        sim = ref_gpu.RefSim(sc.n, sc.extent, dp)
        sim.build_scenario(sc)
        res[f"grid_psi0_{tag}"] = sim.get_psi()
        if not dp:
            res["grid_V"] = sim.get_potential()
        sim.split_step(sc.dt, 1.0, GRID_STEPS)
        res[f"grid_psi_{tag}"] = sim.get_psi()
        res[f"grid_vp_{tag}"] = np.array([sim.volume_probability(b, c) for b, c in GRID_BOXES])
        er, er2 = sim.expected_location(*GRID_BOXES[1])
        res[f"grid_el_{tag}"] = np.concatenate([er, er2])

    # -- power series ---------------------------------------------------------------
    sc = taylor_scenario()
    sim = ref_gpu.RefSim(sc.n, sc.extent, False)
    sim.build_scenario(sc)
    res["taylor_V_planes"] = sim.get_potential()[TAYLOR_PLANES]
    sim.taylor_step(sc.dt, 1.0, 10, TAYLOR_STEPS)
    psi = sim.get_psi()
    res["taylor_psi_planes"] = psi[TAYLOR_PLANES]
    res["taylor_sums"] = grid_sums(psi, sim.dx)

    # -- config 1: 64^3 complex128 barrier, 200 steps, series every 10 -----------------
    sc = orc.config1_barrier_64()
    sim = ref_gpu.RefSim(sc.n, sc.extent, True)
    sim.build_scenario(sc)
    norms, locs = [], []
    for _ in range(20):
        norms.append(sim.volume_probability((0, 0, 0), (63, 63, 63)))
        locs.append(sim.expected_location((0, 0, 0), (63, 63, 63))[0])
        sim.split_step(sc.dt, 1.0, 10)
    res["cfg1_norm_series"] = np.array(norms)
    res["cfg1_loc_series"] = np.array(locs)
    psi = sim.get_psi()
    res["cfg1_psi_plane32"] = psi[32]
    res["cfg1_sums"] = grid_sums(psi, sim.dx)

    # -- config 3: 256^3 complex64 double slit ------------------------------------------
    sc = orc.config3_double_slit(256, 80.0)
    sim = ref_gpu.RefSim(sc.n, sc.extent, False)
    sim.build_scenario(sc)
    sim.split_step(sc.dt, 1.0, 2)
    psi = sim.get_psi()
    res["cfg3_psi2_sub8"] = psi[::8, ::8, ::8]
    res["cfg3_sums2"] = grid_sums(psi, sim.dx)
    bv, cnt = cfg3_box()
    sim = ref_gpu.RefSim(sc.n, sc.extent, False)
    sim.build_scenario(sc)
    series = []
    for _ in range(100):
        series.append(sim.volume_probability(bv, cnt))
        sim.split_step(sc.dt, 1.0, 20)
    res["cfg3_p_series"] = np.array(series)
    psi = sim.get_psi()
    res["cfg3_psi2000_sub16"] = psi[::16, ::16, ::16]
    res["cfg3_sums2000"] = grid_sums(psi, sim.dx)
    res["cfg3_p_final"] = np.array([sim.volume_probability(bv, cnt)])
    del sim
    torch.cuda.empty_cache()
    sim = ref_gpu.RefSim(sc.n, sc.extent, True)
    sim.build_scenario(sc)
    series = []
    for _ in range(100):
        series.append(sim.volume_probability(bv, cnt))
        sim.split_step(sc.dt, 1.0, 20)
    res["cfg3d_p_series"] = np.array(series)
    psi = sim.get_psi()
    res["cfg3d_psi2000_sub16"] = psi[::16, ::16, ::16]
    res["cfg3d_sums2000"] = grid_sums(psi, sim.dx)

    np.savez_compressed(out, **res)
    print(f"wrote {out}: " + ", ".join(f"{k}{list(v.shape)}" for k, v in res.items()))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_ref_gpu_golden.py OUT.npz")
    if not ref_gpu.available():
        sys.exit("reference kernels missing: run oracle/build_ref.py first")
    main(sys.argv[1])
