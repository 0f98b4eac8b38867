"""The drop-in modules end to end on the GPU: a reference-schema config through
SimState / MeasurementTools / core_sim, checked against the oracle (GPU only)."""
import copy
import os

import numpy as np
import pytest

from oracle import wfs_oracle as orc

pytestmark = pytest.mark.gpu


def base_config(tmp_path, method="fourier", dbl=True, saving=False):
    return {
        "simulation": {"method": method, "order_of_approximation": 10, "delta_time_h_bar_per_hartree": 0.02,
                       "total_iteration_count": 12, "is_dynamic_potential_mode": False,
                       "enable_wave_function_saving": saving, "wave_function_save_iteration_interval": 4,
                       "double_precision_calculation": dbl},
        "wave_packet": {"path": "", "particle_mass_electron_rest_mass": 1.0,
                        "initial_position_bohr_radii_3": [-4.0, 0.0, 0.0],
                        "initial_velocity_bohr_radii_hartree_per_h_bar_3": [1.5, 0.0, 0.0],
                        "initial_standard_deviation_bohr_radii_3": [2.0, 2.0, 2.0]},
        "volume": {"simulated_volume_dimensions_bohr_radii_3": [32.0, 16.0, 16.0],
                   "number_of_voxels_3": [64, 32, 32],
                   "observation_box_bottom_corner_bohr_radii_3": [-12.0, -6.0, -6.0],
                   "observation_box_top_corner_bohr_radii_3": [12.0, 6.0, 6.0]},
        "absorbing_boundary_condition": {"outer_potential_in_positive_xyz_direction_hartree_3": [-20.0, -5.0, -5.0],
                                         "outer_potential_in_negative_xyz_direction_hartree_3": [-20.0, -5.0, -5.0],
                                         "start_offset": 0.5,
                                         "slope_exponent_in_positive_xyz_direction_3": [2.0, 2.0, 2.0],
                                         "slope_exponent_in_negative_xyz_direction_3": [2.0, 2.0, 2.0],
                                         "enable": True},
        "potential": {"walls": [{"potential_hartree": 2.0, "center_bohr_radii_3": [1.0, 0.0, 0.0],
                                 "normal_vector_3": [1.0, 0.0, 0.0], "plateau_thickness_bohr_radii": 1.0,
                                 "slope_thickness_bohr_radii": 0.5, "slope_exponent": 1.5, "slit_count": 2,
                                 "slit_spacing_bohr_radii": 4.0, "slit_width_bohr_radii": 1.5,
                                 "slit_rotation_radian": 1.5707963, "enable": True}]},
        "measurement": {"expected_location": {"enable_image": True},
                        "volume_probabilities": [
                            {"name": "left", "bottom_corner_bohr_radii_3": [-12.0, -6.0, -6.0],
                             "top_corner_bohr_radii_3": [0.0, 6.0, 6.0], "enable_image": True},
                            {"name": "right", "bottom_corner_bohr_radii_3": [0.0, -6.0, -6.0],
                             "top_corner_bohr_radii_3": [12.0, 6.0, 6.0], "enable_image": True}]},
        "paths": {"cache_dir": str(tmp_path / "cache"), "output_dir": str(tmp_path / "output")},
    }


def oracle_run(cfg, s):
    """Oracle: psi0 and V built the reference's way, then measure-before-step for every step."""
    n = tuple(cfg["volume"]["number_of_voxels_3"])
    L = tuple(cfg["volume"]["simulated_volume_dimensions_bohr_radii_3"])
    dx = orc.delta_x(L, n)
    wp = cfg["wave_packet"]
    psi = orc.gaussian_wave_packet(n, dx, wp["initial_standard_deviation_bohr_radii_3"],
                                   wp["initial_position_bohr_radii_3"], wp["initial_velocity_bohr_radii_hartree_per_h_bar_3"],
                                   True)
    ab = cfg["absorbing_boundary_condition"]
    V = np.zeros(n, np.complex64)
    orc.add_absorbing_potential(V, dx, orc.Absorbing(
        bottom=tuple(s.get_observation_box_bottom_corner_bohr_radii_3()), top=tuple(s.get_observation_box_top_corner_bohr_radii_3()),
        offset=ab["start_offset"], potential_pos=ab["outer_potential_in_positive_xyz_direction_hartree_3"],
        potential_neg=ab["outer_potential_in_negative_xyz_direction_hartree_3"],
        exponent_pos=ab["slope_exponent_in_positive_xyz_direction_3"], exponent_neg=ab["slope_exponent_in_negative_xyz_direction_3"]))
    w = cfg["potential"]["walls"][0]
    orc.add_potential_wall(V, dx, orc.Wall(potential_hartree=w["potential_hartree"], center_bohr_radii_3=w["center_bohr_radii_3"],
                                           normal_vector_3=w["normal_vector_3"], plateau_thickness_bohr_radii=w["plateau_thickness_bohr_radii"],
                                           slope_thickness_bohr_radii=w["slope_thickness_bohr_radii"], slope_exponent=w["slope_exponent"],
                                           slit_count=w["slit_count"], slit_spacing_bohr_radii=w["slit_spacing_bohr_radii"],
                                           slit_width_bohr_radii=w["slit_width_bohr_radii"], slit_rotation_radian=w["slit_rotation_radian"]))
    return dx, V, psi


@pytest.mark.parametrize("saving", [False, True])
def test_run_iteration_matches_oracle(tmp_path, saving):
    from wavefunctionsimpython_gb300 import config_read_helper, core_sim
    from wavefunctionsimpython_gb300.iter_data import IterData
    from wavefunctionsimpython_gb300.measurement import MeasurementTools
    from wavefunctionsimpython_gb300.sim_state import SimState

    config_read_helper.QUIET = True
    cfg = base_config(tmp_path, saving=saving)
    s = SimState(copy.deepcopy(cfg))
    s.set_use_cache(False)
    s.initialize_state()
    mt = MeasurementTools(copy.deepcopy(cfg), s)
    it = IterData(cfg)
    dx, V, psi = oracle_run(cfg, s)
    np.testing.assert_allclose(s.engine.get_potential(), V, rtol=1e-5, atol=1e-4)
    core_sim.run_iteration(s, mt, it)
    mt.finish(s)
    vols = mt.active_volume_probabilities()
    loc = mt.expected_location()
    dt = cfg["simulation"]["delta_time_h_bar_per_hartree"]
    for i in range(cfg["simulation"]["total_iteration_count"]):
        for v in vols:
            ref = orc.volume_probability(psi, dx, *v.box)
            assert abs(v.get_probability_evolution_with_name()[0][i] - ref) < 1e-9
        er, er2 = orc.expected_location(psi, dx, *loc.box)
        np.testing.assert_allclose(loc.get_expected_location_evolution()[i], er, rtol=1e-9, atol=1e-11)
        np.testing.assert_allclose(loc.get_standard_deviation_evolution()[i], np.sqrt(er2 - er ** 2), rtol=1e-7)
        psi = orc.split_step(psi, V, dx, dt, 1.0, nsteps=1)
    assert np.linalg.norm(s.get_wave_function() - psi) / np.linalg.norm(psi) < 1e-11
    out = cfg["paths"]["output_dir"]
    assert os.path.exists(os.path.join(out, "measurable_npy", "volume_probability_evolution_left.npy"))
    assert os.path.exists(os.path.join(out, "measurable_raw", "expected_location_evolution.bin"))
    assert os.path.exists(os.path.join(out, "potential_raw", "potential.bin"))
    if saving:
        wf = np.load(os.path.join(out, "wave_function_npy", "wave_function_000004.npy"))
        assert wf.dtype == np.complex128 and wf.ndim == 3


def test_power_series_method_through_sim_state(tmp_path):
    from wavefunctionsimpython_gb300 import config_read_helper
    from wavefunctionsimpython_gb300.sim_state import SimState

    config_read_helper.QUIET = True
    cfg = base_config(tmp_path, method="power_series", dbl=False)
    cfg["simulation"]["delta_time_h_bar_per_hartree"] = 0.002
    s = SimState(copy.deepcopy(cfg))
    s.set_use_cache(False)
    s.initialize_state()
    dx, V, psi = oracle_run(cfg, s)
    for _ in range(3):
        s.evolve_state()
    ref = orc.taylor_step(psi, V, dx, 0.002, 1.0, order=10, stencil_order=2, nsteps=3)
    assert np.linalg.norm(s.get_wave_function() - ref) / np.linalg.norm(ref) < 1e-5


@pytest.mark.parametrize("method", ["fourier", "power_series"])
def test_checkpoint_resume_is_exact_with_moving_wall(tmp_path, method):
    """A run checkpointed after 5 steps and resumed in a fresh SimState ends bit-identical
    to the uninterrupted run, moving wall and iteration counters included."""
    from wavefunctionsimpython_gb300 import iter_data as idm
    from wavefunctionsimpython_gb300 import sim_state as ssm

    cfg = base_config(tmp_path, method=method, dbl=False)
    cfg["simulation"]["is_dynamic_potential_mode"] = True
    cfg["potential"]["walls"][0]["velocity_bohr_radius_hartree_per_h_bar_3"] = [0.5, 0.0, 0.0]

    def advance(s, it, n):
        for _ in range(n):
            s.evolve_state()
            s.update_potential()
            it.i += 1
            it.total_simulated_time += s.get_delta_time_h_bar_per_hartree()

    a = ssm.SimState(copy.deepcopy(cfg))
    a.set_use_cache(False)
    a.initialize_state()
    ita = idm.IterData(cfg)
    advance(a, ita, 5)
    ckpt = str(tmp_path / "state.npz")
    a.save_checkpoint(ckpt, ita)
    advance(a, ita, 4)
    ref_psi, ref_v = a.get_wave_function(), a.engine.get_potential()

    b = ssm.SimState(copy.deepcopy(cfg))
    b.set_use_cache(False)
    b.initialize_state()
    itb = idm.IterData(cfg)
    b.load_checkpoint(ckpt, itb)
    assert itb.i == 5
    advance(b, itb, 4)
    assert itb.i == ita.i and itb.total_simulated_time == ita.total_simulated_time
    assert np.array_equal(b.engine.get_potential(), ref_v)
    assert np.array_equal(b.get_wave_function(), ref_psi)
    assert np.allclose(b.get_potential_walls()[0].center_bohr_radii_3, a.get_potential_walls()[0].center_bohr_radii_3)

    other = copy.deepcopy(cfg)
    other["volume"]["number_of_voxels_3"] = [32, 32, 32]
    c = ssm.SimState(other)
    c.set_use_cache(False)
    with pytest.raises(ValueError):
        c.load_checkpoint(ckpt)


def test_run_iteration_moving_wall_stays_on_device(tmp_path):
    """Dynamic potential mode with a moving wall: run_iteration keeps the fused device loop
    (the engine advects the wall and rebuilds V after each step) and records the same
    series as the reference's measure / evolve / update_potential loop, restated by the
    oracle with the engine's absorbing ramp (which does not move; the ramp's float32 atan
    and pow round differently on the host by up to two ulps)."""
    from wavefunctionsimpython_gb300 import config_read_helper, core_sim
    from wavefunctionsimpython_gb300.iter_data import IterData
    from wavefunctionsimpython_gb300.measurement import MeasurementTools
    from wavefunctionsimpython_gb300.sim_state import SimState

    config_read_helper.QUIET = True
    cfg = base_config(tmp_path)
    cfg["simulation"]["is_dynamic_potential_mode"] = True
    w = cfg["potential"]["walls"][0]
    w["velocity_bohr_radius_hartree_per_h_bar_3"] = [-0.8, 0.3, 0.0]
    w["slope_exponent"] = 1.0  # a linear slope: the host's float32 pow and the device's powf agree
    s = SimState(copy.deepcopy(cfg))
    s.set_use_cache(False)
    s.initialize_state()
    mt = MeasurementTools(copy.deepcopy(cfg), s)
    it = IterData(cfg)
    assert core_sim._can_fuse(s, mt)
    dx, V, psi = oracle_run(cfg, s)
    ramp = s.engine.get_potential().imag.astype(np.float32)
    wall = orc.Wall(potential_hartree=w["potential_hartree"], center_bohr_radii_3=tuple(w["center_bohr_radii_3"]),
                    normal_vector_3=tuple(w["normal_vector_3"]), plateau_thickness_bohr_radii=w["plateau_thickness_bohr_radii"],
                    slope_thickness_bohr_radii=w["slope_thickness_bohr_radii"], slope_exponent=w["slope_exponent"],
                    slit_count=w["slit_count"], slit_spacing_bohr_radii=w["slit_spacing_bohr_radii"],
                    slit_width_bohr_radii=w["slit_width_bohr_radii"], slit_rotation_radian=w["slit_rotation_radian"])
    walls, vel = [wall], [w["velocity_bohr_radius_hartree_per_h_bar_3"]]
    V = (V.real + 1j * ramp).astype(np.complex64)
    core_sim.run_iteration(s, mt, it)
    dt = cfg["simulation"]["delta_time_h_bar_per_hartree"]
    vols = mt.active_volume_probabilities()
    for i in range(cfg["simulation"]["total_iteration_count"]):
        for v in vols:
            assert abs(v.get_probability_evolution_with_name()[0][i] - orc.volume_probability(psi, dx, *v.box)) < 1e-9
        psi = orc.split_step(psi, V, dx, dt, 1.0, nsteps=1)
        walls = orc.advect_walls(walls, vel, dt)
        V = (orc.rebuild_potential(V.shape, dx, walls, None).real + 1j * ramp).astype(np.complex64)
    assert np.array_equal(s.engine.get_potential(), V)
    np.testing.assert_array_equal(s.get_potential_walls()[0].center_bohr_radii_3, walls[0].center_bohr_radii_3)
    assert np.linalg.norm(s.get_wave_function() - psi) / np.linalg.norm(psi) < 1e-11
