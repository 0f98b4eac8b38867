"""Host-side logic vs golden vectors produced by the reference's own Python code
(tests/golden/make_golden.py runs the reference's SimState, MeasurementTools and
math_utils on its shipped TOML configs). CPU only: no engine is created."""
import json
import re
from pathlib import Path

import numpy as np
import pytest

from wavefunctionsimpython_gb300 import config_read_helper, math_utils
from wavefunctionsimpython_gb300.measurement import MeasurementTools
from wavefunctionsimpython_gb300.sim_state import SimState

GOLD = json.loads((Path(__file__).parent / "golden" / "reference_host.json").read_text())
config_read_helper.QUIET = True


def load_cfg(name):
    """The parsed TOML config the fixture was generated from (golden input)."""
    return json.loads(json.dumps(GOLD["configs"][name]["config"]))


@pytest.mark.parametrize("name", sorted(GOLD["configs"]))
def test_sim_state_matches_reference(name):
    g = GOLD["configs"][name]
    s = SimState(load_cfg(name))
    np.testing.assert_allclose(s.get_delta_x_bohr_radii_3(), g["delta_x"], rtol=0, atol=0)
    assert s.get_simulation_method().name == g["method"]
    assert s.is_double_precision() == g["double_precision"]
    np.testing.assert_array_equal(s.get_observation_box_bottom_corner_bohr_radii_3(), g["obs_bottom_bohr"])
    np.testing.assert_array_equal(s.get_observation_box_top_corner_bohr_radii_3(), g["obs_top_bohr"])
    np.testing.assert_array_equal(s.get_observation_box_bottom_corner_voxel_3(), g["obs_bottom_voxel"])
    np.testing.assert_array_equal(s.get_observation_box_top_corner_voxel_3(), g["obs_top_voxel"])
    walls = s.get_potential_walls()
    assert len(walls) == len(g["walls"])
    for w, gw in zip(walls, g["walls"]):
        np.testing.assert_allclose(w.normal_vector_3, gw["normal"], rtol=0, atol=0)
        assert w.slit_count == gw["slit_count"] and w.enable == gw["enable"]


@pytest.mark.parametrize("name", sorted(GOLD["configs"]))
def test_measurement_boxes_match_reference(name):
    g = GOLD["configs"][name]
    s = SimState(load_cfg(name))
    mt = MeasurementTools(load_cfg(name), s)
    # ExpectedLocation mutates SimState's top voxel in the reference; kept
    np.testing.assert_array_equal(s.get_observation_box_top_corner_voxel_3(), g["obs_top_voxel_after_measurement_init"])
    n = s.get_number_of_voxels_3()
    vols = [v for v in mt._MeasurementTools__volume_probabilities]
    assert len(vols) == len(g["volume_probabilities"])
    templates = [t for t in g["kernel_templates"] if t.startswith("volume_probability_kernel")]
    for v, gv, tmpl in zip(vols, g["volume_probabilities"], templates):
        assert v.get_name() == gv["name"]
        cnt = [int(x) for x in re.findall(r"-?\d+", tmpl)[:3]]
        assert cnt == gv["sample_count"]
        b, c = v.box
        bv = np.array(gv["bottom_voxel"])
        # same box unless the reference's box runs past the grid (it reads out of bounds there)
        if np.all(bv + np.array(cnt) <= n):
            np.testing.assert_array_equal(b, bv)
            np.testing.assert_array_equal(c, cnt)
    loc = [t for t in g["kernel_templates"] if t.startswith("expected_location_kernel")]
    if loc:
        cnt = [int(x) for x in re.findall(r"-?\d+", loc[0])[:3]]
        np.testing.assert_array_equal(mt.expected_location().box[1], cnt)
    planes = [t for t in g["kernel_templates"] if t.startswith("probability_current_density_kernel")]
    for p, tmpl in zip(mt.active_plane_currents(), planes):
        cnt = [int(x) for x in re.findall(r"-?\d+", tmpl)[:2]]
        np.testing.assert_array_equal(p.sample_count, cnt)


def test_math_utils_match_reference():
    g = GOLD["math_utils"]
    for k, d in g["indefinite_simpson_integral"].items():
        got = math_utils.indefinite_simpson_integral(np.array(d["input"]), 0.05)
        np.testing.assert_allclose(got, d["integral"], rtol=1e-14, atol=1e-15)
    np.testing.assert_allclose(math_utils.predict_free_space_standard_devation(0.01, 2.0, 1.0, 50), g["predict_sigma"], rtol=1e-15)
    np.testing.assert_allclose(math_utils.predict_free_space_expected_location(0.01, -10.0, 2.0, 50), g["predict_x"], rtol=1e-15)
    for k, v in g["nearest_power_of_2"].items():
        assert math_utils.nearest_power_of_2(int(k)) == v


def test_malformed_toml_raises(tmp_path):
    p = tmp_path / "bad.toml"
    p.write_text("[simulation\ndelta = ")
    with pytest.raises(ValueError):
        config_read_helper.load_toml(p)


def test_missing_delta_time_is_required():
    """simulation.delta_time_h_bar_per_hartree is read by direct indexing in the reference."""
    with pytest.raises(KeyError):
        SimState({"simulation": {}})


def test_try_read_param_default():
    assert config_read_helper.try_read_param({"a": {"b": 3}}, "a.b", 1) == 3
    assert config_read_helper.try_read_param({"a": {}}, "a.c.d", 7) == 7
