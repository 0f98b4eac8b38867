"""MeasurementTools — drop-in for sources/measurement.py on the GB300 engine.

Volume probabilities and the expected location are Simpson-weighted FP64
reductions done by the engine in one launch per measurement. The plane
probability current is computed by its own kernel (see ``PlaneProbabilityCurrent``).
Output files keep the reference's names and byte layout
(sources/measurement.py:626-642, :707-843). Plots and the volumetric renderer
are not part of this package.
"""
from __future__ import annotations

import os
from typing import Dict

import numpy as np

from . import math_utils
from .config_read_helper import try_read_param
from .iter_data import IterData
from .sim_state import SimState


def _simpson_box(bottom_voxel, top_voxel_exclusive, n):
    """Odd sample count box (sources/measurement.py:103-116). Boxes are also
    clipped to the grid; the reference reads past the array there."""
    b = np.array(bottom_voxel, dtype=np.int64)
    t = np.array(top_voxel_exclusive, dtype=np.int64)
    cnt = t - b
    for i in range(3):
        b[i] = min(max(b[i], 0), int(n[i]) - 1)
        cnt[i] = min(cnt[i], int(n[i]) - b[i])
        if cnt[i] % 2 == 0:
            cnt[i] -= 1
        cnt[i] = max(cnt[i], 1)
    return b, cnt


class VolumeProbability:
    """sources/measurement.py:65-188."""

    def __init__(self, config: Dict, sim_state: SimState):
        self.__name = try_read_param(config, "name", "Volume probability", "measurement.volume_probabilities")
        b = np.array(try_read_param(config, "bottom_corner_bohr_radii_3", [-10.0] * 3, "measurement.volume_probabilities"), dtype=np.float64)
        t = np.array(try_read_param(config, "top_corner_bohr_radii_3", [10.0] * 3, "measurement.volume_probabilities"), dtype=np.float64)
        for i in range(3):
            if b[i] > t[i]:
                b[i], t[i] = t[i], b[i]
        self.__bottom_corner_bohr_radii_3 = b
        self.__top_corner_bohr_radii_3 = t
        self.__enable_image = try_read_param(config, "enable_image", True, "measurement.volume_probabilities")
        bottom_voxel = sim_state.transform_physical_coordinate_to_voxel_3(b).astype(np.int64)
        top_voxel = sim_state.transform_physical_coordinate_to_voxel_3(t).astype(np.int64) + 1
        self.box = _simpson_box(bottom_voxel, top_voxel, sim_state.get_number_of_voxels_3())
        self.__probability_evolution = np.empty(shape=0, dtype=np.float64)

    def get_name(self):
        return self.__name

    def set_name(self, n):
        self.__name = n

    def is_enable_image(self):
        return self.__enable_image

    def append(self, value):
        self.__probability_evolution = np.append(self.__probability_evolution, value)

    def get_probability_evolution_with_name(self):
        return self.__probability_evolution, self.__name

    def clear(self):
        self.__probability_evolution = np.empty(shape=0, dtype=np.float64)


class ExpectedLocation:
    """sources/measurement.py:305-407: <r> and sigma = sqrt(<r^2> - <r>^2) over the observation box."""

    def __init__(self, config: Dict, sim_state: SimState):
        self.__enable_image = try_read_param(config, "measurement.expected_location.enable_image", False)
        bottom = sim_state.get_observation_box_bottom_corner_voxel_3()
        # The reference adds 1 to SimState's own top-voxel array here (in place) and
        # takes 1 off again per axis with an even count; that mutation is kept.
        top = sim_state.get_observation_box_top_corner_voxel_3()
        top += np.array([1, 1, 1], dtype=top.dtype)
        cnt = top - bottom
        for i in range(3):
            if cnt[i] % 2 == 0:
                cnt[i] -= 1
                top[i] -= 1
        self.box = _simpson_box(bottom, np.array(bottom, dtype=np.int64) + cnt, sim_state.get_number_of_voxels_3())
        self.__expected_location_evolution = np.zeros(shape=(0, 3), dtype=np.float64)
        self.__standard_deviation_evolution = np.zeros(shape=(0, 3), dtype=np.float64)

    def is_enable_image(self):
        return self.__enable_image

    def append(self, er, er2):
        er = np.asarray(er, dtype=np.float64).reshape(1, 3)
        er2 = np.asarray(er2, dtype=np.float64).reshape(1, 3)
        self.__expected_location_evolution = np.concatenate((self.__expected_location_evolution, er), axis=0)
        self.__standard_deviation_evolution = np.concatenate(
            (self.__standard_deviation_evolution, np.sqrt(er2 - np.power(er, 2))), axis=0)

    def get_expected_location_evolution(self):
        return self.__expected_location_evolution

    def get_standard_deviation_evolution(self):
        return self.__standard_deviation_evolution


class PlaneProbabilityCurrent:
    """sources/measurement.py:190-303 — probability flux through a sampled plane."""

    def __init__(self, config: Dict, sim_state: SimState):
        self.__name = try_read_param(config, "name", "Probability current", "measurement.plane_probability_currents")
        self.center = np.array(try_read_param(config, "center_bohr_radii_3", [0.0, 0.0, 0.0]), dtype=np.float64)
        self.normal = math_utils.normalize(np.array(try_read_param(config, "normal_vector_3", [1.0, 0.0, 0.0])))
        self.__enable_image = try_read_param(config, "enable_image", True, "measurement.plane_probability_currents")
        self.size = np.array(try_read_param(config, "size_bohr_radii_2", [60.0, 60.0]), dtype=np.float64)
        cnt = np.array(try_read_param(config, "resolution_2", [512, 512]), dtype=np.int64) + 1
        for i in range(2):
            if cnt[i] % 2 == 0:
                cnt[i] -= 1
        self.sample_count = cnt
        self.__delta_t = sim_state.get_delta_time_h_bar_per_hartree()
        self.__evolution = np.empty(shape=0, dtype=np.float64)

    def get_name(self):
        return self.__name

    def set_name(self, n):
        self.__name = n

    def is_enable_image(self):
        return self.__enable_image

    def append(self, value):
        self.__evolution = np.append(self.__evolution, value)

    def get_probability_current_evolution_with_name(self):
        return self.__evolution, self.__name

    def get_integrated_probability_current_evolution_with_name(self):
        return math_utils.indefinite_simpson_integral(self.__evolution, self.__delta_t), self.__name


class MeasurementTools:
    """sources/measurement.py:482-843."""

    def __init__(self, config: Dict, sim_state: SimState):
        self.__volume_probabilities = []
        self.__plane_probability_currents = []
        self.__expected_location = None
        self.__volumetric_requested = bool(try_read_param(config, "measurement.volumetric.enable_animation", False)
                                           or try_read_param(config, "measurement.volumetric.enable_image", False))
        # sources/measurement.py:521-535: headless frames instead of the vispy canvas (animation not written)
        self.__enable_volumetric_image = bool(try_read_param(config, "measurement.volumetric.enable_image", False))
        self.__volumetric_image_capture_interval = int(
            try_read_param(config, "measurement.volumetric.image_capture_iteration_interval", 100))
        self.__volumetric = None
        if self.__enable_volumetric_image:
            from .volumetric_visualization import VolumetricVisualization

            self.__volumetric = VolumetricVisualization(
                sim_state._make_engine(),
                cam_rotation_speed=try_read_param(config, "measurement.volumetric.camera_rotation_speed", 0.0),
                azimuth=try_read_param(config, "measurement.volumetric.camera_azimuth", 0.0))
        for conf in try_read_param(config, "measurement.volume_probabilities", []):
            v = VolumeProbability(conf, sim_state)
            self._resolve_naming_conflicts(self.__volume_probabilities, v)
            self.__volume_probabilities.append(v)
        for conf in try_read_param(config, "measurement.plane_probability_currents", []):
            p = PlaneProbabilityCurrent(conf, sim_state)
            self._resolve_naming_conflicts(self.__plane_probability_currents, p)
            self.__plane_probability_currents.append(p)
        if try_read_param(config, "measurement.expected_location.enable_image", False):
            self.__expected_location = ExpectedLocation(config, sim_state)

    @staticmethod
    def _resolve_naming_conflicts(lst, new_item):
        """sources/measurement.py:502-518."""
        for item in lst:
            if item.get_name() == new_item.get_name():
                index = 1
                unique = False
                while not unique:
                    unique = True
                    for item2 in lst:
                        if new_item.get_name() + f"_{index}" == item2.get_name():
                            unique = False
                            index += 1
                            break
                new_item.set_name(new_item.get_name() + f"_{index}")
                break

    # ---------------------------------------------------------------
    def active_volume_probabilities(self):
        return [v for v in self.__volume_probabilities if v.is_enable_image()]

    def active_plane_currents(self):
        return [p for p in self.__plane_probability_currents if p.is_enable_image()]

    def expected_location(self):
        return self.__expected_location

    def fusable(self) -> bool:
        """True when every enabled measurement is computed by the fused device loop
        (volume probabilities, the expected location and plane probability currents)."""
        return len(self.active_volume_probabilities()) <= 8 and self.__volumetric is None

    def observation_request(self):
        boxes = [v.box for v in self.active_volume_probabilities()]
        loc = self.__expected_location.box if self.__expected_location is not None else None
        return boxes, loc

    def plane_request(self):
        """(center, normal, size, sample_count) of every enabled plane current."""
        return [(p.center, p.normal, p.size, p.sample_count) for p in self.active_plane_currents()]

    def record_fluxes(self, fluxes):
        for p, f in zip(self.active_plane_currents(), fluxes):
            p.append(float(f))

    def record(self, probs, er=None, er2=None):
        for v, p in zip(self.active_volume_probabilities(), probs):
            v.append(p)
        if self.__expected_location is not None and er is not None:
            self.__expected_location.append(er, er2)

    def write_wave_function_to_file(self, sim_state: SimState, iter_data: IterData):
        """sources/measurement.py:626-642: .npy and raw .bin of the observation-box view."""
        if iter_data.i % sim_state.get_wave_function_save_interval() != 0:
            return
        out = sim_state.get_output_dir()
        os.makedirs(os.path.join(out, "wave_function_npy"), exist_ok=True)
        os.makedirs(os.path.join(out, "wave_function_raw"), exist_ok=True)
        wf = np.ascontiguousarray(sim_state.get_view_into_wave_function())
        np.save(os.path.join(out, "wave_function_npy", f"wave_function_{iter_data.i:06d}.npy"), wf)
        type_str = "float64" if sim_state.is_double_precision() else "float32"
        wf.view(dtype=type_str).astype(type_str).tofile(
            os.path.join(out, "wave_function_raw", f"wave_function_{iter_data.i:06d}.bin"))

    def measure_and_render(self, sim_state: SimState, iter_data: IterData):
        """sources/measurement.py:644-705; volumetric frames are ray-marched on the GPU
        (volumetric_visualization.py), plots are not drawn."""
        if sim_state.is_wave_function_saving():
            self.write_wave_function_to_file(sim_state, iter_data)
        if self.__volumetric is not None and iter_data.i % self.__volumetric_image_capture_interval == 0:
            self.__volumetric.update(iter_data.i, sim_state.get_delta_time_h_bar_per_hartree())
            self.__volumetric.render_to_png(sim_state.get_output_dir(), iter_data.i)
        boxes, loc = self.observation_request()
        if boxes or loc is not None:
            probs, er, er2 = sim_state.engine.observe(boxes, loc)
            self.record(probs, er, er2)
        for p in self.active_plane_currents():
            p.append(sim_state.engine.plane_current(p.center, p.normal, p.size, p.sample_count,
                                                    sim_state.get_particle_mass()))

    def finish(self, sim_state: SimState):
        """sources/measurement.py:707-843: series as .npy and raw .bin; dwell time and
        transfer probability printed. Plot files are not produced."""
        type_str = "float64" if sim_state.is_double_precision() else "float32"
        out = sim_state.get_output_dir()
        f_npy = os.path.join(out, "measurable_npy")
        f_bin = os.path.join(out, "measurable_raw")
        os.makedirs(f_npy, exist_ok=True)
        os.makedirs(f_bin, exist_ok=True)
        dt = sim_state.get_delta_time_h_bar_per_hartree()
        if self.__expected_location is not None:
            e = self.__expected_location.get_expected_location_evolution()
            np.save(os.path.join(f_npy, "expected_location_evolution.npy"), e)
            e.view(dtype=type_str).astype(type_str).tofile(os.path.join(f_bin, "expected_location_evolution.bin"))
            s = self.__expected_location.get_standard_deviation_evolution()
            np.save(os.path.join(f_npy, "standard_deviation_evolution.npy"), s)
            s.view(dtype=type_str).astype(type_str).tofile(os.path.join(f_bin, "standard_deviation_evolution.bin"))
        for v in self.active_volume_probabilities():
            arr, name = v.get_probability_evolution_with_name()
            np.save(os.path.join(f_npy, f"volume_probability_evolution_{name}.npy"), arr)
            arr.view(dtype=type_str).astype(type_str).tofile(os.path.join(f_bin, f"volume_probability_evolution_{name}.bin"))
            dwell = math_utils.indefinite_simpson_integral(arr, dt)
            if dwell.size:
                print(f"Dwell time in {name}: {dwell[-1]:.5f} hbar/Hartree")
        for p in self.active_plane_currents():
            arr, name = p.get_probability_current_evolution_with_name()
            np.save(os.path.join(f_npy, f"probability_current_evolution_{name}.npy"), arr)
            arr.view(dtype=type_str).astype(type_str).tofile(os.path.join(f_bin, f"probability_current_evolution_{name}.bin"))
            iarr, _ = p.get_integrated_probability_current_evolution_with_name()
            np.save(os.path.join(f_npy, f"integrated_probability_current_{name}.npy"), iarr)
            iarr.view(dtype=type_str).astype(type_str).tofile(os.path.join(f_bin, f"integrated_probability_current_{name}.bin"))
            if iarr.size:
                print(f"Transfer probability on {name}: {iarr[-1]:.5f}")
