"""SimState — drop-in for sources/sim_state.py on the GB300 engine.

Same constructor (a parsed TOML dict), same method names and return meaning.
Device arrays are owned by the engine handle; ``get_wave_function`` returns a
host copy of psi (the reference returns a CuPy array) and
``get_wave_function_device`` a zero-copy view exposing
``__cuda_array_interface__``.
"""
from __future__ import annotations

import io
import os
from enum import Enum
from typing import Dict

import numpy as np

from . import math_utils, potential, wave_packet
from ._lib import Engine
from .config_read_helper import try_read_param


class SimulationMethod(Enum):
    FOURIER = 0
    POWER_SERIES = 1


class DevicePsi:
    """Zero-copy view of the engine's real-space psi (valid until the next propagation call)."""

    def __init__(self, engine: Engine):
        self.engine = engine
        self.ptr = engine.psi_device_ptr()
        self.shape = engine.n
        self.dtype = np.dtype(engine.dtype)

    @property
    def __cuda_array_interface__(self):
        return {"shape": self.shape, "typestr": self.dtype.str, "data": (self.ptr, False), "version": 3,
                "strides": None}

    def get(self):
        return self.engine.get_psi()


class SimState:
    def __init__(self, config: Dict):
        self.config = config
        self.__cache_dir = try_read_param(config, "paths.cache_dir", "./cache")
        self.__output_dir = try_read_param(config, "paths.output_dir", "./output")
        # method selection (sources/sim_state.py:69-77): "fdtd" maps to the power series
        method_name = str(try_read_param(config, "simulation.method", "fourier")).lower()
        if method_name not in ["fft", "fourier", "fdtd", "power_series"]:
            self.__simulation_method = SimulationMethod.FOURIER
        else:
            self.__simulation_method = (SimulationMethod.FOURIER if method_name in ["fft", "fourier"]
                                        else SimulationMethod.POWER_SERIES)
        self.__order_of_approximation = try_read_param(config, "simulation.order_of_approximation", 10)
        self.__is_dynamic_potential_mode = try_read_param(config, "simulation.is_dynamic_potential_mode", True)
        self.__enable_wave_function_saving = try_read_param(config, "simulation.enable_wave_function_saving", False)
        self.__wave_function_save_iteration_interval = try_read_param(
            config, "simulation.wave_function_save_iteration_interval", 1)
        self.__double_precision = try_read_param(config, "simulation.double_precision_calculation", False)
        # GB300-specific knobs live in their own table so reference configs load unchanged
        self.__stencil_order = int(try_read_param(config, "gb300.laplacian_stencil_order", 2)) if "gb300" in config else 2
        self.__device = int(config.get("gb300", {}).get("device", 0))

        self.__wave_packet = wave_packet.GaussianWavePacket(config)
        self.__simulated_volume_dimensions_bohr_radii_3 = np.array(
            try_read_param(config, "volume.simulated_volume_dimensions_bohr_radii_3", [100.0, 100.0, 100.0]), dtype=np.float64)
        self.__number_of_voxels_3 = np.array(try_read_param(config, "volume.number_of_voxels_3", [256, 256, 256]))
        self.__delta_x_bohr_radii_3 = self.__simulated_volume_dimensions_bohr_radii_3 / self.__number_of_voxels_3
        self.__upper_limit_on_delta_time_h_per_hartree = (
            4.0 / np.pi * (3.0 * np.max(self.__delta_x_bohr_radii_3) * np.max(self.__delta_x_bohr_radii_3)) / 3.0)
        self.__delta_time_h_bar_per_hartree = config["simulation"]["delta_time_h_bar_per_hartree"]

        # observation box (sources/sim_state.py:105-161)
        L = self.__simulated_volume_dimensions_bohr_radii_3
        b = np.array(try_read_param(config, "volume.observation_box_bottom_corner_bohr_radii_3", [-25.0] * 3), dtype=np.float64)
        t = np.array(try_read_param(config, "volume.observation_box_top_corner_bohr_radii_3", [25.0] * 3), dtype=np.float64)
        for i in range(3):
            if b[i] > t[i]:
                b[i], t[i] = t[i], b[i]
        for i in range(3):
            if b[i] < -L[i] * 0.5:
                b[i] = -L[i] * 0.5
            if t[i] > L[i] * 0.5:
                t[i] = L[i] * 0.5
        self.__observation_box_bottom_corner_bohr_radii_3 = b
        self.__observation_box_top_corner_bohr_radii_3 = t
        self.__observation_box_bottom_corner_voxel_3 = np.array(
            math_utils.transform_center_origin_to_corner_origin_system(b, L) / self.__delta_x_bohr_radii_3, dtype=np.int32)
        self.__observation_box_top_corner_voxel_3 = np.array(
            math_utils.transform_center_origin_to_corner_origin_system(t, L) / self.__delta_x_bohr_radii_3, dtype=np.int32)
        for i in range(3):
            if self.__observation_box_top_corner_voxel_3[i] >= self.__number_of_voxels_3[i]:
                self.__observation_box_top_corner_voxel_3[i] = self.__number_of_voxels_3[i] - 1
        for i in range(3):
            if self.__observation_box_bottom_corner_voxel_3[i] < 0:
                self.__observation_box_bottom_corner_voxel_3[i] = 0
        self.__observation_box_dimensions_bohr_radii_3 = t - b
        self.__observation_box_dimensions_voxel_3 = (self.__observation_box_top_corner_voxel_3
                                                     - self.__observation_box_bottom_corner_voxel_3)

        self.__pre_initialized_potential = potential.PreInitializedPotential(config)
        if self.__pre_initialized_potential.is_enabled():
            self.__is_dynamic_potential_mode = False
        self.__absorbing_boundary_condition = potential.AbsorbingBoundaryCondition(config, b, t)
        # per-instance wall list (the reference shares a class-level list between instances)
        self.__potential_walls = [potential.PotentialWall(w) for w in try_read_param(config, "potential.walls", [])]
        self.__use_cache = True
        self.__engine_dynamic_walls = False
        self.engine: Engine | None = None

    # ------------------------------------------------------------------ init
    def _make_engine(self):
        if self.engine is None:
            self.engine = Engine(tuple(int(x) for x in self.__number_of_voxels_3),
                                 tuple(float(x) for x in self.__simulated_volume_dimensions_bohr_radii_3),
                                 double_precision=self.__double_precision, device=self.__device)
        return self.engine

    def initialize_state(self):
        """sources/sim_state.py:185-300: psi0 (cache, raw file or Gaussian), V (cache or
        pre-initialised file + absorbing ramp + walls), potential.bin output."""
        eng = self._make_engine()
        full_init = True
        if self.__use_cache:
            try:
                eng.set_psi(np.load(os.path.join(self.__cache_dir, "gaussian_wave_packet.npy")))
                full_init = False
            except (OSError, ValueError):
                pass
        if full_init:
            self.__wave_packet.init_wave_packet(eng, self.__double_precision)
            self._try_save(os.path.join(self.__cache_dir, "gaussian_wave_packet.npy"), eng.get_psi)
        full_init = True
        if self.__use_cache:
            try:
                eng.set_potential(np.load(os.path.join(self.__cache_dir, "localized_potential.npy")))
                full_init = False
            except (OSError, ValueError):
                pass
        if full_init:
            eng.potential_clear()
            if self.__pre_initialized_potential.is_enabled():
                self.__pre_initialized_potential.add_potential(eng)
            self.__absorbing_boundary_condition.add_potential(eng)
            for wall in self.__potential_walls:
                wall.add_potential(eng)
            self._try_save(os.path.join(self.__cache_dir, "localized_potential.npy"), eng.get_potential)
        try:
            os.makedirs(os.path.join(self.__output_dir, "potential_raw"), exist_ok=True)
            eng.get_potential().view(np.float32).astype(np.float32).tofile(
                os.path.join(self.__output_dir, "potential_raw", "potential.bin"))
        except OSError as e:
            print(f"Failed writing potential.bin: {e}")
        self._register_dynamic_walls()

    @staticmethod
    def _try_save(path, getter):
        try:
            os.makedirs(os.path.dirname(path), exist_ok=True)
            np.save(path, getter())
        except OSError as e:
            print(f"Failed writing cache file {path}: {e}")

    # ------------------------------------------------------------- getters
    def get_delta_time_h_bar_per_hartree(self):
        return self.__delta_time_h_bar_per_hartree

    def get_delta_x_bohr_radii_3(self):
        return self.__delta_x_bohr_radii_3

    def set_wave_function(self, wave_func):
        self._make_engine().set_psi(wave_func)

    def get_wave_function(self):
        return self.engine.get_psi()

    def get_wave_function_device(self) -> DevicePsi:
        return DevicePsi(self.engine)

    def is_wave_function_saving(self):
        return self.__enable_wave_function_saving

    def get_wave_function_save_interval(self):
        return self.__wave_function_save_iteration_interval

    def get_simulation_method(self):
        return self.__simulation_method

    def is_use_cache(self):
        return self.__use_cache

    def set_use_cache(self, uc: bool):
        self.__use_cache = uc

    def get_cache_dir(self):
        return self.__cache_dir

    def get_output_dir(self):
        return self.__output_dir

    def get_number_of_voxels_3(self):
        return self.__number_of_voxels_3

    def get_observation_box_bottom_corner_voxel_3(self):
        return self.__observation_box_bottom_corner_voxel_3

    def get_observation_box_top_corner_voxel_3(self):
        return self.__observation_box_top_corner_voxel_3

    def get_observation_box_bottom_corner_bohr_radii_3(self):
        return self.__observation_box_bottom_corner_bohr_radii_3

    def get_observation_box_top_corner_bohr_radii_3(self):
        return self.__observation_box_top_corner_bohr_radii_3

    def get_simulated_volume_dimensions_bohr_radii_3(self):
        return self.__simulated_volume_dimensions_bohr_radii_3

    def is_double_precision(self) -> bool:
        return self.__double_precision

    def is_dynamic_potential_mode(self) -> bool:
        return self.__is_dynamic_potential_mode

    def get_order_of_approximation(self):
        return self.__order_of_approximation

    def get_laplacian_stencil_order(self):
        return self.__stencil_order

    def get_potential_walls(self):
        return self.__potential_walls

    def get_absorbing_boundary_condition(self):
        return self.__absorbing_boundary_condition

    def get_wave_packet(self):
        return self.__wave_packet

    def transform_physical_coordinate_to_voxel_3(self, pos_bohr_radii_3):
        return (math_utils.transform_center_origin_to_corner_origin_system(
            pos_bohr_radii_3, self.__simulated_volume_dimensions_bohr_radii_3) / self.__delta_x_bohr_radii_3).astype(np.uint)

    def transform_voxel_to_physical_coordinate_3(self, voxel_3):
        return math_utils.transform_corner_origin_to_center_origin_system(
            voxel_3, self.__number_of_voxels_3) * self.__delta_x_bohr_radii_3

    def get_view_into_wave_function(self):
        return math_utils.cut_bounding_box(self.get_wave_function(), self.__observation_box_bottom_corner_voxel_3,
                                           self.__observation_box_top_corner_voxel_3)

    def get_view_into_probability_density(self):
        psi = self.get_view_into_wave_function()
        return (psi.real.astype(np.float64) ** 2 + psi.imag.astype(np.float64) ** 2)

    def get_view_into_potential(self):
        return math_utils.cut_bounding_box(np.real(self.engine.get_potential()), self.__observation_box_bottom_corner_voxel_3,
                                           self.__observation_box_top_corner_voxel_3)

    def get_view_into_complex_potential(self):
        return math_utils.cut_bounding_box(self.engine.get_potential(), self.__observation_box_bottom_corner_voxel_3,
                                           self.__observation_box_top_corner_voxel_3)

    def get_particle_mass(self):
        return self.__wave_packet.get_particle_mass_electron_rest_mass()

    def get_dxdydz(self):
        return float(np.prod(self.__delta_x_bohr_radii_3))

    # ---------------------------------------------------------- evolution
    def _enabled_walls(self):
        return [w for w in self.__potential_walls if w.enable]

    def _register_dynamic_walls(self):
        """Dynamic potential mode (sources/sim_state.py:466-509): the engine is given the
        enabled walls with their velocities and the absorbing ramp, and after every step it
        advects the walls (x clamped at 0) and rebuilds V on the device, so stepping never
        returns to the host for it. Without a moving wall the rebuild would reproduce V
        unchanged (no pre-initialised potential exists in this mode), so nothing is set."""
        self.__engine_dynamic_walls = False
        if self.engine is None or not self.has_moving_potential():
            return
        walls = self._enabled_walls()
        ab = self.__absorbing_boundary_condition
        self.engine.set_dynamic_walls([w.engine_args() for w in walls],
                                      [w.velocity_bohr_radius_hartree_per_h_bar_3 for w in walls],
                                      ab.engine_args() if ab.enable else None)
        self.__engine_dynamic_walls = True

    def sync_dynamic_walls(self):
        """Copies the engine's current wall centres back into the wall objects."""
        if self.__engine_dynamic_walls:
            for w, c in zip(self._enabled_walls(), self.engine.get_dynamic_walls()):
                w.center_bohr_radii_3 = np.array(c, dtype=np.float64)

    def update_potential(self):
        """sources/sim_state.py:466-509. In dynamic mode the engine has already advected
        the moving walls and rebuilt V after each step of evolve_state; the walls' new
        centres are read back here."""
        if not self.__is_dynamic_potential_mode:
            return
        self.sync_dynamic_walls()

    def has_moving_potential(self) -> bool:
        return self.__is_dynamic_potential_mode and any(w.enable and w.is_moving() for w in self.__potential_walls)

    def evolve_state(self, nsteps: int = 1):
        """sources/sim_state.py:754-762 — one (or nsteps) step(s) of the configured method."""
        if self.__simulation_method == SimulationMethod.FOURIER:
            self.engine.step_split(nsteps, self.__delta_time_h_bar_per_hartree, self.get_particle_mass())
        else:
            self.engine.step_taylor(nsteps, self.__delta_time_h_bar_per_hartree, self.get_particle_mass(),
                                    self.__order_of_approximation, self.__stencil_order)

    # ---------------------------------------------------------- checkpoint
    CHECKPOINT_VERSION = 1

    def save_checkpoint(self, path, iter_data=None):
        """Writes psi, V, the moving walls and the iteration counters to one .npz file so
        a run resumes exactly where it stopped. The reference has no working psi
        checkpoint (its snapshot writer is commented out, sources/snapshot_io.py:12-16)."""
        eng = self.engine
        self.sync_dynamic_walls()
        walls = np.array([np.concatenate([w.center_bohr_radii_3, w.velocity_bohr_radius_hartree_per_h_bar_3,
                                          [float(w.potential_hartree)]]) for w in self.__potential_walls],
                         dtype=np.float64).reshape(-1, 7)
        it = {} if iter_data is None else {"i": iter_data.i, "total_simulated_time": iter_data.total_simulated_time,
                                          "elapsed_system_time_s": iter_data.elapsed_system_time_s}
        np.savez(path, version=self.CHECKPOINT_VERSION, psi=eng.get_psi(), potential=eng.get_potential(),
                 number_of_voxels_3=np.asarray(self.__number_of_voxels_3, dtype=np.int64),
                 volume_bohr_radii_3=np.asarray(self.__simulated_volume_dimensions_bohr_radii_3, dtype=np.float64),
                 double_precision=self.__double_precision, delta_time=self.__delta_time_h_bar_per_hartree,
                 walls=walls, iteration=np.asarray([it.get("i", 0)], dtype=np.int64),
                 times=np.asarray([it.get("total_simulated_time", 0.0), it.get("elapsed_system_time_s", 0.0)]))

    def load_checkpoint(self, path, iter_data=None):
        """Restores a file written by save_checkpoint: psi and V on the GPU, the walls'
        positions, and (when given) the IterData counters. Raises ValueError when the
        checkpoint's grid, extent, precision or wall count differ from this state's."""
        with np.load(path) as f:
            if int(f["version"]) != self.CHECKPOINT_VERSION:
                raise ValueError(f"unsupported checkpoint version {int(f['version'])}")
            if (tuple(int(x) for x in f["number_of_voxels_3"]) != tuple(int(x) for x in self.__number_of_voxels_3)
                    or not np.allclose(f["volume_bohr_radii_3"], self.__simulated_volume_dimensions_bohr_radii_3)
                    or bool(f["double_precision"]) != bool(self.__double_precision)):
                raise ValueError("checkpoint grid, extent or precision differ from this simulation")
            walls = f["walls"]
            if walls.shape[0] != len(self.__potential_walls):
                raise ValueError("checkpoint wall count differs from this simulation")
            eng = self._make_engine()
            eng.set_psi(f["psi"])
            eng.set_potential(f["potential"])
            for w, row in zip(self.__potential_walls, walls):
                w.center_bohr_radii_3 = row[0:3].copy()
                w.velocity_bohr_radius_hartree_per_h_bar_3 = row[3:6].copy()
                w.potential_hartree = float(row[6])
            self._register_dynamic_walls()
            if iter_data is not None:
                iter_data.i = int(f["iteration"][0])
                iter_data.total_simulated_time = float(f["times"][0])
                iter_data.elapsed_system_time_s = float(f["times"][1])

    def get_simulation_method_text(self, use_colors=False):
        text = io.StringIO()
        if self.__simulation_method == SimulationMethod.FOURIER:
            text.write("Using the Split-Operator Fourier method to simulate the time development.\n")
        else:
            text.write("Using the Power Series method to simulate the time development.\n")
            text.write(f"The order of approximation is p = {self.__order_of_approximation}.\n")
        return text.getvalue()
