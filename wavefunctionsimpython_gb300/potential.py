"""Potential descriptions read from the TOML config (sources/potential.py).

The classes keep the reference's names, keys and defaults; ``add_potential``
builds the contribution on the GPU through the engine (no host loops).
"""
from __future__ import annotations

from typing import Dict

import numpy as np

from . import math_utils
from .config_read_helper import try_read_param

_FLOAT_TYPES = {"float64": np.float64, "float32": np.float32, "complex64": np.complex64, "complex128": np.complex128}


class PreInitializedPotential:
    """sources/potential.py:14-55 — raw potential file added to V."""

    def __init__(self, config: Dict):
        self.path = try_read_param(config, "potential.pre_initialized_potential.path", "")
        self.enable = try_read_param(config, "potential.pre_initialized_potential.enable", False)
        if len(self.path) == 0:
            self.enable = False
        self.visible = try_read_param(config, "potential.pre_initialized_potential.visible", True)
        type_str = try_read_param(config, "potential.pre_initialized_potential.float_type", "float64")
        if type_str not in _FLOAT_TYPES:
            print(f"Unrecognised float type for the pre-initialized potential \"{self.path}\"! "
                  "Available options are: float32, float64, complex64, complex128. Falling back to float64.")
            type_str = "float64"
        self.float_type = _FLOAT_TYPES[type_str]

    def is_enabled(self):
        return self.enable

    def is_visible(self):
        return self.visible

    def load(self, shape):
        return np.fromfile(self.path, dtype=self.float_type).reshape(shape)

    def add_potential(self, engine):
        engine.add_raw_potential(self.load(engine.n))


class AbsorbingBoundaryCondition:
    """sources/potential.py:57-158 — imaginary ramp outside the observation box."""

    def __init__(self, config, bottom_corner, top_corner):
        self.boundary_bottom_corner_bohr_radii_3 = np.asarray(bottom_corner, dtype=np.float64)
        self.boundary_top_corner_bohr_radii_3 = np.asarray(top_corner, dtype=np.float64)
        p = "absorbing_boundary_condition."
        self.outer_potential_in_positive_xyz_direction_hartree_3 = np.array(
            try_read_param(config, p + "outer_potential_in_positive_xyz_direction_hartree_3", [-100.0] * 3))
        self.outer_potential_in_negative_xyz_direction_hartree_3 = np.array(
            try_read_param(config, p + "outer_potential_in_negative_xyz_direction_hartree_3", [-100.0] * 3))
        self.start_offset = try_read_param(config, p + "start_offset", 1.0)
        self.slope_exponent_in_positive_xyz_direction_3 = np.array(
            try_read_param(config, p + "slope_exponent_in_positive_xyz_direction_3", [2.0] * 3))
        self.slope_exponent_in_negative_xyz_direction_3 = np.array(
            try_read_param(config, p + "slope_exponent_in_negative_xyz_direction_3", [2.0] * 3))
        self.enable = try_read_param(config, p + "enable", True)

    def engine_args(self):
        """The seven Engine.add_absorbing arguments."""
        return (self.boundary_bottom_corner_bohr_radii_3, self.boundary_top_corner_bohr_radii_3,
                self.start_offset, self.outer_potential_in_positive_xyz_direction_hartree_3,
                self.outer_potential_in_negative_xyz_direction_hartree_3,
                self.slope_exponent_in_positive_xyz_direction_3, self.slope_exponent_in_negative_xyz_direction_3)

    def add_potential(self, engine):
        if not self.enable:
            return
        engine.add_absorbing(*self.engine_args())


class PotentialWall:
    """sources/potential.py:161-242 — slab with 0-4 slits, plateau and power-law slope."""

    def __init__(self, wall_config: Dict):
        self.potential_hartree = try_read_param(wall_config, "potential_hartree", 20)
        self.center_bohr_radii_3 = np.array(try_read_param(wall_config, "center_bohr_radii_3", [0.0, 0.0, 0.0]), dtype=np.float64)
        self.normal_vector_3 = math_utils.normalize(np.array(try_read_param(wall_config, "normal_vector_3", [1.0, 0.0, 0.0])))
        self.plateau_thickness_bohr_radii = try_read_param(wall_config, "plateau_thickness_bohr_radii", 5.0)
        self.slope_thickness_bohr_radii = try_read_param(wall_config, "slope_thickness_bohr_radii", 0.0)
        self.slope_exponent = try_read_param(wall_config, "slope_exponent", 1.0)
        self.velocity_bohr_radius_hartree_per_h_bar_3 = np.array(
            try_read_param(wall_config, "velocity_bohr_radius_hartree_per_h_bar_3", [0.0, 0.0, 0.0]), dtype=np.float64)
        self.angular_velocity_rad_hartree_per_h_bar_3 = np.array(
            try_read_param(wall_config, "angular_velocity_rad_hartree_per_h_bar_3", [0.0, 0.0, 0.0]), dtype=np.float64)
        self.potential_change_rate_hartree_sqr_per_h_bar = try_read_param(
            wall_config, "potential_change_rate_hartree_sqr_per_h_bar", 0.0)
        self.slit_count = try_read_param(wall_config, "slit_count", 0)
        if self.slit_count > 4:
            print("Potential wall slit count is currently supported only up to 4 slits!")
            self.slit_count = 4
        elif self.slit_count < 0:
            print("Negative potential wall slit count is invalid!")
            self.slit_count = 0
        self.slit_spacing_bohr_radii = try_read_param(wall_config, "slit_spacing_bohr_radii", 1.0)
        self.slit_width_bohr_radii = try_read_param(wall_config, "slit_width_bohr_radii", 0.5)
        self.slit_rotation_radian = try_read_param(wall_config, "slit_rotation_radian", 0.0)
        self.visible = try_read_param(wall_config, "visible", True)
        self.enable = try_read_param(wall_config, "enable", True)

    def is_moving(self):
        return bool(np.any(self.velocity_bohr_radius_hartree_per_h_bar_3 != 0.0))

    def engine_args(self):
        """The ten Engine.add_wall arguments."""
        return (self.potential_hartree, self.center_bohr_radii_3, self.normal_vector_3,
                self.plateau_thickness_bohr_radii, self.slope_thickness_bohr_radii, self.slope_exponent,
                self.slit_count, self.slit_spacing_bohr_radii, self.slit_width_bohr_radii, self.slit_rotation_radian)

    def add_potential(self, engine):
        if not self.enable:
            return
        engine.add_wall(*self.engine_args())


def generate_potential_from_walls_and_drain(engine, absorbing: AbsorbingBoundaryCondition, walls):
    """sources/potential.py:508-522 — V.fill(0), walls, absorbing ramp (on the GPU)."""
    engine.potential_clear()
    for w in walls:
        w.add_potential(engine)
    absorbing.add_potential(engine)
