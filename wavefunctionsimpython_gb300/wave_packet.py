"""Gaussian wave packet parameters (sources/wave_packet.py:63-151)."""
from __future__ import annotations

from typing import Dict

import numpy as np

from . import math_utils
from .config_read_helper import try_read_param


class GaussianWavePacket:
    def __init__(self, config: Dict):
        self.path = try_read_param(config, "wave_packet.path", "")
        self._particle_mass_electron_rest_mass = try_read_param(config, "wave_packet.particle_mass_electron_rest_mass", 1.0)
        self._initial_position_bohr_radii_3 = np.array(
            try_read_param(config, "wave_packet.initial_position_bohr_radii_3", [0.0, 0.0, 0.0]), dtype=np.float64)
        self._initial_wp_velocity_bohr_radii_hartree_per_h_bar_3 = np.array(
            try_read_param(config, "wave_packet.initial_velocity_bohr_radii_hartree_per_h_bar_3", [0.0, 0.0, 0.0]),
            dtype=np.float64)
        # k0 = m v (sources/wave_packet.py:76-79)
        self._initial_momentum_h_per_bohr_radii_3 = math_utils.classical_momentum(
            self._particle_mass_electron_rest_mass, self._initial_wp_velocity_bohr_radii_hartree_per_h_bar_3)
        p = float(np.dot(self._initial_momentum_h_per_bohr_radii_3, self._initial_momentum_h_per_bohr_radii_3) ** 0.5)
        self._de_broglie_wave_length_bohr_radii = math_utils.get_de_broglie_wave_length_bohr_radii(p)
        self.__initial_standard_deviation_bohr_radii_3 = np.array(
            try_read_param(config, "wave_packet.initial_standard_deviation_bohr_radii_3", [5.0, 5.0, 5.0]), dtype=np.float64)

    def get_initial_wp_position_bohr_radii_3(self):
        return self._initial_position_bohr_radii_3

    def get_initial_wp_velocity_bohr_radii_hartree_per_h_bar_3(self):
        return self._initial_wp_velocity_bohr_radii_hartree_per_h_bar_3

    def get_initial_wp_momentum_h_per_bohr_radii_3(self):
        return self._initial_momentum_h_per_bohr_radii_3

    def get_particle_mass_electron_rest_mass(self):
        return self._particle_mass_electron_rest_mass

    def get_de_broglie_wave_length_bohr_radii(self):
        return self._de_broglie_wave_length_bohr_radii

    def get_initial_standard_deviation_bohr_radii(self):
        return self.__initial_standard_deviation_bohr_radii_3

    def init_wave_packet(self, engine, double_precision=False):
        """Fills the engine's psi (sources/wave_packet.py:97-151): a raw file when
        ``wave_packet.path`` is set, else the Gaussian kernel."""
        if len(self.path) > 0:
            arr = np.fromfile(self.path, dtype=np.complex128 if double_precision else np.complex64).reshape(engine.n)
            engine.set_psi(arr)
            return
        engine.init_gaussian(self.__initial_standard_deviation_bohr_radii_3, self._initial_position_bohr_radii_3,
                             self._initial_momentum_h_per_bohr_radii_3)
