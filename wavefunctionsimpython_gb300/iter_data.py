"""Iteration counters (sources/iter_data.py:5-14)."""
from __future__ import annotations

from typing import Dict

from .config_read_helper import try_read_param


class IterData:
    def __init__(self, config: Dict):
        self.i = 0
        self.elapsed_system_time_s = 0.0
        self.average_iteration_system_time_s = 0.0
        self.total_simulated_time = 0.0
        self.is_quit = False
        self.total_iteration_count = try_read_param(config, "simulation.total_iteration_count", 1000)
