"""Non-interactive initialisation (sources/initialisation.py:16-124).

``initialize(config_path)`` loads a TOML file, builds SimState (psi0 and V on
the GPU), MeasurementTools and IterData. The cache check against
``cached_parameters.toml`` is kept; the interactive config-selection and
overwrite prompts of the reference are not.
"""
from __future__ import annotations

import os
import tomllib

from .config_read_helper import load_toml
from .iter_data import IterData
from .measurement import MeasurementTools
from .sim_state import SimState


def initialize(config_path, use_cache: bool = True):
    config = load_toml(config_path)
    sim_state = SimState(config)
    cached = os.path.join(sim_state.get_cache_dir(), "cached_parameters.toml")
    if use_cache:
        try:
            with open(cached, "rb") as f:
                if tomllib.load(f) != config:
                    use_cache = False
        except (OSError, tomllib.TOMLDecodeError):
            use_cache = False
    sim_state.set_use_cache(use_cache)
    os.makedirs(sim_state.get_output_dir(), exist_ok=True)
    sim_state.initialize_state()
    measurement_tools = MeasurementTools(config, sim_state)
    iter_data = IterData(config)
    try:
        os.makedirs(sim_state.get_cache_dir(), exist_ok=True)
        with open(config_path, "rb") as src, open(cached, "wb") as dst:
            dst.write(src.read())
    except OSError as e:
        print(f"Error while creating parameter cache: {e}")
    return sim_state, measurement_tools, iter_data
