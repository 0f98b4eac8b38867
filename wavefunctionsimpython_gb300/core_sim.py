"""Driver loop — drop-in for sources/core_sim.py:19-65.

``time_step`` keeps the reference order (measure, evolve, update potential).
``run_iteration`` runs the whole loop on the device when every enabled
measurement is a fused observable (volume probabilities, the expected
location and plane probability currents) and no wave function is saved: the
engine then records the
observables before each step, exactly as the per-step loop would, and in
dynamic potential mode advects the walls and rebuilds V after each step,
without a host round trip per step. Otherwise it steps from Python.
The loop stops between chunks on SIGINT and calls ``finish`` (the reference's
``write_snapshot`` + ``finish`` + exit, sources/core_sim.py:52-55).
"""
from __future__ import annotations

import signal
import time

import numpy as np

from .iter_data import IterData
from .measurement import MeasurementTools
from .sim_state import SimState, SimulationMethod

FUSED_CHUNK = 2000


def time_step(sim_state: SimState, measurement_tools: MeasurementTools, iter_data: IterData):
    measurement_tools.measure_and_render(sim_state, iter_data)
    sim_state.evolve_state()
    sim_state.update_potential()


def _can_fuse(sim_state: SimState, mt: MeasurementTools) -> bool:
    return (sim_state.get_simulation_method() == SimulationMethod.FOURIER and mt.fusable()
            and not sim_state.is_wave_function_saving())


def run_iteration(sim_state: SimState, measurement_tools: MeasurementTools, iter_data: IterData,
                  observation_interval: int = 1):
    """Runs total_iteration_count steps. ``observation_interval`` > 1 records the
    observables every k-th step only (a GB300-specific option; 1 is the reference)."""
    iter_data.is_quit = False
    prev = signal.getsignal(signal.SIGINT)

    def _quit(signum, frame):
        iter_data.is_quit = True

    try:
        signal.signal(signal.SIGINT, _quit)
    except ValueError:  # not the main thread
        prev = None
    try:
        start = iter_data.i
        total = int(iter_data.total_iteration_count)
        if _can_fuse(sim_state, measurement_tools):
            boxes, loc = measurement_tools.observation_request()
            planes = measurement_tools.plane_request()
            dt = sim_state.get_delta_time_h_bar_per_hartree()
            m = sim_state.get_particle_mass()
            i = start
            while i < total and not iter_data.is_quit:
                n = min(FUSED_CHUNK - FUSED_CHUNK % observation_interval if FUSED_CHUNK >= observation_interval
                        else observation_interval, total - i)
                t0 = time.time()
                if planes:
                    probs, locs, fluxes = sim_state.engine.run_split_planes(n, dt, m, observation_interval, boxes,
                                                                            loc, planes)
                else:
                    probs, locs = sim_state.engine.run_split(n, dt, m, observation_interval, boxes, loc)
                    fluxes = None
                sim_state.engine.synchronize()
                iter_data.elapsed_system_time_s += time.time() - t0
                for k in range(probs.shape[0] if (boxes or loc is not None or planes) else 0):
                    er = locs[k, :3] if loc is not None else None
                    er2 = locs[k, 3:] if loc is not None else None
                    measurement_tools.record(probs[k] if boxes else [], er, er2)
                    if fluxes is not None:
                        measurement_tools.record_fluxes(fluxes[k])
                sim_state.sync_dynamic_walls()
                i += n
                iter_data.i = i
        else:
            for iter_data.i in range(start, total):
                t0 = time.time()
                if iter_data.i % observation_interval == 0:
                    measurement_tools.measure_and_render(sim_state, iter_data)
                sim_state.evolve_state()
                sim_state.update_potential()
                iter_data.elapsed_system_time_s += time.time() - t0
                if iter_data.is_quit:
                    break
            else:
                iter_data.i = total
        if iter_data.is_quit:
            measurement_tools.finish(sim_state)
        iter_data.total_simulated_time = sim_state.get_delta_time_h_bar_per_hartree() * total
        iter_data.average_iteration_system_time_s = iter_data.elapsed_system_time_s / float(max(total, 1))
    finally:
        if prev is not None:
            signal.signal(signal.SIGINT, prev)
    return sim_state, measurement_tools, iter_data
