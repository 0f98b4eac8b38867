"""Generates tests/golden/reference_host.json from the reference's own Python code.

Run in a container that has the reference checked out (path given as the
first argument). The reference's host-side logic (config parsing,
observation box, Simpson sample boxes, time-series helpers) is imported and
executed as is; only third-party modules that are absent here and unused by
that logic (cupy's kernels, numba, colorama, vispy, matplotlib, imageio) are
replaced by inert stand-ins, with cupy's array helpers mapped to numpy.
RawModule stand-ins record the kernel template names, which carry the
reference's sample counts (sources/measurement.py:124, :341).

    python tests/golden/make_golden.py /path/to/WaveFunctionSimPython
"""
from __future__ import annotations

import json
import os
import sys
import tomllib
import types
from pathlib import Path

import numpy as np

OUT = Path(__file__).resolve().parent / "reference_host.json"
CONFIGS = ["nicer_parameters.toml", "abc_test.toml", "WS_comparison.toml", "lightweight_for_RL.toml",
           "loaded_potential.toml"]


def install_stand_ins(captured):
    class _Any:
        def __init__(self, *a, **k):
            pass

        def __call__(self, *a, **k):
            return _Any()

        def __getattr__(self, name):
            return _Any()

    cp = types.ModuleType("cupy")
    for name in ["zeros", "array", "asarray", "float32", "float64", "complex64", "complex128", "pi", "dot",
                 "linspace", "meshgrid", "stack", "square", "abs", "real", "sqrt", "int32", "uint32"]:
        setattr(cp, name, getattr(np, name))
    cp.ndarray = np.ndarray
    cp.dtype = np.dtype
    cp.asnumpy = np.asarray
    cp.fft = np.fft

    class RawModule:
        def __init__(self, code=None, name_expressions=(), **k):
            captured.extend(name_expressions)

        def get_function(self, name):
            return _Any()

    cp.RawModule = RawModule
    cp.RawKernel = _Any
    cuda = types.ModuleType("cupy.cuda")
    cuda.Stream = _Any
    cp.cuda = cuda
    sys.modules["cupy"] = cp
    sys.modules["cupy.cuda"] = cuda

    numba = types.ModuleType("numba")
    numba.jit = lambda *a, **k: (a[0] if a and callable(a[0]) else (lambda f: f))
    numba.njit = numba.jit
    numba.vectorize = numba.jit
    numba.types = _Any()
    exp = types.ModuleType("numba.experimental")
    exp.jitclass = numba.jit
    numba.experimental = exp
    sys.modules["numba"] = numba
    sys.modules["numba.experimental"] = exp

    col = types.ModuleType("colorama")
    col.Fore = types.SimpleNamespace(RED="", GREEN="", BLUE="")
    col.Style = types.SimpleNamespace(RESET_ALL="")
    col.Back = types.SimpleNamespace()
    sys.modules["colorama"] = col
    for mod in ["sources.volumetric_visualization", "sources.animation", "sources.plot"]:
        m = types.ModuleType(mod)
        m.VolumetricVisualization = _Any
        m.AnimationWriter = _Any
        sys.modules[mod] = m
    # numpy 1.x aliases the reference's annotations use (removed in numpy 2)
    np.complex_ = np.complex128
    np.float_ = np.float64
    spt = types.ModuleType("scipy.spatial.transform")
    spt.Rotation = _Any
    sys.modules.setdefault("scipy.spatial.transform", spt)


def tolist(x):
    return np.asarray(x).tolist()


def main(ref_root):
    ref_root = os.path.abspath(ref_root)
    captured = []
    install_stand_ins(captured)
    os.chdir(ref_root)
    sys.path.insert(0, ref_root)
    from sources import math_utils, measurement, sim_state

    out = {"configs": {}, "math_utils": {}}
    for name in CONFIGS:
        with open(os.path.join("config", name), "rb") as f:
            config = tomllib.load(f)
        # the reference keeps walls and measurement lists at class level; reset per config
        sim_state.SimState._SimState__potential_walls = []
        measurement.MeasurementTools._MeasurementTools__volume_probabilities = []
        measurement.MeasurementTools._MeasurementTools__plane_probability_currents = []
        captured.clear()
        s = sim_state.SimState(config)
        rec = {
            "config": config,
            "delta_x": tolist(s.get_delta_x_bohr_radii_3()),
            "method": s.get_simulation_method().name,
            "double_precision": bool(s.is_double_precision()),
            "obs_bottom_bohr": tolist(s.get_observation_box_bottom_corner_bohr_radii_3()),
            "obs_top_bohr": tolist(s.get_observation_box_top_corner_bohr_radii_3()),
            "obs_bottom_voxel": tolist(s.get_observation_box_bottom_corner_voxel_3()),
            "obs_top_voxel": tolist(s.get_observation_box_top_corner_voxel_3()),
            "mass": float(s.get_particle_mass()),
            "walls": [],
        }
        for w in s._SimState__potential_walls:
            rec["walls"].append({"normal": tolist(w.normal_vector_3), "center": tolist(w.center_bohr_radii_3),
                                 "potential": float(w.potential_hartree), "slit_count": int(w.slit_count),
                                 "enable": bool(w.enable)})
        # psi placeholder (zero-memory view) for the wave-function-saving banner of MeasurementTools
        s._SimState__wave_tensor = np.broadcast_to(np.zeros(1, np.complex64), tuple(s.get_number_of_voxels_3()))
        mt = measurement.MeasurementTools(config, s)
        rec["obs_top_voxel_after_measurement_init"] = tolist(s.get_observation_box_top_corner_voxel_3())
        vols = []
        for v in mt._MeasurementTools__volume_probabilities:
            vols.append({"name": v.get_name(), "bottom_voxel": tolist(v._VolumeProbability__bottom_voxel),
                         "sample_count": tolist(v._VolumeProbability__sample_count),
                         "enable": bool(v.is_enable_image())})
        rec["volume_probabilities"] = vols
        rec["kernel_templates"] = list(captured)
        out["configs"][name] = rec
    rng = np.random.default_rng(7)
    series = {}
    for n in [0, 1, 2, 3, 4, 5, 6, 7, 20, 21]:
        a = rng.standard_normal(n)
        series[str(n)] = {"input": a.tolist(), "integral": tolist(math_utils.indefinite_simpson_integral(a, 0.05))}
    out["math_utils"]["indefinite_simpson_integral"] = series
    out["math_utils"]["predict_sigma"] = tolist(math_utils.predict_free_space_standard_devation(0.01, 2.0, 1.0, 50))
    out["math_utils"]["predict_x"] = tolist(math_utils.predict_free_space_expected_location(0.01, -10.0, 2.0, 50))
    out["math_utils"]["nearest_power_of_2"] = {str(k): math_utils.nearest_power_of_2(k) for k in [1, 3, 5, 31, 33, 255, 257]}
    OUT.write_text(json.dumps(out, indent=1))
    print(f"wrote {OUT}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py REFERENCE_ROOT  (the reference project's checkout)")
    main(sys.argv[1])
