"""CUDA volume ray march against the NumPy restatement of the reference's shader (GPU only)."""
import copy
import os

import numpy as np
import pytest

from oracle import render_oracle as ro

pytestmark = pytest.mark.gpu


def scene():
    n = (16, 20, 24)
    i, j, k = np.meshgrid(*(np.arange(m) - (m - 1) / 2 for m in n), indexing="ij")
    psi = (0.004 * np.exp(-((i - 1) ** 2 + j ** 2 + (k + 2) ** 2) / 10.0) * np.exp(1j * (0.9 * k + 0.3 * j)))
    V = np.where(np.abs(k - 3) < 1.5, 5.0, 0.0) - 1j * 0.5 * np.maximum(0, np.abs(i) - 5)
    return n, psi.astype(np.complex64), V.astype(np.complex64)


@pytest.mark.parametrize("shadow_steps,azimuth", [(0, 30.0), (6, -60.0)])
def test_render_matches_oracle(shadow_steps, azimuth):
    from wavefunctionsimpython_gb300 import Engine
    from wavefunctionsimpython_gb300._lib import render_desc

    n, psi, V = scene()
    e = Engine(n, (8.0, 10.0, 12.0))
    e.set_psi(psi)
    e.set_potential(V)
    kw = dict(width=48, height=36, azimuth=azimuth, elevation=35.0, relative_step=0.2, shadow_steps=shadow_steps)
    got = e.render(render_desc(float_output=True, **kw))[:, :, :3]
    ref = ro.render(psi, V, **kw)
    diff = np.abs(got - ref).max(axis=2)
    assert np.quantile(diff, 0.99) < 2e-3, np.quantile(diff, 0.99)
    assert diff.max() < 0.05
    assert np.abs(ref - ro.aces(np.ones((1, 3)))[0]).max() > 0.1  # the scene is not empty
    rgba = e.render(render_desc(**kw))
    assert rgba.dtype == np.uint8 and rgba.shape == (36, 48, 4)
    assert np.abs(rgba[:, :, :3].astype(int) - np.round(got * 255).astype(int)).max() <= 1
    assert (rgba[:, :, 3] == 255).all()


def test_measurement_writes_volumetric_frames(tmp_path):
    from test_gpu_dropin import base_config
    from wavefunctionsimpython_gb300 import core_sim, iter_data, measurement, sim_state

    cfg = base_config(tmp_path, dbl=False)
    cfg["simulation"]["total_iteration_count"] = 5
    cfg["measurement"]["volumetric"] = {"enable_image": True, "image_capture_iteration_interval": 2,
                                        "camera_rotation_speed": 10.0}
    s = sim_state.SimState(copy.deepcopy(cfg))
    s.set_use_cache(False)
    s.initialize_state()
    mt = measurement.MeasurementTools(cfg, s)
    it = iter_data.IterData(cfg)
    core_sim.run_iteration(s, mt, it)
    d = os.path.join(cfg["paths"]["output_dir"], "probability_density_3D")
    names = sorted(os.listdir(d))
    assert names == [f"probability_density_3D_{i:04d}.png" for i in (0, 2, 4)]
    with open(os.path.join(d, names[0]), "rb") as f:
        head = f.read(24)
    assert head[:8] == b"\x89PNG\r\n\x1a\n" and head[16:24] == (1024).to_bytes(4, "big") + (768).to_bytes(4, "big")
