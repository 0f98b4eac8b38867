"""Headless volume view of psi and V (replaces sources/volumetric_visualization.py).

The reference draws psi and V with vispy/OpenGL into a window-less canvas and
saves PNG frames (sources/volumetric_visualization.py:38-270). There is no
graphics stack here; the same emission-absorption shader math runs as a CUDA ray
march (csrc/render.cu, `wfs_render`) into an image buffer, and frames are
written as PNG files with the reference's names and camera motion.
"""
from __future__ import annotations

import os
import struct
import zlib

import numpy as np

from ._lib import Engine, render_desc


def write_png(path, image: np.ndarray):
    """Writes an (H, W, 3) or (H, W, 4) uint8 array as an 8-bit RGB(A) PNG (zlib, no dependencies)."""
    img = np.ascontiguousarray(image, dtype=np.uint8)
    h, w, c = img.shape
    if c not in (3, 4):
        raise ValueError("image must have 3 or 4 channels")
    raw = b"".join(b"\x00" + img[y].tobytes() for y in range(h))

    def chunk(tag, data):
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)

    head = struct.pack(">IIBBBBB", w, h, 8, 6 if c == 4 else 2, 0, 0, 0)
    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", head) + chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b""))


class VolumetricVisualization:
    """sources/volumetric_visualization.py:20-270 without a window: the camera turns by
    cam_rotation_speed and rises by cam_elevation_speed per unit of simulated time,
    and render() returns the (768, 1024, 3) uint8 frame."""

    cam_rotation_speed = 0.0
    cam_elevation_speed = 0.1
    elevation = 45.0

    def __init__(self, engine: Engine, cam_rotation_speed=0.0, azimuth=0.0, width=1024, height=768, shadow_steps=0,
                 light=(1.0, 1.0, -1.0)):
        self.engine = engine
        self.cam_rotation_speed = cam_rotation_speed
        self.azimuth = azimuth
        self.width, self.height = int(width), int(height)
        self.shadow_steps = int(shadow_steps)
        self.light = tuple(light)
        self._az, self._el = float(azimuth), float(self.elevation)

    def update(self, iter_count, delta_time_h_bar_per_hartree):
        """Camera angles for this frame (sources/volumetric_visualization.py:234-241)."""
        t = iter_count * delta_time_h_bar_per_hartree
        self._az = self.azimuth + self.cam_rotation_speed * t
        self._el = self.elevation + self.cam_elevation_speed * t

    def render(self) -> np.ndarray:
        d = render_desc(self.width, self.height, azimuth=self._az, elevation=self._el, light=self.light,
                        shadow_steps=self.shadow_steps)
        return self.engine.render(d)[:, :, :3]

    def render_to_png(self, out_dir, index):
        """sources/volumetric_visualization.py:256-262: probability_density_3D/probability_density_3D_NNNN.png."""
        d = os.path.join(out_dir, "probability_density_3D")
        os.makedirs(d, exist_ok=True)
        write_png(os.path.join(d, f"probability_density_3D_{index:04d}.png"), self.render())
