"""Volume-render oracle and PNG writer checks (CPU only)."""
import struct
import zlib

import numpy as np

from oracle import render_oracle as ro


def test_empty_volume_is_tone_mapped_background():
    img = ro.render(np.zeros((6, 7, 8), np.complex64), None, width=10, height=8)
    bg = ro.aces(np.ones((1, 3)))[0]
    assert np.allclose(img, bg[None, None, :], atol=1e-12)
    assert 0.80 < bg.min() <= bg.max() < 0.81  # the ACES fit maps the white background to light grey


def test_packet_is_visible_and_shadows_darken():
    n = 12
    z, y, x = np.meshgrid(*(np.arange(n) - (n - 1) / 2,) * 3, indexing="ij")
    psi = (0.004 * np.exp(-(x * x + y * y + z * z) / 8.0) * np.exp(1j * 0.8 * x)).astype(np.complex64)
    plain = ro.render(psi, None, width=16, height=12, relative_step=0.25)
    shaded = ro.render(psi, None, width=16, height=12, relative_step=0.25, shadow_steps=4)
    bg = ro.aces(np.ones((1, 3)))[0]
    centre = plain[6, 8]
    assert np.abs(centre - bg).max() > 0.05          # the packet changes the centre pixel
    assert np.allclose(plain[0, 0], bg)               # the corner ray misses the box
    assert shaded.sum() <= plain.sum() + 1e-9        # shadows only remove light


def test_png_writer_round_trip(tmp_path):
    from wavefunctionsimpython_gb300.volumetric_visualization import write_png

    img = (np.arange(5 * 7 * 3) % 256).astype(np.uint8).reshape(5, 7, 3)
    p = tmp_path / "a.png"
    write_png(p, img)
    data = p.read_bytes()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    w, h, depth, ctype = struct.unpack(">IIBB", data[16:26])
    assert (w, h, depth, ctype) == (7, 5, 8, 2)
    idat_len = struct.unpack(">I", data[33:37])[0]
    raw = zlib.decompress(data[41:41 + idat_len])
    rows = [raw[r * (1 + 21) + 1:(r + 1) * (1 + 21)] for r in range(5)]
    assert np.array_equal(np.frombuffer(b"".join(rows), np.uint8).reshape(5, 7, 3), img)
