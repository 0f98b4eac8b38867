"""Mean energy gain of the split step's transforms from rounded constants (CPU only).

In complex64 the butterflies multiply by roots of unity rounded to float32, and
those rounded roots are not exactly of modulus 1. The engine computes each
transform's mean energy gain from the constants it uses and folds the inverse
into its kinetic tables. These tests restate that model in NumPy and check
wfs_split_step_gain against it, from the plan table the kernels are built
with. The model is: the inner radix roots as the register DFTs apply them, the
two-stage outer twiddle tables, and the rounded scale factors. The effect of
the compensation on a 2000-step run is checked on the GPU.
"""
import ctypes as C
import math
import re
import shutil
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
PLANS = {int(L): (int(P), int(Q)) for L, P, Q in
         re.findall(r"M\((\d+), (\d+), (\d+)\)", (ROOT / "wavefunctionsimpython_gb300/csrc/kernels.h").read_text())}


def norm2(c, s, dt):
    c, s = float(dt(c)), float(dt(s))
    return c * c + s * s


def const_root_norm2(m, n, dt):
    """|w|^2 of exp(2 pi i m / n) rounded to dt (multiples of n/4 are applied exactly)."""
    m %= n
    if m == 0 or 4 * m == n or 2 * m == n or 4 * m == 3 * n:
        return 1.0
    a = 2.0 * math.pi * m / n
    return norm2(math.cos(a), math.sin(a), dt)


def dft_gain(n, dt):
    """Register DFT of length n split as F x M (F = 4, 2 or 3) with twiddles w_n^(j k)."""
    if n <= 2 or n == 4:
        return 1.0
    if n == 3:
        s3 = float(dt(math.sqrt(3.0) / 2.0))
        return (6.0 + 4.0 * s3 * s3) / 9.0
    f = 4 if n % 4 == 0 else (2 if n % 2 == 0 else 3)
    m = n // f
    tw = np.mean([const_root_norm2(j * k, n, dt) for j in range(f) for k in range(m)])
    return dft_gain(m, dt) * tw * dft_gain(f, dt)


def fft_gain(L, dt):
    P, Q = PLANS[L]
    tw = np.mean([norm2(math.cos(-2 * math.pi * ((t * k) % L) / L), math.sin(-2 * math.pi * ((t * k) % L) / L), dt)
                  for t in range(P) for k in range(Q)])
    return dft_gain(Q, dt) * tw * dft_gain(P, dt)


def split_step_gains(n, dt):
    sx, sy, sz = float(dt(1.0 / n[0])), float(dt(1.0 / math.sqrt(n[1]))), float(dt(1.0 / n[2]))
    gx, gy, gz = fft_gain(n[0], dt), fft_gain(n[1], dt), fft_gain(n[2], dt)
    g_x = gx * gx * (n[0] * sx) ** 2
    gys = gy * n[1] * sy * sy
    return g_x, gys * gys * gz * gz * (n[2] * sz) ** 2


@pytest.fixture(scope="module")
def lib():
    if shutil.which("nvcc") is None and not Path("/usr/local/cuda/bin/nvcc").exists():
        pytest.skip("nvcc is not available to build the engine")
    from wavefunctionsimpython_gb300 import _lib, build_ext

    build_ext.build()
    return _lib.load()


def engine_gains(lib, n, dtype):
    gx, gyz = C.c_double(), C.c_double()
    rc = lib.wfs_split_step_gain((C.c_int32 * 3)(*n), dtype, C.byref(gx), C.byref(gyz))
    assert rc == 0
    return gx.value, gyz.value


@pytest.mark.parametrize("n", [(256, 256, 256), (64, 64, 64), (128, 96, 48), (512, 384, 24), (32, 192, 1024)])
def test_complex64_gains_match_restated_model(lib, n):
    gx, gyz = engine_gains(lib, n, 0)
    rx, ryz = split_step_gains(n, np.float32)
    assert abs(gx - rx) < 1e-13 and abs(gyz - ryz) < 1e-13
    assert abs(gx - 1.0) < 1e-6 and abs(gyz - 1.0) < 2e-6
    if all(v & (v - 1) == 0 for v in n):
        # power-of-two lengths have exact scale factors, and their rounded roots shrink the
        # norm; with a factor 3 the rounded 1/sqrt(L) and 1/L can push the gain above 1
        assert gx < 1.0 and gyz < 1.0


def test_256_per_step_loss_is_the_measured_drift(lib):
    """-3.2e-7 of the norm per step at 256^3: over the 2000-step double-slit run that is
    -6.4e-4, against -5.6e-4 measured between the complex64 and complex128 engines."""
    gx, gyz = engine_gains(lib, (256, 256, 256), 0)
    assert gx * gyz - 1.0 == pytest.approx(-3.19e-7, rel=2e-2)


def test_complex128_gains_are_one(lib):
    gx, gyz = engine_gains(lib, (256, 96, 48), 1)
    assert abs(gx - 1.0) < 1e-15 and abs(gyz - 1.0) < 1e-15


def test_unsupported_length_and_dtype_are_rejected(lib):
    gx, gyz = C.c_double(), C.c_double()
    assert lib.wfs_split_step_gain((C.c_int32 * 3)(256, 100, 256), 0, C.byref(gx), C.byref(gyz)) == 5
    assert lib.wfs_split_step_gain((C.c_int32 * 3)(256, 256, 256), 7, C.byref(gx), C.byref(gyz)) == 1
