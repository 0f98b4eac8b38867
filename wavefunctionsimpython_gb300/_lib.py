"""ctypes binding of the engine's C ABI (``include/wfs.h``).

The library ``_wfs.so`` is built in-tree by ``build_ext.build()``. There is no
fallback: if the library is missing or cannot be loaded, importing the engine
raises, so a missing CUDA extension can never be mistaken for a working path.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_wfs.so"

WFS_OK = 0
WFS_ERR_ARG = 1
WFS_ERR_CUDA = 2
WFS_ERR_TIMEOUT = 3
WFS_ERR_NONFINITE = 4
WFS_ERR_UNSUPPORTED = 5
WFS_ERR_STATE = 6
WFS_C64 = 0
WFS_C128 = 1
RAW_TYPES = {"float32": 0, "float64": 1, "complex64": 2, "complex128": 3}
MAX_BOX = 8

# Every entry point include/wfs.h declares (checked by the CPU test suite).
EXPORTED = [
    "wfs_abi_version", "wfs_global_error", "wfs_create", "wfs_destroy", "wfs_last_error", "wfs_synchronize",
    "wfs_set_copy_wait_limit",
    "wfs_potential_clear", "wfs_potential_add_wall", "wfs_potential_add_absorbing", "wfs_potential_add_raw",
    "wfs_set_potential", "wfs_get_potential", "wfs_set_dynamic_walls", "wfs_get_dynamic_walls", "wfs_init_gaussian", "wfs_set_psi", "wfs_get_psi",
    "wfs_psi_device_ptr", "wfs_step_split", "wfs_step_taylor", "wfs_kinetic_operator", "wfs_potential_operator",
    "wfs_observe", "wfs_run_split", "wfs_run_split_planes", "wfs_norm", "wfs_profile_enable", "wfs_profile_read", "wfs_launch_count",
    "wfs_set_schedule", "wfs_split_step_gain",
    "wfs_batch_create", "wfs_batch_destroy", "wfs_batch_last_error", "wfs_batch_synchronize",
    "wfs_batch_init_gaussian", "wfs_batch_add_wall", "wfs_batch_add_absorbing", "wfs_batch_set_potential",
    "wfs_batch_set_psi", "wfs_batch_get_psi", "wfs_batch_run", "wfs_batch_observe", "wfs_batch_set_config",
    "wfs_batch_autotune", "wfs_batch_launch_count", "wfs_observe_noalloc", "wfs_plane_current",
    "wfs_render", "wfs_render_volume",
]
# Every entry point include/wfs_fno.h declares (the surrogate's kernels).
FNO_EXPORTED = [
    "wfs_fno_pointwise", "wfs_fno_pointwise_backward", "wfs_fno_wgrad_scratch", "wfs_fno_weight_grad",
    "wfs_fno_fft3", "wfs_fno_gather", "wfs_fno_scatter", "wfs_fno_pack_weights", "wfs_fno_mix",
    "wfs_fno_spectral_weight_grad", "wfs_fno_adam", "wfs_fno_loss", "wfs_fno_sample_norms",
    "wfs_fno_make_input", "wfs_fno_scale_samples", "wfs_fno_fast_lift", "wfs_fno_fast_layer",
    "wfs_fno_fast_last", "wfs_fno_fast_xmix", "wfs_fno_pack_mix_interleaved",
    "wfs_fno_to_bf16", "wfs_fno_set_wait_limit",
]
SCHEDULES = {"auto": 0, "axis": 1, "plane": 2}
NPASS = 8
PASS_NAMES = ["x_kin", "y", "z_vph", "z", "observe", "taylor", "other", "plane"]


class WfsError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"wfs error {code}: {msg}")
        self.code = code


class GridDesc(C.Structure):
    _fields_ = [("n", C.c_int32 * 3), ("extent", C.c_double * 3), ("dtype", C.c_int32),
                ("device", C.c_int32), ("stream", C.c_void_p)]


class WallDesc(C.Structure):
    _fields_ = [("potential_hartree", C.c_double), ("center", C.c_double * 3), ("normal", C.c_double * 3),
                ("plateau_thickness", C.c_double), ("slope_thickness", C.c_double), ("slope_exponent", C.c_double),
                ("slit_count", C.c_int32), ("slit_spacing", C.c_double), ("slit_width", C.c_double),
                ("slit_rotation", C.c_double)]


class PlaneDesc(C.Structure):
    _fields_ = [("center", C.c_double * 3), ("normal", C.c_double * 3), ("size", C.c_double * 2),
                ("count", C.c_int32 * 2)]


class AbsorbingDesc(C.Structure):
    _fields_ = [("bottom", C.c_double * 3), ("top", C.c_double * 3), ("offset", C.c_double),
                ("potential_pos", C.c_double * 3), ("potential_neg", C.c_double * 3),
                ("exponent_pos", C.c_double * 3), ("exponent_neg", C.c_double * 3)]


class Box(C.Structure):
    _fields_ = [("bottom", C.c_int32 * 3), ("count", C.c_int32 * 3)]


class BatchDesc(C.Structure):
    _fields_ = [("ninst", C.c_int32), ("n", C.POINTER(C.c_int32)), ("extent", C.POINTER(C.c_double)),
                ("device", C.c_int32), ("stream", C.c_void_p)]


_lib = None


class RenderDesc(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("azimuth_deg", C.c_double),
                ("elevation_deg", C.c_double), ("fov_deg", C.c_double), ("distance", C.c_double),
                ("relative_step", C.c_double), ("wave_function_scale", C.c_double),
                ("potential_scale", C.c_double), ("light", C.c_double * 3), ("shadow_steps", C.c_int32),
                ("show_potential", C.c_int32), ("format", C.c_int32)]


def render_desc(width=1024, height=768, azimuth=0.0, elevation=45.0, fov=45.0, distance=0.0, relative_step=0.1,
                wave_function_scale=0.005, potential_scale=0.0, light=(1.0, 1.0, -1.0), shadow_steps=0,
                show_potential=True, float_output=False) -> RenderDesc:
    """Render settings with the reference's defaults (sources/volumetric_visualization.py,
    sources/multi_volume_visual.py): 1024 x 768, elevation 45, fov 45, step 0.1 voxel,
    colour limit 0.005, light (1, 1, -1). Shadows (the reference's 50-step march per
    sample) are off by default because they multiply the cost by ~100."""
    return RenderDesc(int(width), int(height), float(azimuth), float(elevation), float(fov), float(distance),
                      float(relative_step), float(wave_function_scale), float(potential_scale),
                      (C.c_double * 3)(*light), int(shadow_steps), 1 if show_potential else 0,
                      1 if float_output else 0)


def load(path: str | os.PathLike | None = None):
    """Loads ``_wfs.so`` once and declares argument types. Raises if absent."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise ImportError(f"{p} is missing: build it with wavefunctionsimpython_gb300.build_ext.build()")
    lib = C.CDLL(str(p))
    vp, i32, dbl, i64 = C.c_void_p, C.c_int32, C.c_double, C.c_int64
    dp = C.POINTER(C.c_double)
    sig = {
        "wfs_abi_version": ([], C.c_int),
        "wfs_global_error": ([], C.c_char_p),
        "wfs_create": ([C.POINTER(GridDesc), C.POINTER(vp)], C.c_int),
        "wfs_destroy": ([vp], C.c_int),
        "wfs_last_error": ([vp], C.c_char_p),
        "wfs_synchronize": ([vp], C.c_int),
        "wfs_set_copy_wait_limit": ([vp, dbl], C.c_int),
        "wfs_potential_clear": ([vp], C.c_int),
        "wfs_potential_add_wall": ([vp, C.POINTER(WallDesc)], C.c_int),
        "wfs_potential_add_absorbing": ([vp, C.POINTER(AbsorbingDesc)], C.c_int),
        "wfs_set_dynamic_walls": ([vp, C.POINTER(WallDesc), dp, i32, C.POINTER(AbsorbingDesc)], C.c_int),
        "wfs_get_dynamic_walls": ([vp, dp, i32], C.c_int),
        "wfs_potential_add_raw": ([vp, vp, i32, i32], C.c_int),
        "wfs_set_potential": ([vp, vp, i32], C.c_int),
        "wfs_get_potential": ([vp, vp, i32], C.c_int),
        "wfs_init_gaussian": ([vp, dp, dp, dp], C.c_int),
        "wfs_set_psi": ([vp, vp, i32], C.c_int),
        "wfs_get_psi": ([vp, vp, i32], C.c_int),
        "wfs_psi_device_ptr": ([vp, C.POINTER(vp)], C.c_int),
        "wfs_step_split": ([vp, i32, dbl, dbl], C.c_int),
        "wfs_step_taylor": ([vp, i32, dbl, dbl, i32, i32], C.c_int),
        "wfs_kinetic_operator": ([vp, dbl, dbl, dbl, vp, i32], C.c_int),
        "wfs_potential_operator": ([vp, dbl, vp, i32], C.c_int),
        "wfs_observe": ([vp, C.POINTER(Box), i32, C.POINTER(Box), dp, dp, dp], C.c_int),
        "wfs_run_split": ([vp, i32, dbl, dbl, i32, C.POINTER(Box), i32, C.POINTER(Box), dp, dp], C.c_int),
        "wfs_run_split_planes": ([vp, i32, dbl, dbl, i32, C.POINTER(Box), i32, C.POINTER(Box), C.POINTER(PlaneDesc),
                                  i32, dp, dp, dp], C.c_int),
        "wfs_norm": ([vp, dp], C.c_int),
        "wfs_profile_enable": ([vp, i32], C.c_int),
        "wfs_profile_read": ([vp, dp, C.POINTER(C.c_int64), i32], C.c_int),
        "wfs_launch_count": ([vp, C.POINTER(C.c_int64)], C.c_int),
        "wfs_set_schedule": ([vp, i32], C.c_int),
        "wfs_split_step_gain": ([C.POINTER(C.c_int32), i32, dp, dp], C.c_int),
        "wfs_batch_create": ([C.POINTER(BatchDesc), C.POINTER(vp)], C.c_int),
        "wfs_batch_destroy": ([vp], C.c_int),
        "wfs_batch_last_error": ([vp], C.c_char_p),
        "wfs_batch_synchronize": ([vp], C.c_int),
        "wfs_batch_init_gaussian": ([vp, i32, dp, dp, dp], C.c_int),
        "wfs_batch_add_wall": ([vp, i32, C.POINTER(WallDesc)], C.c_int),
        "wfs_batch_add_absorbing": ([vp, i32, C.POINTER(AbsorbingDesc)], C.c_int),
        "wfs_batch_set_potential": ([vp, i32, vp, i32], C.c_int),
        "wfs_batch_set_psi": ([vp, i32, vp, i32], C.c_int),
        "wfs_batch_get_psi": ([vp, i32, vp, i32], C.c_int),
        "wfs_batch_run": ([vp, i32, dbl, dbl, i32], C.c_int),
        "wfs_batch_observe": ([vp, C.POINTER(Box), dp], C.c_int),
        "wfs_batch_set_config": ([vp, i32, i32], C.c_int),
        "wfs_batch_autotune": ([vp, dbl, dbl, i32, C.POINTER(i32), C.POINTER(i32), dp], C.c_int),
        "wfs_batch_launch_count": ([vp, C.POINTER(C.c_int64)], C.c_int),
        "wfs_observe_noalloc": ([vp, i32, C.POINTER(i32), dp, C.POINTER(Box), i32, C.POINTER(Box), dp, vp], C.c_int),
        "wfs_plane_current": ([vp, dp, dp, dp, C.POINTER(i32), dbl, dp, vp, i32], C.c_int),
        "wfs_render": ([vp, C.POINTER(RenderDesc), vp, i32], C.c_int),
        "wfs_render_volume": ([vp, i32, C.POINTER(i32), vp, C.POINTER(RenderDesc), vp, vp], C.c_int),
        # surrogate kernels (include/wfs_fno.h); every pointer is a device pointer
        "wfs_fno_pointwise": ([vp, i32, vp, vp, vp, vp, vp, vp, i32, i32, i64, i32, vp], C.c_int),
        "wfs_fno_pointwise_backward": ([vp, vp, vp, i32, vp, vp, vp, i32, i32, i32, i64, vp], C.c_int),
        "wfs_fno_wgrad_scratch": ([i32, i32], C.c_int64),
        "wfs_fno_weight_grad": ([vp, i32, vp, i32, i32, i64, vp, vp, vp], C.c_int),
        "wfs_fno_fft3": ([vp, i64, i32, i32, vp], C.c_int),
        "wfs_fno_gather": ([vp, vp, i32, i32, i32, i32, vp], C.c_int),
        "wfs_fno_scatter": ([vp, vp, i32, i32, i32, i32, vp], C.c_int),
        "wfs_fno_pack_weights": ([vp, vp, vp, i32, i32, vp], C.c_int),
        "wfs_fno_mix": ([vp, vp, vp, i32, i32, i32, vp], C.c_int),
        "wfs_fno_spectral_weight_grad": ([vp, vp, vp, i32, i32, i32, vp], C.c_int),
        "wfs_fno_adam": ([vp, vp, vp, vp, i64, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, i32, vp],
                         C.c_int),
        "wfs_fno_loss": ([vp, vp, i64, i32, C.c_float, vp, vp, vp, vp], C.c_int),
        "wfs_fno_sample_norms": ([vp, vp, i64, i32, vp, vp, vp], C.c_int),
        "wfs_fno_make_input": ([vp, vp, C.c_float, vp, vp, i32, i64, vp], C.c_int),
        "wfs_fno_scale_samples": ([vp, vp, i32, i32, i64, vp], C.c_int),
        "wfs_fno_fast_lift": ([vp, i64, vp, i64, C.c_float, vp, vp, vp, vp, vp, i32, vp], C.c_int),
        "wfs_fno_fast_layer": ([vp, vp, vp, vp, vp, i32, vp], C.c_int),
        "wfs_fno_fast_last": ([vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, i32, vp], C.c_int),
        "wfs_fno_fast_xmix": ([vp, vp, i32, vp], C.c_int),
        "wfs_fno_pack_mix_interleaved": ([vp, vp, i32, i32, vp], C.c_int),
        "wfs_fno_to_bf16": ([vp, i32, i32, vp, i32, i32, i32, vp], C.c_int),
        "wfs_fno_set_wait_limit": ([C.c_double], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    _lib = lib
    return lib


def _d3(v):
    return (C.c_double * 3)(*[float(x) for x in v])


def make_box(bottom, count) -> Box:
    b = Box()
    for i in range(3):
        b.bottom[i] = int(bottom[i])
        b.count[i] = int(count[i])
    return b


class Engine:
    """One engine handle: psi, V and tables of one grid on one CUDA device."""

    def __init__(self, n, extent, double_precision=False, device=0, stream=None):
        self.lib = load()
        self.n = tuple(int(x) for x in n)
        self.extent = tuple(float(x) for x in extent)
        self.double_precision = bool(double_precision)
        self.dtype = np.complex128 if double_precision else np.complex64
        d = GridDesc()
        for i in range(3):
            d.n[i] = self.n[i]
            d.extent[i] = self.extent[i]
        d.dtype = WFS_C128 if double_precision else WFS_C64
        d.device = int(device)
        d.stream = stream
        h = C.c_void_p()
        rc = self.lib.wfs_create(C.byref(d), C.byref(h))
        if rc != WFS_OK:
            raise WfsError(rc, self.lib.wfs_global_error().decode())
        self.h = h

    @property
    def dx(self):
        return tuple(self.extent[i] / self.n[i] for i in range(3))

    def _ck(self, rc):
        if rc != WFS_OK:
            raise WfsError(rc, self.lib.wfs_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.wfs_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- potential ---
    def potential_clear(self):
        self._ck(self.lib.wfs_potential_clear(self.h))

    def add_wall(self, potential_hartree, center, normal, plateau, slope=0.0, slope_exponent=1.0,
                 slit_count=0, slit_spacing=1.0, slit_width=0.5, slit_rotation=0.0):
        w = WallDesc(float(potential_hartree), _d3(center), _d3(normal), float(plateau), float(slope),
                     float(slope_exponent), int(slit_count), float(slit_spacing), float(slit_width),
                     float(slit_rotation))
        self._ck(self.lib.wfs_potential_add_wall(self.h, C.byref(w)))

    def add_absorbing(self, bottom, top, offset, potential_pos, potential_neg, exponent_pos, exponent_neg):
        a = AbsorbingDesc(_d3(bottom), _d3(top), float(offset), _d3(potential_pos), _d3(potential_neg),
                          _d3(exponent_pos), _d3(exponent_neg))
        self._ck(self.lib.wfs_potential_add_absorbing(self.h, C.byref(a)))

    def set_dynamic_walls(self, walls, velocities, absorbing=None):
        """Dynamic potential mode. walls: sequences of add_wall's arguments (potential,
        center, normal, plateau, slope, slope_exponent, slit_count, slit_spacing,
        slit_width, slit_rotation); velocities: one 3-vector per wall; absorbing: the
        seven add_absorbing arguments or None. After every later step the walls advect
        and V is rebuilt from them and the absorbing ramp on the device."""
        n = len(walls)
        arr = (WallDesc * max(n, 1))()
        for i, w in enumerate(walls):
            defaults = [0.0, 1.0, 0, 1.0, 0.5, 0.0]  # slope, slope exponent, slits, spacing, width, rotation
            w = list(w) + defaults[len(w) - 4:]
            arr[i] = WallDesc(float(w[0]), _d3(w[1]), _d3(w[2]), float(w[3]), float(w[4]), float(w[5]), int(w[6]),
                              float(w[7]), float(w[8]), float(w[9]))
        vel = np.ascontiguousarray(np.asarray(velocities, np.float64).reshape(n, 3) if n else np.zeros((1, 3)))
        ab = None
        if absorbing is not None:
            b, t, off, pp, pn, ep, en = absorbing
            ab = AbsorbingDesc(_d3(b), _d3(t), float(off), _d3(pp), _d3(pn), _d3(ep), _d3(en))
        self._ck(self.lib.wfs_set_dynamic_walls(self.h, arr, vel.ctypes.data_as(C.POINTER(C.c_double)), n,
                                                C.byref(ab) if ab is not None else None))
        self._ndyn = n

    def get_dynamic_walls(self):
        """Current centres of the dynamic walls, shape (nwall, 3)."""
        n = getattr(self, "_ndyn", 0)
        out = np.zeros((max(n, 1), 3), np.float64)
        self._ck(self.lib.wfs_get_dynamic_walls(self.h, out.ctypes.data_as(C.POINTER(C.c_double)), n))
        return out[:n]

    def add_raw_potential(self, array: np.ndarray):
        arr = np.ascontiguousarray(array)
        if arr.shape != self.n:
            raise ValueError(f"raw potential shape {arr.shape} != grid {self.n}")
        t = RAW_TYPES.get(arr.dtype.name)
        if t is None:
            raise ValueError(f"unsupported raw potential dtype {arr.dtype}")
        self._ck(self.lib.wfs_potential_add_raw(self.h, arr.ctypes.data, t, 0))

    def set_potential(self, V: np.ndarray):
        arr = np.ascontiguousarray(V, dtype=np.complex64)
        if arr.shape != self.n:
            raise ValueError("potential shape mismatch")
        self._ck(self.lib.wfs_set_potential(self.h, arr.ctypes.data, 0))

    def get_potential(self) -> np.ndarray:
        out = np.empty(self.n, dtype=np.complex64)
        self._ck(self.lib.wfs_get_potential(self.h, out.ctypes.data, 0))
        return out

    # --- psi ---
    def init_gaussian(self, sigma, r0, k0):
        self._ck(self.lib.wfs_init_gaussian(self.h, _d3(sigma), _d3(r0), _d3(k0)))

    def set_psi(self, psi):
        if hasattr(psi, "__cuda_array_interface__"):
            ci = psi.__cuda_array_interface__
            if tuple(ci["shape"]) != self.n or np.dtype(ci["typestr"]) != np.dtype(self.dtype):
                raise ValueError("device psi has the wrong shape or dtype")
            if ci.get("strides") not in (None,):
                exp = tuple(np.dtype(self.dtype).itemsize * int(np.prod(self.n[i + 1:])) for i in range(3))
                if tuple(ci["strides"]) != exp:
                    raise ValueError("device psi must be C-contiguous")
            self._ck(self.lib.wfs_set_psi(self.h, C.c_void_p(ci["data"][0]), 1))
            return
        arr = np.ascontiguousarray(psi, dtype=self.dtype)
        if arr.shape != self.n:
            raise ValueError(f"psi shape {arr.shape} != grid {self.n}")
        self._ck(self.lib.wfs_set_psi(self.h, arr.ctypes.data, 0))

    def get_psi(self, out: np.ndarray | None = None) -> np.ndarray:
        """Real-space psi copied to host memory (``out`` may be a pinned, C-contiguous buffer)."""
        if out is None:
            out = np.empty(self.n, dtype=self.dtype)
        elif out.shape != self.n or out.dtype != np.dtype(self.dtype) or not out.flags.c_contiguous:
            raise ValueError("out must be a C-contiguous array of the grid's shape and dtype")
        self._ck(self.lib.wfs_get_psi(self.h, out.ctypes.data, 0))
        return out

    def psi_device_ptr(self) -> int:
        p = C.c_void_p()
        self._ck(self.lib.wfs_psi_device_ptr(self.h, C.byref(p)))
        return int(p.value or 0)

    # --- propagation ---
    def step_split(self, nsteps, dt, mass=1.0):
        self._ck(self.lib.wfs_step_split(self.h, int(nsteps), float(dt), float(mass)))

    def step_taylor(self, nsteps, dt, mass=1.0, order=10, stencil_order=2):
        self._ck(self.lib.wfs_step_taylor(self.h, int(nsteps), float(dt), float(mass), int(order), int(stencil_order)))

    def kinetic_operator(self, dt, mass=1.0, fraction=0.25) -> np.ndarray:
        out = np.empty(self.n, dtype=self.dtype)
        self._ck(self.lib.wfs_kinetic_operator(self.h, float(dt), float(mass), float(fraction), out.ctypes.data, 0))
        return out

    def potential_operator(self, dt, inout: np.ndarray) -> np.ndarray:
        arr = np.ascontiguousarray(inout, dtype=self.dtype).copy()
        self._ck(self.lib.wfs_potential_operator(self.h, float(dt), arr.ctypes.data, 0))
        return arr

    def synchronize(self):
        self._ck(self.lib.wfs_synchronize(self.h))

    def set_copy_wait_limit(self, seconds):
        """Limit of a copy-staged pass's wait for a staged tile (test hook: 0 gives up at once)."""
        self._ck(self.lib.wfs_set_copy_wait_limit(self.h, float(seconds)))

    # --- observables ---
    @staticmethod
    def _boxes(boxes):
        nb = len(boxes)
        if nb > MAX_BOX:
            raise ValueError(f"at most {MAX_BOX} volume boxes per observation")
        arr = (Box * max(nb, 1))()
        for i, (b, c) in enumerate(boxes):
            arr[i] = make_box(b, c)
        return arr, nb

    def observe(self, boxes=(), loc=None):
        """boxes: [(bottom_voxel, count)], loc: (bottom_voxel, count) or None.
        Returns (probabilities[nbox], <r>[3] or None, <r^2>[3] or None)."""
        arr, nb = self._boxes(boxes)
        lb = make_box(*loc) if loc is not None else None
        prob = (C.c_double * max(nb, 1))()
        r = (C.c_double * 3)()
        r2 = (C.c_double * 3)()
        self._ck(self.lib.wfs_observe(self.h, arr, nb, C.byref(lb) if lb is not None else None, prob, r, r2))
        return (np.array(prob[:nb]), np.array(r[:]) if lb is not None else None,
                np.array(r2[:]) if lb is not None else None)

    def run_split(self, nsteps, dt, mass=1.0, interval=1, boxes=(), loc=None):
        arr, nb = self._boxes(boxes)
        lb = make_box(*loc) if loc is not None else None
        nrec = -(-int(nsteps) // int(interval)) if (nb or lb is not None) else 0
        ps = np.zeros((max(nrec, 1), max(nb, 1)), dtype=np.float64)
        ls = np.zeros((max(nrec, 1), 6), dtype=np.float64)
        self._ck(self.lib.wfs_run_split(self.h, int(nsteps), float(dt), float(mass), int(interval), arr, nb,
                                        C.byref(lb) if lb is not None else None,
                                        ps.ctypes.data_as(C.POINTER(C.c_double)),
                                        ls.ctypes.data_as(C.POINTER(C.c_double))))
        return ps[:nrec, :nb], ls[:nrec]

    def run_split_planes(self, nsteps, dt, mass=1.0, interval=1, boxes=(), loc=None, planes=()):
        """run_split that also records, before every interval-th step, the probability flux
        through each plane (center, normal, size[2], count[2]). Returns (probabilities,
        locations, fluxes[nrec, nplane])."""
        arr, nb = self._boxes(boxes)
        lb = make_box(*loc) if loc is not None else None
        npl = len(planes)
        parr = (PlaneDesc * max(npl, 1))()
        for i, (c, nrm, size, count) in enumerate(planes):
            parr[i] = PlaneDesc(_d3(c), _d3(nrm), (C.c_double * 2)(*[float(x) for x in size]),
                                (C.c_int32 * 2)(*[int(x) for x in count]))
        nrec = -(-int(nsteps) // int(interval)) if (nb or lb is not None or npl) else 0
        ps = np.zeros((max(nrec, 1), max(nb, 1)), dtype=np.float64)
        ls = np.zeros((max(nrec, 1), 6), dtype=np.float64)
        fs = np.zeros((max(nrec, 1), max(npl, 1)), dtype=np.float64)
        self._ck(self.lib.wfs_run_split_planes(self.h, int(nsteps), float(dt), float(mass), int(interval), arr, nb,
                                               C.byref(lb) if lb is not None else None, parr, npl,
                                               ps.ctypes.data_as(C.POINTER(C.c_double)),
                                               ls.ctypes.data_as(C.POINTER(C.c_double)),
                                               fs.ctypes.data_as(C.POINTER(C.c_double))))
        return ps[:nrec, :nb], ls[:nrec], fs[:nrec, :npl]

    def profile_enable(self, on=True, stride=1):
        """Bracket the launches of every ``stride``-th step with CUDA events (0/False: off)."""
        self._ck(self.lib.wfs_profile_enable(self.h, int(stride) if on else 0))

    def profile_read(self, reset=True):
        """Returns {pass name: (total ms, launches)} accumulated since the last reset."""
        ms = (C.c_double * NPASS)()
        cnt = (C.c_int64 * NPASS)()
        self._ck(self.lib.wfs_profile_read(self.h, ms, cnt, 1 if reset else 0))
        return {PASS_NAMES[k]: (ms[k], cnt[k]) for k in range(NPASS) if cnt[k]}

    def set_schedule(self, name: str):
        """'auto' (fused yz-plane pass where possible), 'axis' (one pass per axis) or 'plane'."""
        self._ck(self.lib.wfs_set_schedule(self.h, SCHEDULES[name]))

    def launch_count(self) -> int:
        v = C.c_int64()
        self._ck(self.lib.wfs_launch_count(self.h, C.byref(v)))
        return v.value

    def plane_current(self, center, normal, size, sample_count, mass=1.0, density=False):
        """Flux of the probability current through a plane (odd sample counts).
        With density=True also returns the sampled current density."""
        flux = C.c_double()
        cnt = (C.c_int32 * 2)(int(sample_count[0]), int(sample_count[1]))
        dens = None
        if density:
            dens = np.empty((int(sample_count[0]), int(sample_count[1])),
                            dtype=np.float64 if self.double_precision else np.float32)
        self._ck(self.lib.wfs_plane_current(self.h, _d3(center), _d3(normal), (C.c_double * 2)(*map(float, size)), cnt,
                                            float(mass), C.byref(flux), dens.ctypes.data if dens is not None else None, 0))
        return (flux.value, dens) if density else flux.value

    def render(self, desc: "RenderDesc | None" = None, **kw) -> np.ndarray:
        """Ray-marched image of psi (and V) as an (height, width, 4) uint8 RGBA array, or
        float32 when desc.format is 1; keyword arguments build the desc (render_desc)."""
        d = desc if desc is not None else render_desc(**kw)
        dtype = np.float32 if d.format == 1 else np.uint8
        img = np.empty((d.height, d.width, 4), dtype=dtype)
        self._ck(self.lib.wfs_render(self.h, C.byref(d), img.ctypes.data, 0))
        return img

    def norm(self) -> float:
        v = C.c_double()
        self._ck(self.lib.wfs_norm(self.h, C.byref(v)))
        return v.value


class Batch:
    """Many independent wave packets on uneven cubic grids, advanced together (complex64)."""

    def __init__(self, sizes, extents, device=0, stream=None):
        self.lib = load()
        self.sizes = [int(s) for s in sizes]
        self.extents = [float(e) for e in extents]
        self.ninst = len(self.sizes)
        n = (C.c_int32 * self.ninst)(*self.sizes)
        ext = (C.c_double * self.ninst)(*self.extents)
        d = BatchDesc(self.ninst, n, ext, int(device), stream)
        h = C.c_void_p()
        rc = self.lib.wfs_batch_create(C.byref(d), C.byref(h))
        if rc != WFS_OK:
            raise WfsError(rc, self.lib.wfs_batch_last_error(None).decode())
        self.h = h

    def _ck(self, rc):
        if rc != WFS_OK:
            raise WfsError(rc, self.lib.wfs_batch_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.wfs_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def init_gaussian(self, i, sigma, r0, k0):
        self._ck(self.lib.wfs_batch_init_gaussian(self.h, int(i), _d3(sigma), _d3(r0), _d3(k0)))

    def add_wall(self, i, potential_hartree, center, normal, plateau, slope=0.0, slope_exponent=1.0,
                 slit_count=0, slit_spacing=1.0, slit_width=0.5, slit_rotation=0.0):
        w = WallDesc(float(potential_hartree), _d3(center), _d3(normal), float(plateau), float(slope),
                     float(slope_exponent), int(slit_count), float(slit_spacing), float(slit_width), float(slit_rotation))
        self._ck(self.lib.wfs_batch_add_wall(self.h, int(i), C.byref(w)))

    def add_absorbing(self, i, bottom, top, offset, potential_pos, potential_neg, exponent_pos, exponent_neg):
        a = AbsorbingDesc(_d3(bottom), _d3(top), float(offset), _d3(potential_pos), _d3(potential_neg),
                          _d3(exponent_pos), _d3(exponent_neg))
        self._ck(self.lib.wfs_batch_add_absorbing(self.h, int(i), C.byref(a)))

    def set_potential(self, i, V):
        arr = np.ascontiguousarray(V, dtype=np.complex64)
        L = self.sizes[i]
        if arr.shape != (L, L, L):
            raise ValueError("potential shape mismatch")
        self._ck(self.lib.wfs_batch_set_potential(self.h, int(i), arr.ctypes.data, 0))

    def set_psi(self, i, psi):
        arr = np.ascontiguousarray(psi, dtype=np.complex64)
        L = self.sizes[i]
        if arr.shape != (L, L, L):
            raise ValueError("psi shape mismatch")
        self._ck(self.lib.wfs_batch_set_psi(self.h, int(i), arr.ctypes.data, 0))

    def get_psi(self, i):
        L = self.sizes[i]
        out = np.empty((L, L, L), dtype=np.complex64)
        self._ck(self.lib.wfs_batch_get_psi(self.h, int(i), out.ctypes.data, 0))
        return out

    # device-pointer variants (complex64 L^3 buffers already on this batch's GPU)
    def set_psi_device(self, i, ptr):
        self._ck(self.lib.wfs_batch_set_psi(self.h, int(i), int(ptr), 1))

    def get_psi_device(self, i, ptr):
        self._ck(self.lib.wfs_batch_get_psi(self.h, int(i), int(ptr), 1))

    def set_potential_device(self, i, ptr):
        self._ck(self.lib.wfs_batch_set_potential(self.h, int(i), int(ptr), 1))

    def run(self, nsteps, dt, mass=1.0, graph=True):
        self._ck(self.lib.wfs_batch_run(self.h, int(nsteps), float(dt), float(mass), 1 if graph else 0))

    def synchronize(self):
        self._ck(self.lib.wfs_batch_synchronize(self.h))

    def observe(self, boxes):
        """boxes: list of (bottom_voxel, count), one per instance -> probabilities."""
        if len(boxes) != self.ninst:
            raise ValueError("one box per instance")
        arr = (Box * self.ninst)()
        for i, (b, c) in enumerate(boxes):
            arr[i] = make_box(b, c)
        out = (C.c_double * self.ninst)()
        self._ck(self.lib.wfs_batch_observe(self.h, arr, out))
        return np.array(out[:])

    def set_config(self, cluster, swap=0):
        self._ck(self.lib.wfs_batch_set_config(self.h, int(cluster), int(swap)))

    def autotune(self, dt, mass=1.0, steps=5):
        """Times the cluster setting {0 (two-pass mode), 1, 2, 4, 8, 16} x radix orientation {0, 1};
        keeps the fastest. Returns (cluster, swap, table of ms per step)."""
        cl, sw = C.c_int32(), C.c_int32()
        ms = (C.c_double * 12)()
        self._ck(self.lib.wfs_batch_autotune(self.h, float(dt), float(mass), int(steps), C.byref(cl), C.byref(sw), ms))
        table = {(c, s): ms[s * 6 + k] for s in (0, 1) for k, c in enumerate((0, 1, 2, 4, 8, 16))}
        return cl.value, sw.value, table

    def launch_count(self) -> int:
        v = C.c_int64()
        self._ck(self.lib.wfs_batch_launch_count(self.h, C.byref(v)))
        return v.value
