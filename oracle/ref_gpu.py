"""GPU oracle: the reference project's own CUDA kernels run on its own call sequence (TEST INFRASTRUCTURE).

``oracle/build_ref.py`` compiles the reference's kernel files, with the
reference's own text substitutions, into fatbinaries under ``oracle/_ref/``.
This module loads them through the CUDA driver API (ctypes on libcuda) and
replays the reference's host logic around them, operation for operation:

* ``SimState._fft_time_evolution`` (``sources/sim_state.py:641-697``): fftn,
  kinetic kernel, ifftn, potential kernel, fftn, kinetic kernel, ifftn, with
  ``norm="ortho"``. CuPy's ``cp.fft.fftn/ifftn`` call cuFFT; here
  ``torch.fft.fftn/ifftn`` call the same library. The wave numbers are
  ``2*pi*fftfreq(N, dx)`` in float64 (``sources/sim_state.py:275-278``).
* ``SimState._power_series_time_evolution`` (``sources/sim_state.py:721-752``):
  grid (64, 64, 64), block N/64 per axis, ping-pong buffers, ``next_s`` per term.
* The initial packet (``sources/wave_packet.py:97-151``), the potential
  (``sources/sim_state.py:210-255``: pre-initialised array, absorbing ramp, then
  each wall built in a zero array and added), ``VolumeProbability.calculate``
  (``sources/measurement.py:92-170``) and ``ExpectedLocation.calculate``
  (``sources/measurement.py:318-382``).
* Launch shapes from ``math_utils.get_grid_size_block_size``
  (``sources/math_utils.py:152-197``), including its cache keyed by shape only.

Nothing in the product imports this module; only tests and the fixture
generator under ``tests/golden/`` do. It needs a GPU, PyTorch and the
fatbinaries; ``available()`` says whether they are present.
"""
from __future__ import annotations

import ctypes
import math
import os
from pathlib import Path

import numpy as np

from oracle import build_ref

REF_DIR = Path(__file__).resolve().parent / "_ref"


def available():
    """True when the reference kernels were built (oracle/_ref/*.fatbin present)."""
    return (REF_DIR / build_ref.fatbin_name("kinetic_operator", "float")).exists()


# ---------------------------------------------------------------------------
# CUDA driver API through ctypes
# ---------------------------------------------------------------------------

_lib = None


def _cuda():
    global _lib
    if _lib is None:
        lib = ctypes.CDLL("libcuda.so.1")
        lib.cuGetErrorString.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p)]
        lib.cuModuleLoad.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_char_p]
        lib.cuModuleGetFunction.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p, ctypes.c_char_p]
        lib.cuModuleGetFunctionCount.argtypes = [ctypes.POINTER(ctypes.c_uint), ctypes.c_void_p]
        lib.cuModuleEnumerateFunctions.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_uint, ctypes.c_void_p]
        lib.cuLaunchKernel.argtypes = [ctypes.c_void_p] + [ctypes.c_uint] * 7 + [ctypes.c_void_p,
                                                                                  ctypes.POINTER(ctypes.c_void_p),
                                                                                  ctypes.c_void_p]
        _lib = lib
    return _lib


def _check(rc, what):
    if rc != 0:
        msg = ctypes.c_char_p()
        _cuda().cuGetErrorString(rc, ctypes.byref(msg))
        raise RuntimeError(f"{what}: CUDA driver error {rc} ({(msg.value or b'?').decode()})")


_functions = {}


def _function(fatbin: str, symbol=None):
    """Load oracle/_ref/<fatbin> (once) and return its kernel; template modules hold one."""
    key = (fatbin, symbol)
    if key in _functions:
        return _functions[key]
    path = REF_DIR / fatbin
    if not path.exists():
        raise FileNotFoundError(f"{path} missing: run oracle/build_ref.py where the reference sources are")
    lib = _cuda()
    mod = ctypes.c_void_p()
    _check(lib.cuModuleLoad(ctypes.byref(mod), str(path).encode()), f"cuModuleLoad {fatbin}")
    fn = ctypes.c_void_p()
    if symbol is not None:
        _check(lib.cuModuleGetFunction(ctypes.byref(fn), mod, symbol.encode()), f"cuModuleGetFunction {symbol}")
    else:
        cnt = ctypes.c_uint()
        _check(lib.cuModuleGetFunctionCount(ctypes.byref(cnt), mod), "cuModuleGetFunctionCount")
        if cnt.value != 1:
            raise RuntimeError(f"{fatbin}: expected one kernel, found {cnt.value}")
        arr = (ctypes.c_void_p * 1)()
        _check(lib.cuModuleEnumerateFunctions(arr, 1, mod), "cuModuleEnumerateFunctions")
        fn = ctypes.c_void_p(arr[0])
    _functions[key] = fn
    return fn


def _launch(fn, grid, block, args, shared=0, stream=None):
    import torch

    holders = []
    for a in args:
        if isinstance(a, torch.Tensor):
            holders.append(ctypes.c_void_p(a.data_ptr()))
        else:
            holders.append(a)
    params = (ctypes.c_void_p * len(holders))(*[ctypes.cast(ctypes.pointer(h), ctypes.c_void_p) for h in holders])
    s = torch.cuda.current_stream().cuda_stream if stream is None else stream
    _check(_cuda().cuLaunchKernel(fn, *[int(g) for g in grid], *[int(b) for b in block], int(shared),
                                  ctypes.c_void_p(s), params, None), "cuLaunchKernel")


# ---------------------------------------------------------------------------
# sources/math_utils.py:137-197
# ---------------------------------------------------------------------------

def nearest_power_of_2(n):
    """math_utils.py:137-146: n if n is a power of two, else the next one."""
    a = int(math.log2(n))
    return n if 2 ** a == n else 2 ** (a + 1)


class LaunchShapes:
    """get_grid_size_block_size with the reference's process-wide cache, which is keyed
    by the shape alone (a later call with reduced_thread_count=True for a cached shape
    gets the earlier, unreduced answer)."""

    def __init__(self):
        self.cache = {}

    def __call__(self, shape, reduced_thread_count=False):
        key = tuple(int(s) for s in shape)
        if key in self.cache:
            g = self.cache[key]
            return tuple(g), tuple(key[i] // g[i] for i in range(len(key)))
        allowed = 256 if reduced_thread_count else 1024
        guess = 2
        while True:
            grid, block, threads = [], [], 1
            for i in range(len(key)):
                grid.append(guess)
                if key[i] < guess:
                    grid[i] = key[i]
                while key[i] % grid[i] != 0:
                    grid[i] += 1
                b = key[i] // grid[i]
                threads *= b
                block.append(b)
            if threads <= allowed:
                break
            guess *= 2
        self.cache[key] = grid
        return tuple(grid), tuple(block)


# ---------------------------------------------------------------------------
# The reference's simulation state, driven through its kernels
# ---------------------------------------------------------------------------

class RefSim:
    """One reference run on the GPU: psi (complex64 or complex128) and V (complex64)
    as torch tensors, mutated by the reference's kernels in the reference's order."""

    def __init__(self, n, extent, double_precision=False, device=0):
        import torch

        self.torch = torch
        self.n = tuple(int(v) for v in n)
        self.extent = tuple(float(v) for v in extent)
        self.dx = np.asarray(self.extent, np.float64) / np.asarray(self.n, np.float64)  # sim_state.py:94
        self.dp = bool(double_precision)
        self.dev = torch.device("cuda", device)
        self.real = ctypes.c_double if self.dp else ctypes.c_float
        self.prec = "double" if self.dp else "float"
        self.shapes = LaunchShapes()
        self.grid, self.block = self.shapes(self.n)
        cdt = torch.complex128 if self.dp else torch.complex64
        self.psi = torch.zeros(self.n, dtype=cdt, device=self.dev)
        self.V = torch.zeros(self.n, dtype=torch.complex64, device=self.dev)
        k = [2.0 * np.pi * np.fft.fftfreq(n=self.n[a], d=self.dx[a]) for a in range(3)]
        self.k = [torch.as_tensor(v, dtype=torch.float64, device=self.dev) for v in k]
        self.ping = None

    # -- state ------------------------------------------------------------
    def init_gaussian(self, sigma, r0, k0):
        """wave_packet.py:97-151 (k0 = m v is given directly)."""
        fn = _function(build_ref.fatbin_name("gaussian_wave_packet", self.prec), "wave_packet_kernel")
        R = self.real
        self.psi.zero_()
        args = [self.psi] + [R(float(v)) for v in (*self.dx, *sigma, *r0, *k0)]
        _launch(fn, self.grid, self.block, args)

    def add_array(self, V):
        """Pre-initialised potential (potential.py:47-55): V += array."""
        self.V += self.torch.as_tensor(np.asarray(V, np.complex64), device=self.dev)

    def add_absorbing(self, ab):
        """potential.py:108-158 with the fields of oracle.wfs_oracle.Absorbing."""
        fn = _function(build_ref.fatbin_name("absorbing_potential", "-"), "absorbing_potential_kernel")
        f = ctypes.c_float
        vals = (*self.dx, *ab.bottom, *ab.top, ab.offset, *ab.potential_pos, *ab.potential_neg,
                *ab.exponent_pos, *ab.exponent_neg)
        g, b = self.shapes(self.n)
        _launch(fn, g, b, [self.V] + [f(float(v)) for v in vals])

    def add_wall(self, w):
        """potential.py:201-242 and sim_state.py:239-245: each wall is built in a zero
        array and added to V."""
        fn = _function(build_ref.fatbin_name("potential_wall", "-"), "potential_wall_kernel")
        f = ctypes.c_float
        tmp = self.torch.zeros(self.n, dtype=self.torch.complex64, device=self.dev)
        g, b = self.shapes(self.n)
        args = [tmp, f(w.potential_hartree), *[f(float(v)) for v in self.dx],
                *[f(float(v)) for v in w.center_bohr_radii_3], *[f(float(v)) for v in w.normal_vector_3],
                f(w.plateau_thickness_bohr_radii), f(w.slope_thickness_bohr_radii), f(w.slope_exponent),
                ctypes.c_uint32(int(w.slit_count)), f(w.slit_spacing_bohr_radii), f(w.slit_width_bohr_radii),
                f(w.slit_rotation_radian)]
        _launch(fn, g, b, args)
        self.V += tmp

    def build_scenario(self, sc):
        """Packet then potential, in SimState.initialize_state's order (sim_state.py:185-255)."""
        self.init_gaussian(sc.sigma, sc.r0, sc.k0)
        if sc.ho_omega is not None:
            from oracle import wfs_oracle as orc

            self.add_array(orc.harmonic_oscillator(self.n, self.dx, sc.ho_omega, sc.mass))
        if sc.absorbing is not None:
            self.add_absorbing(sc.absorbing)
        for w in sc.walls:
            self.add_wall(w)

    def set_psi(self, psi):
        self.psi = self.torch.as_tensor(np.ascontiguousarray(psi), device=self.dev).to(self.psi.dtype)

    def get_psi(self):
        self.torch.cuda.synchronize(self.dev)
        return self.psi.cpu().numpy()

    def get_potential(self):
        self.torch.cuda.synchronize(self.dev)
        return self.V.cpu().numpy()

    # -- propagation --------------------------------------------------------
    def _kinetic(self, dt, mass):
        fn = _function(build_ref.fatbin_name("kinetic_operator", self.prec), "kinetic_operator_kernel")
        _launch(fn, self.grid, self.block, [self.psi, self.real(dt), self.real(mass), *self.k])

    def _potential(self, dt):
        fn = _function(build_ref.fatbin_name("potential_operator", self.prec), "potential_operator_kernel")
        _launch(fn, self.grid, self.block, [self.psi, self.V, self.real(dt)])

    def split_step(self, dt, mass=1.0, nsteps=1, host_sync=False):
        """sim_state.py:641-697, nsteps times; host_sync adds the stream synchronisation
        that ends each of the reference's steps (sim_state.py:697)."""
        fft = self.torch.fft
        for _ in range(nsteps):
            self.psi = fft.fftn(self.psi, norm="ortho")
            self._kinetic(dt, mass)
            self.psi = fft.ifftn(self.psi, norm="ortho")
            self._potential(dt)
            self.psi = fft.fftn(self.psi, norm="ortho")
            self._kinetic(dt, mass)
            self.psi = fft.ifftn(self.psi, norm="ortho")
            if host_sync:
                self.torch.cuda.synchronize(self.dev)

    def taylor_step(self, dt, mass=1.0, order=10, nsteps=1):
        """sim_state.py:721-752 (single precision: the reference's ping-pong buffers and
        next_s operate on complex64)."""
        if self.dp:
            raise ValueError("the reference's power series runs on complex64 buffers only")
        if any(v % 64 for v in self.n):
            raise ValueError("the reference's power series launches a (64, 64, 64) grid: N must be a multiple of 64")
        fn = _function(build_ref.fatbin_name("power_series_operator", "float"), "next_s")
        grid = (64, 64, 64)
        block = tuple(self.n[i] // 64 for i in range(3))
        f = ctypes.c_float
        for _ in range(nsteps):
            ping = [self.torch.zeros_like(self.psi), self.torch.zeros_like(self.psi)]
            idx = 0
            ping[1 - idx] = self.psi.clone()
            for k in range(1, order + 1):
                _launch(fn, grid, block, [ping[1 - idx], ping[idx], self.V, self.psi, f(dt),
                                          f(self.dx[0]), f(self.dx[1]), f(self.dx[2]), f(mass),
                                          ctypes.c_int32(k)])
                idx = 1 - idx

    # -- measurement --------------------------------------------------------
    def _template_launch(self, stem, bottom_voxel, count, args_tail, outs):
        count = tuple(int(c) for c in count)
        box = count + self.n
        fn = _function(build_ref.fatbin_name(stem, self.prec, box))
        kshape = tuple(nearest_power_of_2(c) for c in count)
        g, b = self.shapes(kshape, reduced_thread_count=True)
        item = 8 if self.dp else 4
        shared = (3 if stem == "expected_location" else 1) * item * b[0] * b[1] * b[2]
        ity = ctypes.c_uint32 if stem == "volume_probability" else ctypes.c_int32
        args = [self.psi, *outs] + [self.real(float(v)) for v in self.dx] + [ity(int(v)) for v in bottom_voxel]
        _launch(fn, g, b, args, shared=shared)

    def volume_probability(self, bottom_voxel, count):
        """measurement.py:149-170: zero the buffer, one launch, read the sum."""
        rdt = self.torch.float64 if self.dp else self.torch.float32
        out = self.torch.zeros(1, dtype=rdt, device=self.dev)
        self._template_launch("volume_probability", bottom_voxel, count, (), [out])
        self.torch.cuda.synchronize(self.dev)
        return float(out.cpu().numpy()[0])

    def expected_location(self, bottom_voxel, count):
        """measurement.py:353-382: (<r>, <r^2>) as the kernel leaves them."""
        rdt = self.torch.float64 if self.dp else self.torch.float32
        er = self.torch.zeros(3, dtype=rdt, device=self.dev)
        er2 = self.torch.zeros(3, dtype=rdt, device=self.dev)
        self._template_launch("expected_location", bottom_voxel, count, (), [er, er2])
        self.torch.cuda.synchronize(self.dev)
        return er.cpu().numpy().astype(np.float64), er2.cpu().numpy().astype(np.float64)
