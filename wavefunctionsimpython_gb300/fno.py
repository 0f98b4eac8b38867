"""Fourier-neural-operator surrogate that jumps K split steps at once.

psi(t + K dt) ~ prior + FNO(psi(t), V), where prior is a coarse split step of the
same interval (``prior_steps`` Strang steps of K dt / prior_steps, run by the
batch engine) and the network (include/wfs_fno.h, csrc/fno.cu) learns the
correction. The exact propagator (K plain split steps) is both the training
target and the acceptance test: a jump whose relative L2 error or norm error
exceeds the tolerance is rejected and re-run with the plain method.

The reference has no learned propagator; the surrogate's trajectories come from
the same split step as sources/sim_state.py:641-697 (this package's engine), its
harmonic potentials follow sources/potential.py:414-423 and its barriers
sources/potential.py:161-198.

PyTorch only provides device memory, streams and events here; every compute
step is one of the package's CUDA kernels called through ctypes.
"""
from __future__ import annotations

import ctypes as C
import math
import time
from dataclasses import dataclass

import numpy as np

from . import _lib


@dataclass
class FnoConfig:
    N: int = 64               # grid points per axis
    extent: float = 40.0      # box edge (Bohr)
    width: int = 32           # hidden channels C
    modes: int = 12           # kept modes per axis m
    layers: int = 4           # spectral layers
    hidden: int = 64          # projection width
    jump_steps: int = 50      # K
    dt: float = 0.01          # plain split-step size
    mass: float = 1.0
    prior_steps: int = 2      # coarse Strang steps per jump
    vscale: float = 0.05      # V input scale (1 / Hartree)

    @property
    def n3(self):
        return self.N ** 3

    @property
    def nmodes(self):
        return 4 * self.modes ** 3


def _ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


# (N, width, modes, hidden) of the inference kernels in csrc/fno_fast.cu
FAST_GEOMETRY = (64, 32, 12, 64)


class FNO:
    """Network parameters, workspaces and the forward / backward / optimiser steps.

    Parameters live in one flat float32 device buffer (W then b for every
    pointwise layer, the complex spectral weights as interleaved float pairs), so
    one Adam launch updates all of them; BF16 tensor-core copies of the spectral
    weights are refreshed after each update."""

    def __init__(self, cfg: FnoConfig, device="cuda", seed=0, stream=None):
        import torch

        self.torch = torch
        self.cfg = cfg
        self.lib = _lib.load()
        self.device = torch.device(device)
        self.stream = stream if stream is not None else torch.cuda.current_stream(self.device)
        c, h, nm = cfg.width, cfg.hidden, cfg.nmodes
        layout = [("W0", (c, 4)), ("b0", (c,))]
        for l in range(cfg.layers):
            layout += [(f"W{l + 1}", (c, c)), (f"b{l + 1}", (c,)), (f"R{l + 1}", (nm, c, c, 2))]
        layout += [("Wq1", (h, c)), ("bq1", (h,)), ("Wq2", (2, h)), ("bq2", (2,))]
        self.layout = layout
        self.offsets = {}
        off = 0
        for name, shape in layout:
            n = int(np.prod(shape))
            self.offsets[name] = (off, shape)
            off += n
        self.nparams = off
        f32 = dict(dtype=torch.float32, device=self.device)
        self.flat = torch.zeros(off, **f32)
        self.grad = torch.zeros(off, **f32)
        self.m1 = torch.zeros(off, **f32)
        self.m2 = torch.zeros(off, **f32)
        self.step_count = 0
        self.Wbf = [torch.empty((nm, 2 * c, 2 * c), dtype=torch.bfloat16, device=self.device) for _ in range(cfg.layers)]
        self.WTbf = [torch.empty_like(w) for w in self.Wbf]
        self.ws = None
        self.ws_batch = 0
        self.fast_ws = None
        self.fast_batch = 0
        self.fast_ok = (cfg.N, cfg.width, cfg.modes, cfg.hidden) == FAST_GEOMETRY
        if self.fast_ok:
            bf = dict(dtype=torch.bfloat16, device=self.device)
            self.fast_w = {"W0": torch.empty((c, 16), **bf), "Wq1": torch.empty((h, c), **bf),
                           "Wq2": torch.empty((8, h), **bf)}
            for l in range(cfg.layers):
                self.fast_w[f"W{l + 1}"] = torch.empty((c, c), **bf)
            self.fast_mix = [torch.empty((nm, 2 * c, 2 * c), **bf) for _ in range(cfg.layers)]
        self.init_params(seed)

    # ---- parameters ---------------------------------------------------------------------------
    def view(self, name, buf=None):
        off, shape = self.offsets[name]
        return (self.flat if buf is None else buf)[off:off + int(np.prod(shape))].view(*shape)

    def init_params(self, seed=0):
        """Uniform(+-1/sqrt(fan_in)) pointwise weights, FNO-style spectral weights scaled by
        1/C^2, and a zero last layer so the untrained network returns the prior."""
        rng = np.random.default_rng(seed)
        cfg = self.cfg
        vals = {}

        def lin(o, i):
            b = 1.0 / math.sqrt(i)
            return rng.uniform(-b, b, (o, i)), rng.uniform(-b, b, o)

        vals["W0"], vals["b0"] = lin(cfg.width, 4)
        for l in range(1, cfg.layers + 1):
            vals[f"W{l}"], vals[f"b{l}"] = lin(cfg.width, cfg.width)
            vals[f"R{l}"] = rng.uniform(0, 1, (cfg.nmodes, cfg.width, cfg.width, 2)) / (cfg.width ** 2)
        vals["Wq1"], vals["bq1"] = lin(cfg.hidden, cfg.width)
        vals["Wq2"], vals["bq2"] = np.zeros((2, cfg.hidden)), np.zeros(2)
        self.set_params(vals)

    def set_params(self, vals: dict):
        """vals: name -> array (complex R arrays [nm][C][C] are accepted too)."""
        torch = self.torch
        for name, (off, shape) in self.offsets.items():
            if name not in vals:
                continue
            a = np.asarray(vals[name])
            if np.iscomplexobj(a):
                a = np.stack([a.real, a.imag], axis=-1)
            a = np.ascontiguousarray(a, dtype=np.float32).reshape(shape)
            self.view(name).copy_(torch.from_numpy(a).to(self.device))
        self.pack()

    def get_params(self) -> dict:
        out = {}
        for name, (off, shape) in self.offsets.items():
            a = self.view(name).cpu().numpy().astype(np.float64)
            out[name] = a[..., 0] + 1j * a[..., 1] if name.startswith("R") else a
        return out

    def get_grads(self) -> dict:
        out = {}
        for name, (off, shape) in self.offsets.items():
            a = self.view(name, self.grad).cpu().numpy().astype(np.float64)
            out[name] = a[..., 0] + 1j * a[..., 1] if name.startswith("R") else a
        return out

    def _s(self):
        return C.c_void_p(self.stream.cuda_stream)

    def _ck(self, rc, what):
        if rc != 0:
            raise _lib.WfsError(rc, f"{what} failed ({rc})")

    def pack(self):
        c = self.cfg.width
        for l in range(self.cfg.layers):
            self._ck(self.lib.wfs_fno_pack_weights(_ptr(self.view(f"R{l + 1}")), _ptr(self.Wbf[l]), _ptr(self.WTbf[l]),
                                                   c, self.cfg.nmodes, self._s()), "pack_weights")
        if self.fast_ok:
            for name, dst in self.fast_w.items():
                rows, cols = self.offsets[name][1]
                self._ck(self.lib.wfs_fno_to_bf16(_ptr(self.view(name)), rows, cols, _ptr(dst), dst.shape[0],
                                                  dst.shape[1], 1, self._s()), "to_bf16")
            for l in range(self.cfg.layers):
                self._ck(self.lib.wfs_fno_pack_mix_interleaved(_ptr(self.view(f"R{l + 1}")), _ptr(self.fast_mix[l]),
                                                               c, self.cfg.nmodes, self._s()), "pack_mix")

    # ---- workspaces ---------------------------------------------------------------------------
    def workspace(self, B):
        if self.ws is not None and self.ws_batch >= B:
            return self.ws
        torch = self.torch
        cfg = self.cfg
        c64 = dict(dtype=torch.complex64, device=self.device)
        n3, P, H2, L, nm = cfg.n3, cfg.width // 2, cfg.hidden // 2, cfg.layers, cfg.nmodes
        self.ws = None
        ws = {
            "h": [torch.empty((B, P, n3), **c64) for _ in range(L + 1)],
            "pre": [torch.empty((B, P, n3), **c64) for _ in range(L - 1)],
            "Y": torch.empty((B, P, n3), **c64),
            "Hm": [torch.empty((nm, B, cfg.width), **c64) for _ in range(L)],
            "Zm": torch.empty((nm, B, cfg.width), **c64),
            "Zm2": torch.empty((nm, B, cfg.width), **c64),
            "qpre": torch.empty((B, H2, n3), **c64),
            "q": torch.empty((B, H2, n3), **c64),
            "ga": torch.empty((B, P, n3), **c64),
            "g2": torch.empty((B, n3), **c64),
            "gout": torch.empty((B, n3), **c64),
            "out": torch.empty((B, n3), **c64),
            "sample_err": torch.empty(B, dtype=torch.float32, device=self.device),
            "loss": torch.empty(1, dtype=torch.float32, device=self.device),
        }
        scr = max(int(self.lib.wfs_fno_wgrad_scratch(ci, co)) for ci, co in
                  [(4, cfg.width), (cfg.width, cfg.width), (cfg.width, cfg.hidden), (cfg.hidden, 2)])
        ws["partials"] = torch.empty(scr, dtype=torch.float32, device=self.device)
        self.ws, self.ws_batch = ws, B
        return ws

    # ---- forward / backward -------------------------------------------------------------------
    def forward(self, x, prior, B, out=None, keep_pre=True):
        """x: [B][2][n3] complex64 network input; prior: [B][n3] complex64. Returns
        [B][n3] complex64 = prior + correction (a view of the workspace unless out is given).
        keep_pre=False skips storing the pre-activations, which only backward() reads
        (inference: a quarter less traffic in the hidden layers)."""
        cfg, lib, s = self.cfg, self.lib, self._s()
        ws = self.workspace(B)
        c, hdim, n3, N, m, L = cfg.width, cfg.hidden, cfg.n3, cfg.N, cfg.modes, cfg.layers
        Y = ws["Y"]
        ck = self._ck
        ck(lib.wfs_fno_pointwise(_ptr(x), 4, _ptr(self.view("W0")), _ptr(self.view("b0")), None, None,
                                 _ptr(ws["h"][0]), _ptr(Y), c, B, n3, 0, s), "lift")
        for l in range(L):
            ck(lib.wfs_fno_fft3(_ptr(Y), B * (c // 2), N, -1, s), "fft3")
            ck(lib.wfs_fno_gather(_ptr(Y), _ptr(ws["Hm"][l]), B, c, N, m, s), "gather")
            ck(lib.wfs_fno_mix(_ptr(ws["Hm"][l]), _ptr(self.Wbf[l]), _ptr(ws["Zm"]), B, c, cfg.nmodes, s), "mix")
            ck(lib.wfs_fno_scatter(_ptr(ws["Zm"]), _ptr(Y), B, c, N, m, s), "scatter")
            ck(lib.wfs_fno_fft3(_ptr(Y), B * (c // 2), N, 1, s), "ifft3")
            last = l == L - 1
            ck(lib.wfs_fno_pointwise(_ptr(ws["h"][l]), c, _ptr(self.view(f"W{l + 1}")), _ptr(self.view(f"b{l + 1}")),
                                     _ptr(Y), None if (last or not keep_pre) else _ptr(ws["pre"][l]), _ptr(ws["h"][l + 1]),
                                     None if last else _ptr(Y), c, B, n3, 0 if last else 1, s), "layer")
        ck(lib.wfs_fno_pointwise(_ptr(ws["h"][L]), c, _ptr(self.view("Wq1")), _ptr(self.view("bq1")), None,
                                 _ptr(ws["qpre"]) if keep_pre else None, _ptr(ws["q"]), None, hdim, B, n3, 1, s),
           "projection 1")
        dst = ws["out"] if out is None else out
        ck(lib.wfs_fno_pointwise(_ptr(ws["q"]), hdim, _ptr(self.view("Wq2")), _ptr(self.view("bq2")), _ptr(prior),
                                 None, _ptr(dst), None, 2, B, n3, 0, s), "projection 2")
        return dst[:B]

    def fast_workspace(self, B):
        if self.fast_ws is not None and self.fast_batch >= B:
            return self.fast_ws
        torch = self.torch
        cfg = self.cfg
        i32 = dict(dtype=torch.int32, device=self.device)
        self.fast_ws = None
        self.fast_ws = {"h": [torch.empty((B, cfg.width // 2, cfg.n3), **i32) for _ in range(2)],
                        "sy": torch.empty((B, cfg.N, 2 * cfg.modes, cfg.modes, cfg.width), **i32),
                        "out": torch.empty((B, cfg.n3), dtype=torch.complex64, device=self.device)}
        self.fast_batch = B
        return self.fast_ws

    def forward_fast(self, x, prior, B, out=None):
        """The same network as forward() for inference, on the kept modes only (csrc/fno_fast.cu):
        BF16 tensor-core products with FP32 accumulation and BF16 intermediates, one plane
        kernel per layer. x: [B][2][n3] normalised input, prior: [B][n3] normalised prior.
        Geometry N = 64, width 32, 12 modes, projection width 64."""
        n3 = self.cfg.n3
        return self._fast(x, 2 * n3, x[:, 1], 2 * n3, 1.0, None, prior, B, out, None)

    def jump_fast(self, psi, V, prior, a2, B, out=None, out_norm=None):
        """One surrogate jump on raw fields: out = prior + s_b FNO(psi / s_b, V vscale), with
        s_b = sqrt(a2_b / n3) (a2 from wfs_fno_sample_norms of psi). psi, V, prior:
        [B][n3] complex64; out_norm (optional, B doubles, zeroed by the caller) receives
        sum |out_b|^2."""
        n3 = self.cfg.n3
        return self._fast(psi, n3, V, n3, float(self.cfg.vscale), a2, prior, B, out, out_norm)

    def _fast(self, f0, s0, f1, s1, vscale, a2, prior, B, out, out_norm):
        if not self.fast_ok:
            raise ValueError(f"the inference kernels support (N, width, modes, hidden) = {FAST_GEOMETRY}")
        cfg, lib, s, ck = self.cfg, self.lib, self._s(), self._ck
        # the kernels address SY and H with the B they are given: a smaller batch uses the
        # leading part of each buffer
        ws = self.fast_workspace(B)
        sy, h, L, fw = ws["sy"], ws["h"], cfg.layers, self.fast_w
        dst = ws["out"] if out is None else out
        ck(lib.wfs_fno_fast_lift(_ptr(f0), s0, _ptr(f1), s1, vscale, _ptr(a2), _ptr(fw["W0"]), _ptr(self.view("b0")),
                                 _ptr(h[0]), _ptr(sy), B, s), "lift")
        for l in range(L):
            ck(lib.wfs_fno_fast_xmix(_ptr(sy), _ptr(self.fast_mix[l]), B, s), "xmix")
            hin, hout = h[l % 2], h[(l + 1) % 2]
            if l < L - 1:
                ck(lib.wfs_fno_fast_layer(_ptr(hin), _ptr(sy), _ptr(fw[f"W{l + 1}"]), _ptr(self.view(f"b{l + 1}")),
                                          _ptr(hout), B, s), "layer")
            else:
                ck(lib.wfs_fno_fast_last(_ptr(hin), _ptr(sy), _ptr(fw[f"W{l + 1}"]), _ptr(self.view(f"b{l + 1}")),
                                         _ptr(fw["Wq1"]), _ptr(self.view("bq1")), _ptr(fw["Wq2"]),
                                         _ptr(self.view("bq2")), _ptr(prior), _ptr(a2), _ptr(dst), _ptr(out_norm), B,
                                         s), "last")
        return dst[:B]

    def _wgrad(self, g, cout, x, cin, name_w, B):
        ws = self.ws
        off, _ = self.offsets[name_w]
        dst = C.c_void_p(self.grad.data_ptr() + 4 * off)  # W then b are contiguous in the flat buffer
        self._ck(self.lib.wfs_fno_weight_grad(_ptr(g), cout, _ptr(x), cin, B, self.cfg.n3, _ptr(ws["partials"]), dst,
                                              self._s()), "weight_grad")

    def backward(self, x, gout, B):
        """Gradients of every parameter into self.grad for d loss / d out = gout [B][n3]
        (the last forward call must have been on the same x and B)."""
        cfg, lib, s, ck = self.cfg, self.lib, self._s(), self._ck
        ws = self.ws
        c, hdim, n3, N, m, L = cfg.width, cfg.hidden, cfg.n3, cfg.N, cfg.modes, cfg.layers
        Y, ga, gq = ws["Y"], ws["ga"], ws["qpre"]  # gq reuses qpre's buffer after its last read
        # projection 2: out = Wq2 q + bq2 + prior
        self._wgrad(gout, 2, ws["q"], hdim, "Wq2", B)
        ck(lib.wfs_fno_pointwise_backward(_ptr(gout), None, None, 0, _ptr(self.view("Wq2")), _ptr(ws["g2"]),
                                          _ptr(ws["q"]), hdim, 2, B, n3, s), "projection 2 backward")
        # projection 1: q = GELU(Wq1 h_L + bq1); gq (in q's buffer) -> gqpre (in qpre's buffer)
        ck(lib.wfs_fno_pointwise_backward(_ptr(ws["q"]), None, _ptr(ws["qpre"]), 1, _ptr(self.view("Wq1")), _ptr(gq),
                                          _ptr(ga), c, hdim, B, n3, s), "projection 1 backward")
        self._wgrad(gq, hdim, ws["h"][L], c, "Wq1", B)
        have_spec = False
        for l in reversed(range(L)):
            last = l == L - 1
            ck(lib.wfs_fno_pointwise_backward(_ptr(ga), _ptr(Y) if have_spec else None,
                                              None if last else _ptr(ws["pre"][l]), 0 if last else 1,
                                              _ptr(self.view(f"W{l + 1}")), _ptr(Y), _ptr(ga), c, c, B, n3, s),
               "layer backward")
            self._wgrad(Y, c, ws["h"][l], c, f"W{l + 1}", B)
            ck(lib.wfs_fno_fft3(_ptr(Y), B * (c // 2), N, -1, s), "fft3")
            ck(lib.wfs_fno_gather(_ptr(Y), _ptr(ws["Zm"]), B, c, N, m, s), "gather")
            roff, _ = self.offsets[f"R{l + 1}"]
            ck(lib.wfs_fno_spectral_weight_grad(_ptr(ws["Hm"][l]), _ptr(ws["Zm"]),
                                                C.c_void_p(self.grad.data_ptr() + 4 * roff), B, c, cfg.nmodes, s),
               "spectral weight grad")
            ck(lib.wfs_fno_mix(_ptr(ws["Zm"]), _ptr(self.WTbf[l]), _ptr(ws["Zm2"]), B, c, cfg.nmodes, s), "mix adjoint")
            ck(lib.wfs_fno_scatter(_ptr(ws["Zm2"]), _ptr(Y), B, c, N, m, s), "scatter")
            ck(lib.wfs_fno_fft3(_ptr(Y), B * (c // 2), N, 1, s), "ifft3")
            have_spec = True
        # lift: h0 = W0 x + b0, gradient wrt h0 = ga + Y
        ck(lib.wfs_fno_pointwise_backward(_ptr(ga), _ptr(Y), None, 0, _ptr(self.view("W0")), _ptr(ga), None, 4, c, B,
                                          n3, s), "lift backward")
        self._wgrad(ga, c, x, 4, "W0", B)

    def loss(self, pred, target, B, grad=True, grad_scale=None):
        """Mean relative squared error over the batch (device scalar) and, when grad,
        grad_scale * d loss / d pred in the workspace's gout. The default scale (elements
        per sample) makes it the gradient of the per-element relative error."""
        ws = self.ws
        per = 2 * self.cfg.n3
        gs = float(per if grad_scale is None else grad_scale)
        self._ck(self.lib.wfs_fno_loss(_ptr(pred), _ptr(target), per, B, gs, _ptr(ws["sample_err"]),
                                       _ptr(ws["gout"]) if grad else None, _ptr(ws["loss"]), self._s()), "loss")
        return ws["loss"], ws["sample_err"][:B]

    def adam(self, lr, beta1=0.9, beta2=0.999, eps=1e-8, weight_decay=0.0):
        self.step_count += 1
        self._ck(self.lib.wfs_fno_adam(_ptr(self.flat), _ptr(self.grad), _ptr(self.m1), _ptr(self.m2), self.nparams,
                                       float(lr), float(beta1), float(beta2), float(eps), float(weight_decay),
                                       self.step_count, self._s()), "adam")
        self.pack()

    def train_step(self, x, prior, target, B, lr):
        pred = self.forward(x, prior, B)
        loss, _ = self.loss(pred, target, B, grad=True)
        self.backward(x, self.ws["gout"], B)
        self.adam(lr)
        return loss


# ---------------------------------------------------------------------------------------------
# Training pairs from the plain split step
# ---------------------------------------------------------------------------------------------
def harmonic_potential(N, extent, omega, mass=1.0):
    """V = 1/2 m w^2 |r|^2 with r = voxel * dx - L / 2 (sources/potential.py:414-423), complex64."""
    dx = extent / N
    r = np.arange(N) * dx - 0.5 * extent
    r2 = r[:, None, None] ** 2 + r[None, :, None] ** 2 + r[None, None, :] ** 2
    return (0.5 * mass * omega ** 2 * r2).astype(np.complex64)


@dataclass
class Scenario:
    kind: str          # "wall", "ho" or "free"
    strength: float    # barrier height (Hartree) or omega
    width: float       # barrier thickness (Bohr); 0 otherwise
    sigma: float
    x0: float
    k0: float


@dataclass
class ScenarioRanges:
    """Uniform ranges the scenarios are drawn from. The defaults are the barrier ranges of
    the batched sweep (height U[0.2,2] Ha, thickness U[1,4] Bohr) and harmonic oscillators
    with omega U[0.2,0.8], packets sigma U[1,3], x0 U[-12,-6], k0x U[0.5,3], half of each."""
    p_wall: float = 0.5
    p_ho: float = 0.5
    height: tuple = (0.2, 2.0)
    thickness: tuple = (1.0, 4.0)
    omega: tuple = (0.2, 0.8)
    sigma: tuple = (1.0, 3.0)
    x0: tuple = (-12.0, -6.0)
    k0: tuple = (0.5, 3.0)


def draw_scenarios(n, rng, ranges: ScenarioRanges | None = None):
    r = ranges or ScenarioRanges()
    out = []
    for _ in range(n):
        u = rng.uniform()
        if u < r.p_wall:
            kind, st, w = "wall", rng.uniform(*r.height), rng.uniform(*r.thickness)
        elif u < r.p_wall + r.p_ho:
            kind, st, w = "ho", rng.uniform(*r.omega), 0.0
        else:
            kind, st, w = "free", 0.0, 0.0
        out.append(Scenario(kind, st, w, rng.uniform(*r.sigma), rng.uniform(*r.x0), rng.uniform(*r.k0)))
    return out


class PairGenerator:
    """Generates (input, prior, target) triples with the batch engine on the given stream.

    For G scenarios at once: psi_0 = Gaussian packet, then `windows` jumps of K plain
    steps; the pair of window w is (psi_w, V) -> psi_{w+1}. prior_w is the coarse
    split step of psi_w. Inputs are normalised per sample by the RMS of psi_w (the
    propagator is linear in psi), so targets and priors are divided by it too."""

    def __init__(self, cfg: FnoConfig, group: int, device="cuda", stream=None):
        import torch

        self.torch = torch
        self.cfg = cfg
        self.G = group
        self.device = torch.device(device)
        self.stream = stream if stream is not None else torch.cuda.current_stream(self.device)
        sp = C.c_void_p(self.stream.cuda_stream)
        self.exact = _lib.Batch([cfg.N] * group, [cfg.extent] * group, stream=sp)
        self.coarse = _lib.Batch([cfg.N] * group, [cfg.extent] * group, stream=sp)
        self.builder = _lib.Engine((cfg.N,) * 3, (cfg.extent,) * 3, stream=sp)
        self.lib = _lib.load()
        c64 = dict(dtype=torch.complex64, device=self.device)
        self.V = torch.empty((group, cfg.n3), **c64)
        self.psi = torch.empty((group, cfg.n3), **c64)
        self.a2 = torch.empty(group, dtype=torch.float64, device=self.device)

    def _potential(self, sc: Scenario):
        cfg = self.cfg
        if sc.kind == "ho":
            return harmonic_potential(cfg.N, cfg.extent, sc.strength, cfg.mass)
        if sc.kind == "free":
            return np.zeros((cfg.N,) * 3, np.complex64)
        self.builder.potential_clear()
        self.builder.add_wall(sc.strength, (0.0, 0.0, 0.0), (1.0, 0.0, 0.0), sc.width)
        return self.builder.get_potential()

    def setup(self, scenarios):
        torch = self.torch
        assert len(scenarios) == self.G
        for i, sc in enumerate(scenarios):
            V = torch.from_numpy(self._potential(sc).reshape(-1)).to(self.device)
            self.V[i].copy_(V)
            self.stream.synchronize()
            self.exact.set_potential_device(i, self.V[i].data_ptr())
            self.coarse.set_potential_device(i, self.V[i].data_ptr())
            self.exact.init_gaussian(i, (sc.sigma,) * 3, (sc.x0, 0.0, 0.0), (sc.k0, 0.0, 0.0))

    def snapshot(self, out):
        for i in range(self.G):
            self.exact.get_psi_device(i, out[i].data_ptr())

    def coarse_jump(self, psi_in, out):
        """prior_steps coarse Strang steps over the jump; prior_steps = 0 is the identity."""
        cfg = self.cfg
        if cfg.prior_steps == 0:
            out.copy_(psi_in)
            return
        for i in range(self.G):
            self.coarse.set_psi_device(i, psi_in[i].data_ptr())
        T = cfg.jump_steps * cfg.dt
        self.coarse.run(cfg.prior_steps, T / cfg.prior_steps, cfg.mass, graph=False)
        for i in range(self.G):
            self.coarse.get_psi_device(i, out[i].data_ptr())

    def exact_jump(self):
        cfg = self.cfg
        self.exact.run(cfg.jump_steps, cfg.dt, cfg.mass, graph=True)

    def normalise(self, psi, x, prior, target):
        """x = input from (psi, V); prior and target divided by psi's RMS."""
        lib, s, G, n3 = self.lib, C.c_void_p(self.stream.cuda_stream), self.G, self.cfg.n3
        rc = lib.wfs_fno_sample_norms(_ptr(psi), None, n3, G, _ptr(self.a2), None, s)
        rc = rc or lib.wfs_fno_make_input(_ptr(psi), _ptr(self.V), float(self.cfg.vscale), _ptr(self.a2), _ptr(x), G,
                                          n3, s)
        for t in (prior, target):
            if t is not None:
                rc = rc or lib.wfs_fno_scale_samples(_ptr(t), _ptr(self.a2), 1, G, n3, s)
        if rc:
            raise _lib.WfsError(rc, "normalisation failed")

    def trajectories(self, scenarios, windows, x_out, prior_out, target_out, start=0):
        """Fills rows start + w * G + i of the output tensors for every window w and scenario i."""
        self.setup(scenarios)
        G = self.G
        for w in range(windows):
            rows = slice(start + w * G, start + (w + 1) * G)
            self.snapshot(self.psi)
            self.coarse_jump(self.psi, prior_out[rows])
            self.exact_jump()
            self.snapshot(target_out[rows])
            self.normalise(self.psi, x_out[rows], prior_out[rows], target_out[rows])


def make_dataset(cfg: FnoConfig, npairs, windows, group, seed, device="cuda", stream=None, gen=None,
                 ranges: ScenarioRanges | None = None):
    """npairs (a multiple of windows * group) normalised training triples on the device,
    plus the generator and the scenario of every pair (row start + w * G + i)."""
    import torch

    rng = np.random.default_rng(seed)
    gen = gen or PairGenerator(cfg, group, device, stream)
    per = windows * group
    npairs = max(per, (npairs // per) * per)
    c64 = dict(dtype=torch.complex64, device=torch.device(device))
    x = torch.empty((npairs, 2, cfg.n3), **c64)
    prior = torch.empty((npairs, cfg.n3), **c64)
    target = torch.empty((npairs, cfg.n3), **c64)
    scen = []
    for k in range(npairs // per):
        sc = draw_scenarios(group, rng, ranges)
        gen.trajectories(sc, windows, x, prior, target, start=k * per)
        scen += sc * windows
    return x, prior, target, gen, scen


def train(model: FNO, data, batch, steps, lr, warmup=50, log_every=0, time_budget=None, seed=0, step_offset=0,
          total_steps=None):
    """Adam over random mini-batches of the dataset with a linear warm-up and a cosine
    learning-rate decay over total_steps (default steps); step_offset continues one
    schedule across several datasets."""
    torch = model.torch
    x, prior, target = data
    n = x.shape[0]
    total = total_steps or steps
    g = torch.Generator(device="cpu").manual_seed(seed)
    bx = torch.empty((batch, 2, model.cfg.n3), dtype=torch.complex64, device=x.device)
    bp = torch.empty((batch, model.cfg.n3), dtype=torch.complex64, device=x.device)
    bt = torch.empty_like(bp)
    history = []
    t0 = time.perf_counter()
    done = 0
    for it in range(steps):
        idx = torch.randint(0, n, (batch,), generator=g).to(x.device)
        torch.index_select(x, 0, idx, out=bx)
        torch.index_select(prior, 0, idx, out=bp)
        torch.index_select(target, 0, idx, out=bt)
        gi = step_offset + it
        f = min(1.0, (gi + 1) / max(1, warmup)) * 0.5 * (1.0 + math.cos(math.pi * min(gi, total) / max(1, total)))
        loss = model.train_step(bx, bp, bt, batch, lr * f)
        done += 1
        if log_every and (it % log_every == 0 or it == steps - 1):
            history.append((gi, float(loss.item())))
        if time_budget is not None and time.perf_counter() - t0 > time_budget:
            break
    model.stream.synchronize()
    return {"steps": done, "seconds": time.perf_counter() - t0, "history": history, "pairs_seen": done * batch}


def evaluate(model: FNO, data, batch, fast=False):
    """Relative L2 errors of prior + network and of the prior alone against the exact
    jump, per pair (numpy arrays), on normalised data. fast: the inference kernels
    (FNO.forward_fast) instead of the training forward."""
    torch = model.torch
    x, prior, target = data
    n = x.shape[0]
    cfg = model.cfg
    lib = model.lib
    s = model._s()
    a2 = torch.empty(batch, dtype=torch.float64, device=x.device)
    d2 = torch.empty_like(a2)
    e_net, e_prior, n_net, n_t = [], [], [], []
    for k in range(0, n, batch):
        B = min(batch, n - k)
        if fast:
            pred = model.forward_fast(x[k:k + B], prior[k:k + B], B)
        else:
            pred = model.forward(x[k:k + B], prior[k:k + B], B, keep_pre=False)
        for src, dst in ((pred, e_net), (prior[k:k + B], e_prior)):
            rc = lib.wfs_fno_sample_norms(_ptr(target[k:k + B]), _ptr(src), cfg.n3, B, _ptr(a2), _ptr(d2), s)
            if rc:
                raise _lib.WfsError(rc, "sample_norms failed")
            dst.append((d2[:B] / a2[:B]).sqrt().cpu().numpy())
            if dst is e_net:
                n_t.append(a2[:B].cpu().numpy())
        rc = lib.wfs_fno_sample_norms(_ptr(pred), None, cfg.n3, B, _ptr(a2), None, s)
        if rc:
            raise _lib.WfsError(rc, "sample_norms failed")
        n_net.append(a2[:B].cpu().numpy())
    nt, nn = np.concatenate(n_t), np.concatenate(n_net)
    return {"err_net": np.concatenate(e_net), "err_prior": np.concatenate(e_prior),
            "norm_err_net": np.abs(np.sqrt(nn / nt) - 1.0)}


def _time_inference(argv=None):
    """python -m wavefunctionsimpython_gb300.fno [batch] [reps]: CUDA-event time of the inference
    pass (FNO.forward_fast) of a randomly initialised network on random inputs, in ms per sample."""
    import sys

    import torch

    args = list(sys.argv[1:] if argv is None else argv)
    B = int(args[0]) if args else 64
    reps = int(args[1]) if len(args) > 1 else 5
    cfg = FnoConfig()
    model = FNO(cfg, seed=3)
    g = torch.Generator(device="cuda").manual_seed(0)
    x = torch.randn((B, 2, cfg.n3), dtype=torch.complex64, device="cuda", generator=g)
    prior = torch.zeros((B, cfg.n3), dtype=torch.complex64, device="cuda")
    model.forward_fast(x, prior, B)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(model.stream)
    for _ in range(reps):
        model.forward_fast(x, prior, B)
    e1.record(model.stream)
    torch.cuda.synchronize()
    print(f"inference pass, batch {B}: {e0.elapsed_time(e1) / reps / B:.4f} ms per sample")


if __name__ == "__main__":
    _time_inference()
