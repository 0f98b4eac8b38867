"""FP64 NumPy oracle of the Fourier-neural-operator surrogate (test infrastructure).

This module is a checker only: the tests and the surrogate benchmark compare the
CUDA kernels (wavefunctionsimpython_gb300/csrc/fno.cu) against it. The
reference project has no learned propagator; this file restates the network the
surrogate defines (include/wfs_fno.h) in plain FP64 NumPy, with an optional
emulation of the BF16 rounding the tensor-core channel mixing applies to its
operands, and its analytic backward pass (checked against finite differences in
tests/test_fno_oracle.py).

Channel-major arrays: x [B][4][N][N][N] = (Re psi, Im psi, Re V * vscale, Im V * vscale),
hidden h [B][C][N][N][N], output [B][2][N][N][N] = (Re psi', Im psi').
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf

SQRT1_2 = 0.7071067811865476
INV_SQRT_2PI = 0.3989422804014327


def bf16_round(a):
    """Round float32 values to bfloat16 (round to nearest even) and back to float32."""
    a = np.asarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    u = (u + 0x7FFF + lsb) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def bf16_round_complex(z):
    z = np.asarray(z)
    return bf16_round(z.real.astype(np.float32)).astype(np.float64) + 1j * bf16_round(
        z.imag.astype(np.float32)).astype(np.float64)


def gelu(x):
    return 0.5 * x * (1.0 + erf(x * SQRT1_2))


def gelu_grad(x):
    return 0.5 * (1.0 + erf(x * SQRT1_2)) + x * np.exp(-0.5 * x * x) * INV_SQRT_2PI


def kept_modes(N, m):
    """(kx, ky, kz) index arrays of the kept modes in the kernels' order
    mode = (ix * 2m + iy) * m + iz, k = i for i < m else N - 2m + i (x, y), kz = iz."""
    ix, iy, iz = np.meshgrid(np.arange(2 * m), np.arange(2 * m), np.arange(m), indexing="ij")
    kx = np.where(ix < m, ix, N - 2 * m + ix).ravel()
    ky = np.where(iy < m, iy, N - 2 * m + iy).ravel()
    return kx, ky, iz.ravel()


def init_params(C, m, layers, hidden, seed=0, cin=4, cout=2, zero_last=True):
    """Parameters of the network (float32 values held in float64 arrays)."""
    rng = np.random.default_rng(seed)
    nm = 4 * m ** 3

    def lin(o, i):
        b = 1.0 / np.sqrt(i)
        return (rng.uniform(-b, b, (o, i)).astype(np.float32).astype(np.float64),
                rng.uniform(-b, b, o).astype(np.float32).astype(np.float64))

    p = {}
    p["W0"], p["b0"] = lin(C, cin)
    p["W"], p["b"], p["R"] = [], [], []
    sc = 1.0 / (C * C)
    for _ in range(layers):
        w, b = lin(C, C)
        p["W"].append(w)
        p["b"].append(b)
        r = sc * (rng.uniform(0, 1, (nm, C, C)) + 1j * rng.uniform(0, 1, (nm, C, C)))
        p["R"].append(r.astype(np.complex64).astype(np.complex128))
    p["Wq1"], p["bq1"] = lin(hidden, C)
    if zero_last:
        p["Wq2"], p["bq2"] = np.zeros((cout, hidden)), np.zeros(cout)
    else:
        p["Wq2"], p["bq2"] = lin(cout, hidden)
    return p


def _pointwise(W, b, h):
    return np.einsum("oi,bi...->bo...", W, h) + b[None, :, None, None, None]


def spectral(h, R, m, bf16=False):
    """S(h) = Re F^-1 [R . F(h) on the kept modes]; returns (S(h), Hm [nm][B][C])."""
    B, C, N = h.shape[0], h.shape[1], h.shape[2]
    kx, ky, kz = kept_modes(N, m)
    Hf = np.fft.fftn(h, axes=(2, 3, 4), norm="ortho")
    Hm = np.transpose(Hf[:, :, kx, ky, kz], (2, 0, 1))  # [nm][B][C]
    A, Rw = (bf16_round_complex(Hm), bf16_round_complex(R)) if bf16 else (Hm, R)
    Z = np.einsum("mbi,mio->mbo", A, Rw)
    Zf = np.zeros(Hf.shape, np.complex128)
    Zf[:, :, kx, ky, kz] = np.transpose(Z, (1, 2, 0))
    return np.fft.ifftn(Zf, axes=(2, 3, 4), norm="ortho").real, Hm


def spectral_adjoint(g, R, m, bf16=False):
    """Adjoint of S applied to g; returns (S^T g, G_Z [nm][B][C])."""
    B, C, N = g.shape[0], g.shape[1], g.shape[2]
    kx, ky, kz = kept_modes(N, m)
    Gf = np.fft.fftn(g, axes=(2, 3, 4), norm="ortho")
    Gz = np.transpose(Gf[:, :, kx, ky, kz], (2, 0, 1))
    A, Rw = (bf16_round_complex(Gz), bf16_round_complex(R)) if bf16 else (Gz, R)
    Gh = np.einsum("mbo,mio->mbi", A, np.conj(Rw))
    Zf = np.zeros(Gf.shape, np.complex128)
    Zf[:, :, kx, ky, kz] = np.transpose(Gh, (1, 2, 0))
    return np.fft.ifftn(Zf, axes=(2, 3, 4), norm="ortho").real, Gz


def forward(p, x, prior, m, bf16=False):
    """Network output [B][2][N][N][N] = prior + projection(...); returns (out, cache)."""
    L = len(p["W"])
    cache = {"x": x, "h": [], "pre": [], "Hm": []}
    h = _pointwise(p["W0"], p["b0"], x)
    for l in range(L):
        cache["h"].append(h)
        s, Hm = spectral(h, p["R"][l], m, bf16)
        cache["Hm"].append(Hm)
        pre = _pointwise(p["W"][l], p["b"][l], h) + s
        cache["pre"].append(pre)
        h = gelu(pre) if l < L - 1 else pre
    cache["h"].append(h)
    qpre = _pointwise(p["Wq1"], p["bq1"], h)
    q = gelu(qpre)
    cache["qpre"], cache["q"] = qpre, q
    return _pointwise(p["Wq2"], p["bq2"], q) + prior, cache


def _wgrad(g, x):
    B = g.shape[0]
    gf, xf = g.reshape(B, g.shape[1], -1), x.reshape(B, x.shape[1], -1)
    return np.einsum("bos,bis->oi", gf, xf), gf.sum(axis=(0, 2))


def backward(p, cache, gout, m, bf16=False):
    """Gradients of a loss with d loss / d out = gout, for every parameter.

    Complex weights R get dR = dL/dRe R + i dL/dIm R = sum_b conj(Hm) G_Z."""
    L = len(p["W"])
    g = {}
    g["Wq2"], g["bq2"] = _wgrad(gout, cache["q"])
    gq = np.einsum("oi,bo...->bi...", p["Wq2"], gout)
    gqpre = gq * gelu_grad(cache["qpre"])
    g["Wq1"], g["bq1"] = _wgrad(gqpre, cache["h"][L])
    gh = np.einsum("oi,bo...->bi...", p["Wq1"], gqpre)
    g["W"], g["b"], g["R"] = [None] * L, [None] * L, [None] * L
    for l in reversed(range(L)):
        gpre = gh * gelu_grad(cache["pre"][l]) if l < L - 1 else gh
        g["W"][l], g["b"][l] = _wgrad(gpre, cache["h"][l])
        gs, Gz = spectral_adjoint(gpre, p["R"][l], m, bf16)
        g["R"][l] = np.einsum("mbi,mbo->mio", np.conj(cache["Hm"][l]), Gz)
        gh = np.einsum("oi,bo...->bi...", p["W"][l], gpre) + gs
    g["W0"], g["b0"] = _wgrad(gh, cache["x"])
    return g


def relative_loss(out, target):
    """mean_b |out_b - t_b|^2 / |t_b|^2 and its gradient."""
    B = out.shape[0]
    d = (out - target).reshape(B, -1)
    t2 = (target.reshape(B, -1) ** 2).sum(axis=1)
    e = (d ** 2).sum(axis=1) / t2
    grad = (2.0 / (B * t2))[:, None] * d
    return e.mean(), e, grad.reshape(out.shape)


def make_input(psi, V, vscale):
    """x = (Re psi, Im psi, Re V * vscale, Im V * vscale) from [B][N][N][N] complex arrays."""
    return np.stack([psi.real, psi.imag, V.real * vscale, V.imag * vscale], axis=1).astype(np.float64)


def to_channels(psi):
    return np.stack([psi.real, psi.imag], axis=1)
