"""Inference kernels of the FNO surrogate (csrc/fno_fast.cu) on the GPU (GPU only).

Each stage is checked against a NumPy restatement of the same arithmetic: the BF16
DFT constants, BF16 operands and the BF16 rounding of every stored intermediate,
accumulated in float64 here and in FP32 on the tensor cores; so a wrong index or
layout shows as an O(1) error while rounding order stays at the BF16 level. The whole
pass is then checked against the training forward (FP32 FFTs and activations).
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N, C, M, K = 64, 32, 12, 24


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no GPU")
    return t


def lib():
    from wavefunctionsimpython_gb300 import _lib

    return _lib.load()


def ptr(t):
    import ctypes

    return ctypes.c_void_p(t.data_ptr())


def stream(torch):
    import ctypes

    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def bf16(a):
    """Round to the nearest BF16 (ties to even), as float64."""
    f = np.asarray(a, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def kept(i):
    return i if i < M else i + N - K


def tables():
    """tz[z][j] (64 x 24), F[k][j] (128 x 48) and G[k][j] (48 x 128) as the kernels hold them."""
    s = 1.0 / math.sqrt(N)
    z = np.arange(N)
    th = 2 * np.pi * ((np.arange(M)[None, :] * z[:, None]) % N) / N
    tz = np.empty((N, 2 * M))
    tz[:, 0::2] = bf16(np.cos(th) * s)
    tz[:, 1::2] = bf16(-np.sin(th) * s)
    kk = np.array([kept(i) for i in range(K)])
    th = 2 * np.pi * ((kk[None, :] * z[:, None]) % N) / N   # [n][k']
    c, sn = np.cos(th) * s, np.sin(th) * s
    F = np.empty((2 * N, 2 * K))
    F[0::2, 0::2], F[1::2, 0::2], F[0::2, 1::2], F[1::2, 1::2] = bf16(c), bf16(sn), bf16(-sn), bf16(c)
    G = np.empty((2 * K, 2 * N))
    G[0::2, 0::2], G[1::2, 0::2], G[0::2, 1::2], G[1::2, 1::2] = bf16(c.T), bf16(-sn.T), bf16(sn.T), bf16(c.T)
    return tz, F, G


def rand_words(torch, shape, rng, scale=1.0):
    """Random BF16 pairs on the GPU (int32 words) and the same values in float64 [..., 2]."""
    v = bf16(rng.normal(size=tuple(shape) + (2,)) * scale)
    t = torch.from_numpy(v.astype(np.float32)).to(torch.bfloat16).cuda().contiguous().view(torch.int32)
    return t.reshape(shape), v


def words(t):
    """int32 words on the GPU -> float64 [..., 2] (low half first)."""
    import torch

    a = t.contiguous().cpu().view(torch.bfloat16).float().numpy().astype(np.float64)
    return a.reshape(tuple(t.shape) + (2,))


def rel(a, b):
    return float(np.linalg.norm(np.ravel(a - b)) / np.linalg.norm(np.ravel(b)))


def gelu(x):
    from scipy.special import erf

    return 0.5 * x * (1.0 + erf(x / math.sqrt(2.0)))


BF16_TOL = 3e-3   # relative L2 of a BF16-stored result against the float64 restatement


def test_y_dft_forward_and_inverse(torch):
    _, F, G = tables()
    rng = np.random.default_rng(1)
    B = 3
    sz, v = rand_words(torch, (B, C, N, N, M), rng)
    sy = torch.zeros((K, M, B, C, N), dtype=torch.int32, device="cuda")
    assert lib().wfs_fno_fast_ydft(ptr(sz), ptr(sy), -1, B, stream(torch)) == 0
    a = v.transpose(0, 1, 2, 4, 3, 5).reshape(B, C, N, M, 2 * N)          # [b][c][x][kz][2y+s]
    ref = (a @ F).reshape(B, C, N, M, K, 2).transpose(4, 3, 0, 1, 2, 5)    # [ky][kz][b][c][x][2]
    assert rel(words(sy), ref) < BF16_TOL
    sy2, v2 = rand_words(torch, (K, M, B, C, N), rng)
    out = torch.zeros_like(sz)
    assert lib().wfs_fno_fast_ydft(ptr(sy2), ptr(out), 1, B, stream(torch)) == 0
    a = v2.transpose(2, 3, 4, 1, 0, 5).reshape(B, C, N, M, 2 * K)         # [b][c][x][kz][2ky+s]
    ref = (a @ G).reshape(B, C, N, M, N, 2).transpose(0, 1, 2, 4, 3, 5)   # [b][c][x][y][kz][2]
    assert rel(words(out), ref) < BF16_TOL


@pytest.mark.parametrize("B", [3, 17])
def test_x_dft_mixing_inverse(torch, B):
    """A partial 16-sample chunk (3) and a full chunk plus one (17)."""
    _, F, G = tables()
    rng = np.random.default_rng(B)
    nm = 4 * M ** 3
    sy, v = rand_words(torch, (K, M, B, C, N), rng)
    R = (rng.uniform(-1, 1, (nm, C, C, 2)) / C).astype(np.float32)
    Wi = torch.empty((nm, 2 * C, 2 * C), dtype=torch.bfloat16, device="cuda")
    Rt = torch.from_numpy(R).cuda()
    assert lib().wfs_fno_pack_mix_interleaved(ptr(Rt), ptr(Wi), C, nm, stream(torch)) == 0
    assert lib().wfs_fno_fast_xmix(ptr(sy), ptr(Wi), B, stream(torch)) == 0
    got = words(sy)
    # restatement: forward x DFT (BF16 store), mixing per mode (BF16 store), inverse x DFT
    a = v.reshape(K, M, B, C, 2 * N)                                       # [ky][kz][b][c][2x+s]
    H = bf16(a @ F).reshape(K, M, B, C, K, 2)                              # [ky][kz][b][i][kx][2]
    Hc = H[..., 0] + 1j * H[..., 1]
    Rb = bf16(R[..., 0]) + 1j * bf16(R[..., 1])                            # [mode][i][o]
    mode = (np.arange(K)[:, None, None] * K + np.arange(K)[None, :, None]) * M + np.arange(M)[None, None, :]
    Rm = Rb[mode]                                                          # [kx][ky][kz][i][o]
    Z = np.einsum("yzbik,kyzio->yzbok", Hc, Rm)                            # [ky][kz][b][o][kx]
    Zi = np.stack([bf16(Z.real), bf16(Z.imag)], -1).reshape(K, M, B, C, 2 * K)
    ref = (Zi @ G).reshape(K, M, B, C, N, 2)
    assert rel(got, ref) < BF16_TOL


def zrow_reference(h, sz, W, b, act):
    """pre = W h + b + Re F_z^-1 (kept kz of sz) per z-row; returns h_out and its z-spectra."""
    tz, _, _ = tables()
    Bn = h.shape[0]
    s = np.einsum("zj,bcxyj->bcxyz", tz, sz.reshape(Bn, C, N, N, 2 * M))
    pre = np.einsum("oi,bixyz->boxyz", bf16(W), h) + b[None, :, None, None, None] + s
    out = bf16(gelu(pre) if act else pre)
    spec = np.einsum("bcxyz,zj->bcxyj", out, tz)
    return out, spec.reshape(Bn, C, N, N, M, 2)


def h_words(torch, rng, B):
    t, v = rand_words(torch, (B, C // 2, N ** 3), rng)
    chans = v.transpose(0, 1, 3, 2).reshape(B, C, N, N, N)                 # pair j -> channels 2j, 2j+1
    return t, chans


def test_layer_kernel(torch):
    rng = np.random.default_rng(5)
    B = 2
    h, hv = h_words(torch, rng, B)
    sz, szv = rand_words(torch, (B, C, N, N, M), rng, scale=4.0)
    W = rng.uniform(-1, 1, (C, C)) / math.sqrt(C)
    bias = rng.uniform(-0.5, 0.5, C).astype(np.float32)
    Wt = torch.from_numpy(bf16(W).astype(np.float32)).to(torch.bfloat16).cuda()
    bt = torch.from_numpy(bias).cuda()
    hout = torch.empty_like(h)
    assert lib().wfs_fno_fast_layer(ptr(h), ptr(sz), ptr(Wt), ptr(bt), ptr(hout), B, stream(torch)) == 0
    ref_h, ref_spec = zrow_reference(hv, szv, W, bias.astype(np.float64), True)
    got_h = words(hout).reshape(B, C // 2, N ** 3, 2).transpose(0, 1, 3, 2).reshape(B, C, N, N, N)
    assert rel(got_h, ref_h) < BF16_TOL
    assert rel(words(sz), ref_spec) < BF16_TOL


def test_lift_and_last_kernels(torch):
    rng = np.random.default_rng(6)
    B = 2
    x = (rng.normal(size=(B, 2, N ** 3)) + 1j * rng.normal(size=(B, 2, N ** 3))).astype(np.complex64)
    W0 = rng.uniform(-0.5, 0.5, (C, 4))
    b0 = rng.uniform(-0.5, 0.5, C).astype(np.float32)
    W0p = np.zeros((C, 16))
    W0p[:, :4] = bf16(W0)
    h = torch.empty((B, C // 2, N ** 3), dtype=torch.int32, device="cuda")
    sz = torch.empty((B, C, N, N, M), dtype=torch.int32, device="cuda")
    W0t = torch.from_numpy(W0p.astype(np.float32)).to(torch.bfloat16).cuda()
    assert lib().wfs_fno_fast_lift(ptr(torch.from_numpy(x).cuda()), ptr(W0t), ptr(torch.from_numpy(b0).cuda()),
                                   ptr(h), ptr(sz), B, stream(torch)) == 0
    xc = np.empty((B, 4, N ** 3))
    xc[:, 0::2], xc[:, 1::2] = bf16(x.real), bf16(x.imag)
    pre = np.einsum("oi,bin->bon", bf16(W0), xc) + b0[None, :, None]
    ref_h = bf16(pre).reshape(B, C, N, N, N)
    tz, _, _ = tables()
    ref_spec = np.einsum("bcxyz,zj->bcxyj", ref_h, tz).reshape(B, C, N, N, M, 2)
    got_h = words(h).reshape(B, C // 2, N ** 3, 2).transpose(0, 1, 3, 2).reshape(B, C, N, N, N)
    assert rel(got_h, ref_h) < BF16_TOL
    assert rel(words(sz), ref_spec) < BF16_TOL

    # last layer (no activation) and both projections
    hv = got_h
    szr, szv = rand_words(torch, (B, C, N, N, M), rng, scale=4.0)
    W = rng.uniform(-1, 1, (C, C)) / math.sqrt(C)
    bias = rng.uniform(-0.5, 0.5, C).astype(np.float32)
    Wq1 = rng.uniform(-1, 1, (64, C)) / math.sqrt(C)
    bq1 = rng.uniform(-0.5, 0.5, 64).astype(np.float32)
    Wq2 = rng.uniform(-1, 1, (2, 64)) / 8
    bq2 = rng.uniform(-0.1, 0.1, 2).astype(np.float32)
    Wq2p = np.zeros((8, 64))
    Wq2p[:2] = bf16(Wq2)
    prior = (rng.normal(size=(B, N ** 3)) + 1j * rng.normal(size=(B, N ** 3))).astype(np.complex64)
    out = torch.empty((B, N ** 3), dtype=torch.complex64, device="cuda")

    def bt(a, dt=torch.bfloat16):
        return torch.from_numpy(np.asarray(a, np.float32)).to(dt).cuda()

    assert lib().wfs_fno_fast_last(ptr(h), ptr(szr), ptr(bt(bf16(W))), ptr(bt(bias, torch.float32)),
                                   ptr(bt(bf16(Wq1))), ptr(bt(bq1, torch.float32)), ptr(bt(Wq2p)),
                                   ptr(bt(bq2, torch.float32)), ptr(torch.from_numpy(prior).cuda()), ptr(out), B,
                                   stream(torch)) == 0
    s = np.einsum("zj,bcxyj->bcxyz", tz, szv.reshape(B, C, N, N, 2 * M))
    hl = bf16(np.einsum("oi,bixyz->boxyz", bf16(W), hv) + bias[None, :, None, None, None] + s)
    q = bf16(gelu(np.einsum("oi,bixyz->boxyz", bf16(Wq1), hl) + bq1[None, :, None, None, None]))
    o = np.einsum("oi,bixyz->boxyz", bf16(Wq2), q) + bq2[None, :, None, None, None]
    ref = (o[:, 0] + 1j * o[:, 1]).reshape(B, -1) + prior
    got = out.cpu().numpy()
    assert rel(got - prior, ref - prior) < BF16_TOL


def test_forward_fast_matches_training_forward(torch):
    """A network with every parameter random (the last layer included): the correction of the
    inference pass against the training forward's (FP32 FFTs and activations, BF16 mixing)."""
    from wavefunctionsimpython_gb300 import fno as F

    cfg = F.FnoConfig()
    model = F.FNO(cfg, seed=3)
    rng = np.random.default_rng(9)
    vals = model.get_params()
    vals["Wq2"] = rng.uniform(-1, 1, vals["Wq2"].shape) / 8
    vals["bq2"] = rng.uniform(-0.1, 0.1, 2)
    model.set_params(vals)
    for B in (3, 17):
        x = torch.from_numpy((rng.normal(size=(B, 2, cfg.n3)) + 1j * rng.normal(size=(B, 2, cfg.n3))).astype(
            np.complex64)).cuda()
        prior = torch.from_numpy((rng.normal(size=(B, cfg.n3)) + 1j * rng.normal(size=(B, cfg.n3))).astype(
            np.complex64)).cuda()
        ref = model.forward(x, prior, B, keep_pre=False).clone()
        got = model.forward_fast(x, prior, B).clone()
        torch.cuda.synchronize()
        r = rel((got - prior).cpu().numpy(), (ref - prior).cpu().numpy())
        print(f"B={B}: correction rel L2 fast vs training forward {r:.2e}")
        assert r < 2e-2
