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
    """The kernels' GELU: the tanh form (within 5e-4 of the erf form the network trains with)."""
    return 0.5 * x * (1.0 + np.tanh(0.7978845608 * (x + 0.044715 * x ** 3)))


def frag_cols(W):
    """Columns of each 16-column block in mma fragment order (wfs_fno_to_bf16 with frag_order)."""
    d = np.arange(W.shape[1])
    blk, t, e = d & ~15, (d & 15) >> 2, d & 3
    return W[:, blk + np.where(e < 2, 2 * t + e, 8 + 2 * t + e - 2)]


BF16_TOL = 3e-3   # relative L2 of a BF16-stored result against the float64 restatement


def y_forward(yz):
    """[B][C][X][Y][KZ][2] z-spectra -> SY [B][X][KY][KZ][C][2] (BF16-stored), as the kernels."""
    _, F, _ = tables()
    Bn = yz.shape[0]
    a = yz.transpose(0, 2, 4, 1, 3, 5).reshape(Bn, N, M, C, 2 * N)       # [b][x][kz][c][2y+s]
    return bf16(a @ F).reshape(Bn, N, M, C, K, 2).transpose(0, 1, 4, 2, 3, 5)


def y_inverse(sy):
    """SY [B][X][KY][KZ][C][2] -> z-spectra [B][C][X][Y][KZ][2] (BF16-stored)."""
    _, _, G = tables()
    Bn = sy.shape[0]
    a = sy.transpose(0, 1, 3, 4, 2, 5).reshape(Bn, N, M, C, 2 * K)       # [b][x][kz][c][2ky+s]
    return bf16(a @ G).reshape(Bn, N, M, C, N, 2).transpose(0, 3, 1, 4, 2, 5)


def z_forward(h):
    """h [B][C][X][Y][Z] -> BF16 z-spectra [B][C][X][Y][KZ][2]."""
    tz, _, _ = tables()
    return bf16(h.reshape(-1, N) @ tz).reshape(h.shape[:4] + (M, 2))


def z_inverse(zs):
    """z-spectra [B][C][X][Y][KZ][2] -> Re F_z^-1 [B][C][X][Y][Z]."""
    tz, _, _ = tables()
    return (zs.reshape(-1, 2 * M) @ tz.T).reshape(zs.shape[:4] + (N,))


def pointwise(W, h):
    """W [o][i] times h [B][i][...] (float64)."""
    Bn = h.shape[0]
    return np.matmul(W, h.reshape(Bn, h.shape[1], -1)).reshape((Bn, W.shape[0]) + h.shape[2:])


def h_words(torch, rng, B):
    t, v = rand_words(torch, (B, C // 2, N ** 3), rng)
    chans = v.transpose(0, 1, 3, 2).reshape(B, C, N, N, N)                 # pair j -> channels 2j, 2j+1
    return t, chans


def h_values(t):
    B = t.shape[0]
    return words(t).reshape(B, C // 2, N ** 3, 2).transpose(0, 1, 3, 2).reshape(B, C, N, N, N)


def bf16_tensor(torch, a):
    """Row-major BF16 copy on the GPU (NumPy's fancy indexing may return column-major arrays,
    whose strides torch.from_numpy would keep)."""
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).to(torch.bfloat16).cuda().contiguous()


def f32_tensor(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda().contiguous()


def xmix_reference(v, R, B):
    """Restatement of the x+mixing kernel: forward x DFT (BF16 store), mixing per mode (BF16
    store), inverse x DFT; v is SY as float64 [b][x][ky][kz][c][2]."""
    _, F, G = tables()
    a = v.transpose(2, 3, 0, 4, 1, 5).reshape(K, M, B, C, 2 * N)          # [ky][kz][b][c][2x+s]
    H = bf16(a @ F).reshape(K, M, B, C, K, 2)                              # [ky][kz][b][i][kx][2]
    Hc = H[..., 0] + 1j * H[..., 1]
    Rb = bf16(R[..., 0]) + 1j * bf16(R[..., 1])                            # [mode][i][o]
    mode = (np.arange(K)[:, None, None] * K + np.arange(K)[None, :, None]) * M + np.arange(M)[None, None, :]
    Z = np.einsum("yzbik,kyzio->yzbok", Hc, Rb[mode])                      # [ky][kz][b][o][kx]
    Zi = np.stack([bf16(Z.real), bf16(Z.imag)], -1).reshape(K, M, B, C, 2 * K)
    return (Zi @ G).reshape(K, M, B, C, N, 2).transpose(2, 4, 0, 1, 3, 5)  # [b][x][ky][kz][c][2]


def packed_mixing(torch, rng):
    nm = 4 * M ** 3
    R = (rng.uniform(-1, 1, (nm, C, C, 2)) / C).astype(np.float32)
    Wi = torch.empty((nm, 2 * C, 2 * C), dtype=torch.bfloat16, device="cuda")
    Rt = f32_tensor(torch, R)   # argument tensors stay referenced until the call returns
    assert lib().wfs_fno_pack_mix_interleaved(ptr(Rt), ptr(Wi), C, nm, stream(torch)) == 0
    return R, Wi


@pytest.mark.parametrize("B", [3, 17])
def test_x_dft_mixing_inverse(torch, B):
    """A partial 16-sample chunk (3) and a full chunk plus one (17)."""
    rng = np.random.default_rng(B)
    sy, v = rand_words(torch, (B, N, K, M, C), rng)
    R, Wi = packed_mixing(torch, rng)
    assert lib().wfs_fno_fast_xmix(ptr(sy), ptr(Wi), B, stream(torch)) == 0
    assert rel(words(sy), xmix_reference(v, R, B)) < BF16_TOL


def test_mixing_wait_expiry_writes_nan_and_recovers(torch):
    """With the commit-wait limit at zero every CTA gives up at once: it drains its MMAs,
    frees its tensor memory and writes NaN over its outputs. With the limit restored the
    same call is exact again (tensor memory was freed, the context is intact)."""
    rng = np.random.default_rng(12)
    B = 3
    sy, v = rand_words(torch, (B, N, K, M, C), rng)
    again = sy.clone()
    R, Wi = packed_mixing(torch, rng)
    assert lib().wfs_fno_set_wait_limit(0.0) == 0
    try:
        assert lib().wfs_fno_fast_xmix(ptr(sy), ptr(Wi), B, stream(torch)) == 0
        torch.cuda.synchronize()
    finally:
        assert lib().wfs_fno_set_wait_limit(1.0) == 0
    assert np.isnan(words(sy)).all()
    assert lib().wfs_fno_fast_xmix(ptr(again), ptr(Wi), B, stream(torch)) == 0
    assert rel(words(again), xmix_reference(v, R, B)) < BF16_TOL


def test_lift_plane_kernel(torch):
    """h0 = W0 (psi / s, V vs) + b0 and its kept spectra, from raw psi and V with a2."""
    rng = np.random.default_rng(6)
    B = 2
    psi = (rng.normal(size=(B, N ** 3)) + 1j * rng.normal(size=(B, N ** 3))).astype(np.complex64) * 3
    V = (rng.normal(size=(B, N ** 3)) + 1j * rng.normal(size=(B, N ** 3))).astype(np.complex64)
    a2 = np.array([np.sum(np.abs(psi[b].astype(np.complex128)) ** 2) for b in range(B)])
    vs = 0.25
    W0 = rng.uniform(-0.5, 0.5, (C, 4))
    b0 = rng.uniform(-0.5, 0.5, C)
    W0p = np.zeros((C, 16))
    W0p[:, :4] = bf16(W0)
    h = torch.empty((B, C // 2, N ** 3), dtype=torch.int32, device="cuda")
    sy = torch.empty((B, N, K, M, C), dtype=torch.int32, device="cuda")
    args = [torch.from_numpy(psi).cuda(), torch.from_numpy(V).cuda(), torch.from_numpy(a2).cuda(),
            bf16_tensor(torch, frag_cols(W0p)), f32_tensor(torch, b0)]
    assert lib().wfs_fno_fast_lift(ptr(args[0]), N ** 3, ptr(args[1]), N ** 3, vs, ptr(args[2]), ptr(args[3]),
                                   ptr(args[4]), ptr(h), ptr(sy), B, stream(torch)) == 0
    sb = np.sqrt(a2 / N ** 3).astype(np.float32)
    xs = np.empty((B, 4, N ** 3))
    p32 = (psi / sb[:, None].astype(np.complex64)).astype(np.complex64)
    v32 = (V * np.float32(vs)).astype(np.complex64)
    xs[:, 0], xs[:, 1], xs[:, 2], xs[:, 3] = bf16(p32.real), bf16(p32.imag), bf16(v32.real), bf16(v32.imag)
    ref_h = bf16(pointwise(bf16(W0), xs) + b0.astype(np.float32)[None, :, None]).reshape(B, C, N, N, N)
    assert rel(h_values(h), ref_h) < BF16_TOL
    assert rel(words(sy), y_forward(z_forward(ref_h))) < BF16_TOL


def test_layer_plane_kernel(torch):
    rng = np.random.default_rng(5)
    B = 2
    h, hv = h_words(torch, rng, B)
    sy, syv = rand_words(torch, (B, N, K, M, C), rng, scale=4.0)
    W = rng.uniform(-1, 1, (C, C)) / math.sqrt(C)
    bias = rng.uniform(-0.5, 0.5, C).astype(np.float32)
    hout = torch.empty_like(h)
    Wt, bt = bf16_tensor(torch, frag_cols(bf16(W))), f32_tensor(torch, bias)
    assert lib().wfs_fno_fast_layer(ptr(h), ptr(sy), ptr(Wt), ptr(bt), ptr(hout), B, stream(torch)) == 0
    pre = pointwise(bf16(W), hv) + bias[None, :, None, None, None] + z_inverse(y_inverse(syv))
    ref_h = bf16(gelu(pre))
    assert rel(h_values(hout), ref_h) < BF16_TOL
    assert rel(words(sy), y_forward(z_forward(ref_h))) < BF16_TOL


def test_last_plane_kernel(torch):
    rng = np.random.default_rng(7)
    B = 2
    h, hv = h_words(torch, rng, B)
    sy, syv = rand_words(torch, (B, N, K, M, C), rng, scale=4.0)
    W = rng.uniform(-1, 1, (C, C)) / math.sqrt(C)
    bias = rng.uniform(-0.5, 0.5, C).astype(np.float32)
    Wq1 = rng.uniform(-1, 1, (64, C)) / math.sqrt(C)
    bq1 = rng.uniform(-0.5, 0.5, 64).astype(np.float32)
    Wq2 = rng.uniform(-1, 1, (2, 64)) / 8
    bq2 = rng.uniform(-0.1, 0.1, 2).astype(np.float32)
    Wq2p = np.zeros((8, 64))
    Wq2p[:2] = bf16(Wq2)
    prior = (rng.normal(size=(B, N ** 3)) + 1j * rng.normal(size=(B, N ** 3))).astype(np.complex64)
    a2 = np.array([2.0e5, 7.0e4])
    out = torch.empty((B, N ** 3), dtype=torch.complex64, device="cuda")
    onorm = torch.zeros(B, dtype=torch.float64, device="cuda")
    args = [bf16_tensor(torch, frag_cols(bf16(W))), f32_tensor(torch, bias), bf16_tensor(torch, frag_cols(bf16(Wq1))),
            f32_tensor(torch, bq1), bf16_tensor(torch, frag_cols(Wq2p)), f32_tensor(torch, bq2),
            torch.from_numpy(prior).cuda(), torch.from_numpy(a2).cuda()]
    assert lib().wfs_fno_fast_last(ptr(h), ptr(sy), *[ptr(t) for t in args[:7]], ptr(args[7]), ptr(out), ptr(onorm), B,
                                   stream(torch)) == 0
    hl = bf16(pointwise(bf16(W), hv) + bias[None, :, None, None, None] + z_inverse(y_inverse(syv)))
    q = bf16(gelu(pointwise(bf16(Wq1), hl) + bq1[None, :, None, None, None]))
    o = pointwise(bf16(Wq2), q) + bq2[None, :, None, None, None]
    sb = np.sqrt(a2 / N ** 3)
    ref = prior + sb[:, None] * (o[:, 0] + 1j * o[:, 1]).reshape(B, -1)
    got = out.cpu().numpy()
    assert rel(got - prior, ref - prior) < BF16_TOL
    np.testing.assert_allclose(onorm.cpu().numpy(), np.sum(np.abs(got.astype(np.complex128)) ** 2, axis=1), rtol=1e-5)


def test_forward_fast_matches_training_forward(torch):
    """A network with every parameter random (the last layer included): the correction of the
    inference pass against the training forward's (FP32 FFTs and activations, BF16 mixing),
    and the raw-field jump against the normalised pass."""
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
    # raw fields: psi = s x_0, V = x_1 / vscale, prior_raw = s prior -> out_raw = s out
    B = 3
    s = torch.tensor([2.0, 0.5, 3.0], dtype=torch.float64, device="cuda")
    a2 = s ** 2 * cfg.n3
    psi = (x[:B, 0] * s[:, None].float()).contiguous()
    V = (x[:B, 1] / cfg.vscale).contiguous()
    praw = (prior[:B] * s[:, None].float()).contiguous()
    onorm = torch.zeros(B, dtype=torch.float64, device="cuda")
    got_raw = model.jump_fast(psi, V, praw, a2, B, out_norm=onorm).clone()
    got = model.forward_fast(x[:B].contiguous(), prior[:B].contiguous(), B).clone()
    torch.cuda.synchronize()
    p = prior[:B].cpu().numpy()
    r = rel((got_raw / s[:, None].float()).cpu().numpy() - p, got.cpu().numpy() - p)
    assert r < 5e-3
    np.testing.assert_allclose(onorm.cpu().numpy(), (got_raw.abs() ** 2).sum(1).double().cpu().numpy(), rtol=1e-5)
