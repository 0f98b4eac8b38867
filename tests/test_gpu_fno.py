"""FNO surrogate kernels on the GPU against NumPy and the FP64 FNO oracle (GPU only)."""
import numpy as np
import pytest

from oracle import fno_oracle as fo

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no GPU")
    return t


def _lib():
    from wavefunctionsimpython_gb300 import _lib

    return _lib.load()


def ptr(t):
    import ctypes

    return ctypes.c_void_p(t.data_ptr())


def S(torch):
    import ctypes

    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def packed(torch, chans):
    """[B][C][...] real -> [B][C/2][n3] complex64 on the GPU."""
    B, Cc = chans.shape[:2]
    a = chans.reshape(B, Cc // 2, 2, -1)
    return torch.from_numpy(np.ascontiguousarray((a[:, :, 0] + 1j * a[:, :, 1]).astype(np.complex64))).cuda()


def unpacked(t, N):
    z = t.cpu().numpy()
    B, P = z.shape[:2]
    out = np.empty((B, 2 * P) + (N, N, N))
    out[:, 0::2] = z.real.reshape(B, P, N, N, N)
    out[:, 1::2] = z.imag.reshape(B, P, N, N, N)
    return out


def rel(a, b):
    return float(np.linalg.norm(np.ravel(a - b)) / np.linalg.norm(np.ravel(b)))


@pytest.mark.parametrize("N", [16, 64])
def test_fft3_matches_numpy(torch, N):
    lib = _lib()
    rng = np.random.default_rng(N)
    f = (rng.normal(size=(3, N, N, N)) + 1j * rng.normal(size=(3, N, N, N))).astype(np.complex64)
    t = torch.from_numpy(f.copy()).cuda()
    assert lib.wfs_fno_fft3(ptr(t), 3, N, -1, S(torch)) == 0
    assert rel(t.cpu().numpy(), np.fft.fftn(f, axes=(1, 2, 3), norm="ortho")) < 2e-6
    assert lib.wfs_fno_fft3(ptr(t), 3, N, 1, S(torch)) == 0
    assert rel(t.cpu().numpy(), f) < 2e-6


def test_gather_and_scatter_match_oracle(torch):
    lib = _lib()
    rng = np.random.default_rng(1)
    B, C, N, m = 3, 8, 16, 4
    h = rng.normal(size=(B, C, N, N, N))
    Y = packed(torch, h)
    assert lib.wfs_fno_fft3(ptr(Y), B * C // 2, N, -1, S(torch)) == 0
    nm = 4 * m ** 3
    Hm = torch.empty((nm, B, C), dtype=torch.complex64, device="cuda")
    assert lib.wfs_fno_gather(ptr(Y), ptr(Hm), B, C, N, m, S(torch)) == 0
    kx, ky, kz = fo.kept_modes(N, m)
    ref = np.transpose(np.fft.fftn(h, axes=(2, 3, 4), norm="ortho")[:, :, kx, ky, kz], (2, 0, 1))
    assert rel(Hm.cpu().numpy(), ref) < 2e-6
    Z = (rng.normal(size=(nm, B, C)) + 1j * rng.normal(size=(nm, B, C))).astype(np.complex64)
    Zt = torch.from_numpy(Z).cuda()
    assert lib.wfs_fno_scatter(ptr(Zt), ptr(Y), B, C, N, m, S(torch)) == 0
    assert lib.wfs_fno_fft3(ptr(Y), B * C // 2, N, 1, S(torch)) == 0
    Zf = np.zeros((B, C, N, N, N), complex)
    Zf[:, :, kx, ky, kz] = np.transpose(Z, (1, 2, 0))
    assert rel(unpacked(Y, N), np.fft.ifftn(Zf, axes=(2, 3, 4), norm="ortho").real) < 2e-6


@pytest.mark.parametrize("C,B", [(8, 19), (32, 16), (16, 5)])
def test_tensor_core_mixing_matches_bf16_oracle(torch, C, B):
    lib = _lib()
    rng = np.random.default_rng(C + B)
    nm = 4 * 3 ** 3
    X = (rng.normal(size=(nm, B, C)) + 1j * rng.normal(size=(nm, B, C))).astype(np.complex64)
    R = (rng.normal(size=(nm, C, C)) + 1j * rng.normal(size=(nm, C, C))).astype(np.complex64)
    Rf = torch.from_numpy(np.ascontiguousarray(np.stack([R.real, R.imag], -1))).cuda()
    W = torch.empty((nm, 2 * C, 2 * C), dtype=torch.bfloat16, device="cuda")
    WT = torch.empty_like(W)
    assert lib.wfs_fno_pack_weights(ptr(Rf), ptr(W), ptr(WT), C, nm, S(torch)) == 0
    Xt = torch.from_numpy(X).cuda()
    Y = torch.empty_like(Xt)
    assert lib.wfs_fno_mix(ptr(Xt), ptr(W), ptr(Y), B, C, nm, S(torch)) == 0
    A, Rb = fo.bf16_round_complex(X), fo.bf16_round_complex(R)
    assert rel(Y.cpu().numpy(), np.einsum("mbi,mio->mbo", A, Rb)) < 1e-5
    assert lib.wfs_fno_mix(ptr(Xt), ptr(WT), ptr(Y), B, C, nm, S(torch)) == 0
    assert rel(Y.cpu().numpy(), np.einsum("mbo,mio->mbi", A, np.conj(Rb))) < 1e-5


def _oracle_to_model(p):
    vals = {"W0": p["W0"], "b0": p["b0"], "Wq1": p["Wq1"], "bq1": p["bq1"], "Wq2": p["Wq2"], "bq2": p["bq2"]}
    for l in range(len(p["W"])):
        vals[f"W{l + 1}"], vals[f"b{l + 1}"], vals[f"R{l + 1}"] = p["W"][l], p["b"][l], p["R"][l]
    return vals


def test_forward_and_backward_match_oracle(torch):
    from wavefunctionsimpython_gb300.fno import FNO, FnoConfig

    N, m, Cw, L, H, B = 16, 4, 8, 3, 16, 3
    cfg = FnoConfig(N=N, width=Cw, modes=m, layers=L, hidden=H)
    p = fo.init_params(Cw, m, L, H, seed=7, zero_last=False)
    for l in range(L):
        p["R"][l] = (p["R"][l] * Cw).astype(np.complex64).astype(np.complex128)
    rng = np.random.default_rng(7)
    x = rng.normal(size=(B, 4, N, N, N)).astype(np.float32).astype(np.float64)
    prior = rng.normal(size=(B, 2, N, N, N)).astype(np.float32).astype(np.float64)
    target = rng.normal(size=(B, 2, N, N, N)).astype(np.float32).astype(np.float64)
    model = FNO(cfg, seed=0)
    model.set_params(_oracle_to_model(p))
    xt, pt, tt = packed(torch, x), packed(torch, prior)[:, 0], packed(torch, target)[:, 0]
    out = model.forward(xt, pt, B)
    ref, cache = fo.forward(p, x, prior, m, bf16=True)
    got = unpacked(out[:, None], N)
    assert rel(got, ref) < 5e-4
    loss, errs = model.loss(out, tt, B, grad_scale=1.0)
    ref_loss, ref_e, gout = fo.relative_loss(ref, target)
    assert abs(float(loss.item()) - ref_loss) <= 1e-4 * ref_loss
    model.grad.zero_()
    model.backward(xt, model.ws["gout"], B)
    g = model.get_grads()
    gr = fo.backward(p, cache, gout, m, bf16=True)
    gref = _oracle_to_model(gr)
    for name, ref_g in gref.items():
        assert rel(g[name], ref_g) < 5e-3, name


def test_inference_forward_without_pre_activations_is_identical(torch):
    """forward(keep_pre=False) skips the pre-activation stores that only backward() reads;
    the prediction must be bit-identical to the training-mode forward."""
    from wavefunctionsimpython_gb300.fno import FNO, FnoConfig

    N, m, Cw, L, H, B = 16, 4, 8, 3, 16, 2
    cfg = FnoConfig(N=N, width=Cw, modes=m, layers=L, hidden=H)
    p = fo.init_params(Cw, m, L, H, seed=11, zero_last=False)
    rng = np.random.default_rng(11)
    x = rng.normal(size=(B, 4, N, N, N)).astype(np.float32).astype(np.float64)
    prior = rng.normal(size=(B, 2, N, N, N)).astype(np.float32).astype(np.float64)
    model = FNO(cfg, seed=0)
    model.set_params(_oracle_to_model(p))
    xt, pt = packed(torch, x), packed(torch, prior)[:, 0]
    a = torch.empty((B, N ** 3), dtype=torch.complex64, device="cuda")
    b = torch.empty_like(a)
    model.forward(xt, pt, B, out=a)
    model.forward(xt, pt, B, out=b, keep_pre=False)
    torch.cuda.synchronize()
    assert torch.equal(a, b)


def test_adam_matches_formula(torch):
    lib = _lib()
    rng = np.random.default_rng(2)
    n = 1000
    p, g = rng.normal(size=n).astype(np.float32), rng.normal(size=n).astype(np.float32)
    m1, m2 = (rng.normal(size=n) ** 2 * 0.1).astype(np.float32), (rng.normal(size=n) ** 2 * 0.1).astype(np.float32)
    ts = [torch.from_numpy(a.copy()).cuda() for a in (p, g, m1, m2)]
    lr, b1, b2, eps, wd, step = 1e-3, 0.9, 0.999, 1e-8, 1e-4, 3
    assert lib.wfs_fno_adam(ptr(ts[0]), ptr(ts[1]), ptr(ts[2]), ptr(ts[3]), n, lr, b1, b2, eps, wd, step,
                            S(torch)) == 0
    a = b1 * m1 + (1 - b1) * g
    v = b2 * m2 + (1 - b2) * g * g
    ref = p - lr * ((a / (1 - b1 ** step)) / (np.sqrt(v / (1 - b2 ** step)) + eps) + wd * p)
    assert np.allclose(ts[0].cpu().numpy(), ref, rtol=1e-5, atol=1e-7)


def test_training_learns_free_propagation(torch):
    """With the identity as prior, a small network trained on free-particle pairs from the
    split step learns the 20-step propagator: held-out error drops from ~2 % to well below 1 %."""
    from wavefunctionsimpython_gb300.fno import FNO, FnoConfig, ScenarioRanges, evaluate, make_dataset, train

    cfg = FnoConfig(N=32, width=8, modes=6, layers=2, hidden=16, jump_steps=20, prior_steps=0)
    rg = ScenarioRanges(p_wall=0.0, p_ho=0.0, sigma=(2.0, 3.0), x0=(-4.0, 4.0), k0=(0.0, 0.3))
    data = make_dataset(cfg, npairs=768, windows=6, group=64, seed=1, ranges=rg)
    held = make_dataset(cfg, npairs=128, windows=2, group=64, seed=999, gen=data[3], ranges=rg)
    model = FNO(cfg, seed=0)
    info = train(model, data[:3], batch=8, steps=1000, lr=1e-3, warmup=100)
    assert info["steps"] == 1000
    ev = evaluate(model, held[:3], batch=16)
    assert np.all(np.isfinite(ev["err_net"]))
    assert ev["err_prior"].mean() > 0.01
    assert ev["err_net"].mean() < 0.25 * ev["err_prior"].mean(), (ev["err_net"].mean(), ev["err_prior"].mean())


def test_training_beats_the_coarse_prior(torch):
    """Harmonic oscillators whose packets stay inside the kept modes: the trained network
    corrects the one-step coarse split step of a 50-step jump on held-out seeds."""
    from wavefunctionsimpython_gb300.fno import FNO, FnoConfig, ScenarioRanges, evaluate, make_dataset, train

    cfg = FnoConfig(N=32, extent=24.0, width=8, modes=8, layers=2, hidden=16, jump_steps=50, prior_steps=1)
    rg = ScenarioRanges(p_wall=0.0, p_ho=1.0, omega=(0.2, 0.5), sigma=(1.5, 2.5), x0=(-2.0, -1.0), k0=(0.2, 0.6))
    data = make_dataset(cfg, npairs=768, windows=6, group=64, seed=11, ranges=rg)
    held = make_dataset(cfg, npairs=128, windows=2, group=64, seed=12345, gen=data[3], ranges=rg)
    model = FNO(cfg, seed=3)
    train(model, data[:3], batch=8, steps=1500, lr=1e-3, warmup=100)
    ev = evaluate(model, held[:3], batch=16)
    assert np.all(np.isfinite(ev["err_net"]))
    assert ev["err_net"].mean() < 0.7 * ev["err_prior"].mean(), (ev["err_net"].mean(), ev["err_prior"].mean())
