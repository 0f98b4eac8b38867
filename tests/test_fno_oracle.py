"""The FNO oracle's backward pass against finite differences, and the algebra the
surrogate kernels rely on, restated in NumPy (CPU only)."""
import numpy as np
import pytest

from oracle import fno_oracle as fo


def small_problem(seed=0, N=8, m=2, C=4, L=2, H=8, B=2):
    rng = np.random.default_rng(seed)
    p = fo.init_params(C, m, L, H, seed=seed, zero_last=False)
    for l in range(L):  # spectral weights large enough to matter in the check
        p["R"][l] = p["R"][l] * C
    x = rng.normal(size=(B, 4, N, N, N))
    prior = rng.normal(size=(B, 2, N, N, N))
    target = rng.normal(size=(B, 2, N, N, N))
    return p, x, prior, target, m


def loss_of(p, x, prior, target, m):
    out, _ = fo.forward(p, x, prior, m)
    return fo.relative_loss(out, target)[0]


@pytest.mark.parametrize("name,index", [
    ("W0", (1, 2)), ("b0", (3,)), ("W", (0, 2, 1)), ("b", (1, 0)), ("Wq1", (5, 1)), ("bq1", (2,)),
    ("Wq2", (1, 3)), ("bq2", (0,)), ("R", (0, 5, 1, 2)), ("R", (1, 17, 3, 0)), ("R", (1, 0, 0, 0)),
])
def test_backward_matches_finite_differences(name, index):
    p, x, prior, target, m = small_problem()
    out, cache = fo.forward(p, x, prior, m)
    _, _, gout = fo.relative_loss(out, target)
    g = fo.backward(p, cache, gout, m)

    def get(d):
        return d[name][index[0]][index[1:]] if name in ("W", "b", "R") else d[name][index]

    def bump(h, imag=False):
        q = {k: ([a.copy() for a in v] if isinstance(v, list) else v.copy()) for k, v in p.items()}
        arr = q[name][index[0]] if name in ("W", "b", "R") else q[name]
        sub = index[1:] if name in ("W", "b", "R") else index
        arr[sub] += (1j * h) if imag else h
        return loss_of(q, x, prior, target, m)

    h = 1e-6
    fd = (bump(h) - bump(-h)) / (2 * h)
    an = get(g)
    assert abs(np.real(an) - fd) <= 1e-5 * max(1.0, abs(fd))
    if name == "R":
        fdi = (bump(h, True) - bump(-h, True)) / (2 * h)
        assert abs(np.imag(an) - fdi) <= 1e-5 * max(1.0, abs(fdi))


def test_spectral_adjoint_identity():
    rng = np.random.default_rng(3)
    N, m, C, B = 8, 3, 4, 2
    R = rng.normal(size=(4 * m ** 3, C, C)) + 1j * rng.normal(size=(4 * m ** 3, C, C))
    h = rng.normal(size=(B, C, N, N, N))
    g = rng.normal(size=(B, C, N, N, N))
    Sh, _ = fo.spectral(h, R, m)
    STg, _ = fo.spectral_adjoint(g, R, m)
    assert abs((Sh * g).sum() - (h * STg).sum()) <= 1e-10 * abs((Sh * g).sum())


def test_packed_pair_gather_and_scatter_algebra():
    """Two real channels through one complex FFT: the separation the gather kernel applies,
    and the symmetrised spectrum the scatter kernel writes (csrc/fno.cu)."""
    rng = np.random.default_rng(5)
    N, m = 8, 3
    a, b = rng.normal(size=(N, N, N)), rng.normal(size=(N, N, N))
    Y = np.fft.fftn(a + 1j * b, norm="ortho")
    kx, ky, kz = fo.kept_modes(N, m)
    neg = ((-kx) % N, (-ky) % N, (-kz) % N)
    A = 0.5 * (Y[kx, ky, kz] + np.conj(Y[neg]))
    Bm = -0.5j * (Y[kx, ky, kz] - np.conj(Y[neg]))
    assert np.allclose(A, np.fft.fftn(a, norm="ortho")[kx, ky, kz])
    assert np.allclose(Bm, np.fft.fftn(b, norm="ortho")[kx, ky, kz])
    Za = rng.normal(size=kx.size) + 1j * rng.normal(size=kx.size)
    Zb = rng.normal(size=kx.size) + 1j * rng.normal(size=kx.size)
    full_a = np.zeros((N, N, N), complex)
    full_b = np.zeros((N, N, N), complex)
    full_a[kx, ky, kz], full_b[kx, ky, kz] = Za, Zb

    def sym(Z):
        return 0.5 * (Z + np.conj(Z[(-np.arange(N)) % N][:, (-np.arange(N)) % N][:, :, (-np.arange(N)) % N]))

    out = np.fft.ifftn(sym(full_a) + 1j * sym(full_b), norm="ortho")
    assert np.allclose(out.real, np.fft.ifftn(full_a, norm="ortho").real)
    assert np.allclose(out.imag, np.fft.ifftn(full_b, norm="ortho").real)
    # the scatter only writes kz in [0, m) u (N - m, N): everything else of sym() is zero
    s = sym(full_a)
    kz_all = np.arange(N)
    off = (kz_all >= m) & (kz_all <= N - m)
    assert np.all(s[:, :, off] == 0)


def test_bf16_rounding():
    vals = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 1.0 + 2 ** -7, 3.0e-5], np.float32)
    got = fo.bf16_round(vals)
    assert got[0] == 1.0
    assert got[1] == 1.0                      # tie rounds to even
    assert got[2] == np.float32(1.0 + 2 ** -6)  # tie rounds up to even
    assert got[3] == -2.5
    assert got[4] == np.float32(1.0 + 2 ** -7)
    assert abs(got[5] - 3.0e-5) <= 2 ** -8 * 3.0e-5


def test_untrained_network_returns_prior():
    p = fo.init_params(4, 2, 2, 8, seed=1, zero_last=True)
    rng = np.random.default_rng(1)
    x = rng.normal(size=(1, 4, 8, 8, 8))
    prior = rng.normal(size=(1, 2, 8, 8, 8))
    out, _ = fo.forward(p, x, prior, 2)
    assert np.array_equal(out, prior)
