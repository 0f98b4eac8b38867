"""The surrogate's inference kernels (csrc/fno_fast.cu) reorganise the spectral layer; this
checks, in float64 on the CPU, that their order of operations is the layer the network
defines (include/wfs_fno.h, oracle/fno_oracle.spectral):

  real z-DFT of each channel onto kz < m  ->  DFT along y onto the 2m kept ky
  ->  DFT along x onto the 2m kept kx  ->  per-mode mixing Z = H R
  ->  inverse x and y DFTs from the kept modes  ->  Re of the inverse z-DFT from kz < m

with every DFT unitary (1/sqrt(N) per axis). The GPU kernels do the same in BF16 with FP32
accumulation (tests/test_gpu_fno_fast.py checks them against a BF16 restatement)."""
import numpy as np

from oracle import fno_oracle as fo


def kept_index(N, m):
    i = np.arange(2 * m)
    return np.where(i < m, i, N - 2 * m + i)


def kept_mode_spectral(h, R, m):
    B, C, N = h.shape[0], h.shape[1], h.shape[2]
    s = 1.0 / np.sqrt(N)
    n = np.arange(N)
    Ez = np.exp(-2j * np.pi * np.outer(n, np.arange(m)) / N) * s          # [z][kz]
    Ek = np.exp(-2j * np.pi * np.outer(n, kept_index(N, m)) / N) * s      # [y or x][k']
    Yz = np.einsum("bcxyz,zk->bcxyk", h, Ez)
    Yy = np.einsum("bcxyk,yj->bcxjk", Yz, Ek)
    Yx = np.einsum("bcxjk,xi->bcijk", Yy, Ek)                             # [b][c][kx'][ky'][kz]
    H = Yx.transpose(2, 3, 4, 0, 1).reshape(-1, B, C)                     # mode = (ix 2m + iy) m + iz
    Z = np.einsum("mbi,mio->mbo", H, R)
    Zc = Z.reshape(2 * m, 2 * m, m, B, C).transpose(3, 4, 0, 1, 2)        # [b][o][kx'][ky'][kz]
    Wx = np.einsum("boijk,xi->boxjk", Zc, Ek.conj())
    Wy = np.einsum("boxjk,yj->boxyk", Wx, Ek.conj())
    return np.einsum("boxyk,zk->boxyz", Wy, Ez.conj()).real


def test_kept_mode_order_is_the_spectral_layer():
    rng = np.random.default_rng(3)
    B, C, N, m = 2, 4, 16, 3
    h = rng.normal(size=(B, C, N, N, N))
    nm = 4 * m ** 3
    R = rng.normal(size=(nm, C, C)) + 1j * rng.normal(size=(nm, C, C))
    ref, _ = fo.spectral(h, R, m)
    got = kept_mode_spectral(h, R, m)
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-12


def test_kept_mode_order_at_the_network_geometry():
    """N = 64, m = 12 (the inference kernels' geometry), two channels."""
    rng = np.random.default_rng(4)
    B, C, N, m = 1, 2, 64, 12
    h = rng.normal(size=(B, C, N, N, N))
    nm = 4 * m ** 3
    R = (rng.normal(size=(nm, C, C)) + 1j * rng.normal(size=(nm, C, C))) / C
    ref, _ = fo.spectral(h, R, m)
    got = kept_mode_spectral(h, R, m)
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-12
