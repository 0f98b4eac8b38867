"""NumPy restatement of the headless volume renderer (test infrastructure).

This module is a checker only: tests compare the CUDA ray march
(wavefunctionsimpython_gb300/csrc/render.cu) against it. It restates, in FP64
and vectorised over pixels, the shader math of the reference's volume view:
colormaps sources/volumetric_visualization.py:49-98, volume preparation
:108-160 (colour limit 0.005, max |V|, one voxel of zero padding), gradient
sample sources/multi_volume_shaders.py:104-136 (complexCentralDifferenceGradSample,
whose z component pairs the z and x neighbours), ACES tone map :175-190 and the
main loop :200-310 with per-volume shading :335-390. The reference renders
through OpenGL, which is unavailable here, so parity with its pixels is
unpinned; the restatement is the oracle.
"""
from __future__ import annotations

import math

import numpy as np


def padded_volumes(psi, V, wave_function_scale=0.005, potential_scale=0.0):
    n = psi.shape
    vol = np.zeros((n[0] + 2, n[1] + 2, n[2] + 2, 2))
    vol[1:-1, 1:-1, 1:-1, 0] = np.clip(psi.real.astype(np.float64) / wave_function_scale, -1, 1)
    vol[1:-1, 1:-1, 1:-1, 1] = np.clip(psi.imag.astype(np.float64) / wave_function_scale, -1, 1)
    pot = None
    if V is not None:
        mx = potential_scale if potential_scale > 0 else float(np.abs(V.view(np.float32)).max())
        inv = 1.0 / mx if mx > 0 else 0.0
        pot = np.zeros_like(vol)
        pot[1:-1, 1:-1, 1:-1, 0] = np.clip(V.real.astype(np.float64) * inv, -1, 1)
        pot[1:-1, 1:-1, 1:-1, 1] = np.clip(V.imag.astype(np.float64) * inv, -1, 1)
    return vol, pot


def trilinear(vol, p):
    """vol [N0][N1][N2][C], p [P][3] as (x = axis 2, y = axis 1, z = axis 0) -> [P][C]."""
    N = vol.shape
    cx = np.clip(p[:, 0], 0, N[2] - 1)
    cy = np.clip(p[:, 1], 0, N[1] - 1)
    cz = np.clip(p[:, 2], 0, N[0] - 1)
    x0 = np.minimum(cx.astype(np.int64), N[2] - 2)
    y0 = np.minimum(cy.astype(np.int64), N[1] - 2)
    z0 = np.minimum(cz.astype(np.int64), N[0] - 2)
    fx, fy, fz = (cx - x0)[:, None], (cy - y0)[:, None], (cz - z0)[:, None]

    def g(dz, dy, dx):
        return vol[z0 + dz, y0 + dy, x0 + dx]

    x00 = g(0, 0, 0) * (1 - fx) + g(0, 0, 1) * fx
    x01 = g(0, 1, 0) * (1 - fx) + g(0, 1, 1) * fx
    x10 = g(1, 0, 0) * (1 - fx) + g(1, 0, 1) * fx
    x11 = g(1, 1, 0) * (1 - fx) + g(1, 1, 1) * fx
    return (x00 * (1 - fy) + x01 * fy) * (1 - fz) + (x10 * (1 - fy) + x11 * fy) * fz


def shade_sample(vol, p):
    N = vol.shape
    e = np.eye(3)
    s = trilinear(vol, p)
    nx, ny, nz = (trilinear(vol, p - e[k]) for k in range(3))
    px, py, pz = (trilinear(vol, p + e[k]) for k in range(3))

    def d2(a, b):
        return (a * b).sum(axis=1)

    sn = np.stack([d2(nx, nx), d2(ny, ny), d2(nz, nx)], axis=1)
    sp = np.stack([d2(px, px), d2(py, py), d2(pz, px)], axis=1)
    grad = (sp - sn) * 0.5 * np.array([N[2], N[1], N[0]], dtype=np.float64)
    return s[:, 0], s[:, 1], grad


C0 = np.array([10, 10, 255]) / 255.0
C1 = np.array([10, 255, 10]) / 255.0
C2 = np.array([255, 10, 10]) / 255.0
C3 = np.array([255, 255, 5]) / 255.0


def fire(re, im):
    p = re * re + im * im
    phase = np.arctan2(im, re) / 3.14159 * 0.5 + 0.5
    t = np.minimum((p - 0.01) * 1.0, 1.0)
    q = phase[:, None]
    c = np.where(q < 0.25, C0 * (1 - q / 0.25) + C1 * (q / 0.25),
                 np.where(q < 0.5, C1 * (1 - (q - 0.25) / 0.25) + C2 * ((q - 0.25) / 0.25),
                          np.where(q < 0.75, C2 * (1 - (q - 0.5) / 0.25) + C3 * ((q - 0.5) / 0.25),
                                   C3 * (1 - (q - 0.75) / 0.25) + C0 * ((q - 0.75) / 0.25))))
    on = t > 0
    rgb = np.where(on[:, None], c, 0.0)
    return rgb, np.where(on, t, 0.0)


def green(re):
    t = np.minimum(re - 0.001, 1.0)
    on = t > 0
    tt = np.where(on, t, 0.0)
    rgb = np.stack([tt, np.sqrt(tt), tt * tt], axis=1)
    a = np.where(on, np.maximum(0.0, tt * 1.001 - 0.001) * 0.5, 0.0)
    return np.where(on[:, None], rgb, 0.0), a


def aces(c):
    m1 = np.array([[0.59719, 0.35458, 0.04823], [0.07600, 0.90834, 0.01566], [0.02840, 0.13383, 0.83777]])
    m2 = np.array([[1.60475, -0.53108, -0.07367], [-0.10208, 1.10813, -0.00605], [-0.00327, -0.07276, 1.07602]])
    v = c @ m1.T
    a = v * (v + 0.0245786) - 0.000090537
    b = v * (0.983729 * v + 0.4329510) + 0.238081
    return np.clip((a / b) @ m2.T, 0, 1) ** (1 / 2.2)


def radiance(rgb, alpha, grad, shadow, L, view):
    gl = np.linalg.norm(grad, axis=1)
    ok = gl > 1e-6
    n = -grad / np.where(ok, gl, 1.0)[:, None]
    h = -view + L
    h = h / np.linalg.norm(h, axis=1)[:, None]
    lp = np.array([1.0, 0.976, 0.847])
    gt = np.clip(gl, 0, 1)[:, None]
    nl = np.maximum(0.0, n @ L)[:, None]
    sp = 20.0 * gt * np.maximum(0.0, (n * h).sum(axis=1))[:, None] ** 60.0
    one_s = 1.0 - shadow
    dif = lp * one_s * (30.0 * ((1 - gt) + gt * nl))
    out = alpha[:, None] * ((dif + 0.03) * rgb + lp * one_s * sp)
    return np.where(ok[:, None], out, 0.0)


def camera(npad, width, height, azimuth=0.0, elevation=45.0, fov=45.0, distance=0.0):
    c = 0.5 * (np.array([npad[2], npad[1], npad[0]], dtype=np.float64) - 1)
    half = 0.5 * fov * math.pi / 180
    rad = 0.5 * math.sqrt(sum(float(v) ** 2 for v in npad))
    dist = distance if distance > 0 else 1.05 * rad / math.sin(half)
    az, el = azimuth * math.pi / 180, elevation * math.pi / 180
    d = np.array([math.cos(el) * math.sin(az), math.sin(el), math.cos(el) * math.cos(az)])
    eye, fw = c + dist * d, -d
    rt = np.array([-fw[2], 0.0, fw[0]])
    rl = math.hypot(rt[0], rt[2])
    rt = np.array([1.0, 0.0, 0.0]) if rl < 1e-9 else rt / rl
    up = np.cross(rt, fw)
    return eye, fw, rt, up, math.tan(half), width / height


def render(psi, V=None, width=32, height=24, azimuth=0.0, elevation=45.0, fov=45.0, distance=0.0,
           relative_step=0.1, wave_function_scale=0.005, potential_scale=0.0, light=(1.0, 1.0, -1.0),
           shadow_steps=0, show_potential=True):
    """Tone-mapped RGB image [height][width][3] in [0, 1]."""
    vol, pot = padded_volumes(psi, V if show_potential else None, wave_function_scale, potential_scale)
    N = vol.shape[:3]
    eye, fw, rt, up, tanh, aspect = camera(N, width, height, azimuth, elevation, fov, distance)
    py, px = np.meshgrid(np.arange(height), np.arange(width), indexing="ij")
    u = ((2 * (px.ravel() + 0.5) / width - 1) * tanh * aspect)[:, None]
    v = ((1 - 2 * (py.ravel() + 0.5) / height) * tanh)[:, None]
    d = fw + u * rt + v * up
    d = d / np.linalg.norm(d, axis=1)[:, None]
    lo = np.full(3, -0.5)
    hi = np.array([N[2], N[1], N[0]], dtype=np.float64) - 0.5
    with np.errstate(divide="ignore", invalid="ignore"):
        ta, tb = (lo - eye) / d, (hi - eye) / d
    t0 = np.maximum(0.0, np.minimum(ta, tb).max(axis=1))
    t1 = np.maximum(ta, tb).min(axis=1)
    nsteps = np.where(t1 > t0, ((t1 - t0) / relative_step + 0.5).astype(np.int64), 0)
    h = np.where(nsteps > 0, (t1 - t0) / np.maximum(nsteps, 1), 0.0)
    stepv = d * h[:, None]
    inv_n = 1.0 / np.array([N[2], N[1], N[0]], dtype=np.float64)
    step_size = np.linalg.norm(stepv * inv_n, axis=1)
    L = np.asarray(light, dtype=np.float64)
    L = L / np.linalg.norm(L)
    Lvox = L * np.array([N[2], N[1], N[0]], dtype=np.float64)
    P = d.shape[0]
    acc_c, acc_a = np.zeros((P, 3)), np.zeros((P, 3))
    p = eye + d * t0[:, None]
    alive = nsteps > 0
    for it in range(int(nsteps.max(initial=0))):
        act = alive & (it < nsteps)
        if not act.any():
            break
        idx = np.nonzero(act)[0]
        pa = p[idx]
        shadow = np.zeros((idx.size, 3))
        if shadow_steps > 0:
            sstep = step_size[idx] * 3.0
            sp = pa + Lvox * sstep[:, None]
            disc = 1.0
            satt = 500.0 * 50.0
            for _ in range(shadow_steps):
                w = trilinear(vol, sp)
                rgb, al = fire(w[:, 0], w[:, 1])
                k = (sstep * satt * disc)[:, None]
                s = np.clip(al[:, None] * (0.5 + 0.5 * (1 - rgb)) * k, 0, 1)
                if pot is not None:
                    q = trilinear(pot, sp)
                    rgb2, al2 = green(q[:, 0])
                    s = np.clip(s + al2[:, None] * (0.5 + 0.5 * (1 - rgb2)) * k, 0, 1)
                shadow = shadow + s * (1 - shadow)
                sp = sp + Lvox * sstep[:, None]
                disc *= 0.96
                sstep = sstep * 1.0001
        re, im, grad = shade_sample(vol, pa)
        rgb, al = fire(re, im)
        col = radiance(rgb, al, grad, shadow, L, d[idx])
        ca = al.copy()
        if pot is not None:
            re2, _, grad2 = shade_sample(pot, pa)
            rgb2, al2 = green(re2)
            col2 = radiance(rgb2, al2, grad2, shadow, L, d[idx])
            take = al2 > ca
            col = np.where(take[:, None], col2, col)
            ca = np.where(take, al2, ca)
        cs = (6000.0 * step_size[idx])[:, None]
        asz = (500.0 * step_size[idx])[:, None]
        c = np.maximum(cs * col, 0.0)
        at = np.clip(asz * ca[:, None] * (0.25 + 0.75 * np.maximum(1 - col, 0.0)), 0, 1)
        acc_c[idx] += c * (1 - acc_a[idx])
        acc_a[idx] += at * (1 - acc_a[idx])
        done = (acc_a[idx] > 0.99).all(axis=1)
        acc_a[idx[done]] = 1.0
        alive[idx[done]] = False
        p[idx] = pa + stepv[idx]
    return aces(acc_c + (1 - acc_a)).reshape(height, width, 3)
