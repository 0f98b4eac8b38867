"""CPU oracle for the wave-function propagation hot path (TEST INFRASTRUCTURE).

This module is a NumPy restatement of WaveFunctionSimPython's propagation
path. It is the checker for the CUDA engine and the timed CPU baseline; the
product path never imports it. Only ``tests/``, ``__graft_entry__.smoke()``
and ``bench.py`` (its ``cpu_baseline`` leg and ``--impl reference`` arm) may
use it.

Every function cites the reference file:line it follows (paths relative to the
reference project root). Arithmetic is done in the reference's precision:
``np.float32``/``np.complex64`` in single mode, ``np.float64``/``np.complex128``
in double mode, with the reference's operation order where it matters. The
potential is always complex64, as in the reference
(``sources/sim_state.py:222-227``, ``sources/cuda_kernels/potential_operator.cu:7``).

Pinning: the reference stores no golden vectors and has no tests. The oracle
is pinned by the reference's own analytic known answers
(``sources/math_utils.py:237-267``: free-packet <x>(t) and sigma(t); the unit
norm of ``gaussian_wave_packet``, ``sources/cuda_kernels/common.cu:569-605``),
by the DFT identities the reference relies on (``norm="ortho"`` round trip),
and by committed fixtures under ``tests/golden/`` produced by
``tests/golden/make_golden.py``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

# sources/math_utils.py:3-6 — Hartree atomic units
H_BAR = 1.0
ELECTRON_REST_MASS = 1.0


def real_dtype(double_precision: bool):
    return np.float64 if double_precision else np.float32


def complex_dtype(double_precision: bool):
    return np.complex128 if double_precision else np.complex64


# ---------------------------------------------------------------------------
# Grid / box helpers
# ---------------------------------------------------------------------------

def delta_x(extent, n):
    """sources/sim_state.py:94 — delta_x = L / N per axis (float64)."""
    return np.asarray(extent, dtype=np.float64) / np.asarray(n, dtype=np.float64)


def observation_box_voxels(extent, n, bottom, top):
    """Observation box in voxels: sources/sim_state.py:105-161.

    Flip inverted corners, clip to the simulated volume, convert to voxel
    indices by truncation (``np.array(..., dtype=np.int32)``), then clamp the
    top voxel to N-1 and the bottom voxel to 0.
    """
    extent = np.asarray(extent, dtype=np.float64)
    n = np.asarray(n)
    b = np.array(bottom, dtype=np.float64)
    t = np.array(top, dtype=np.float64)
    for i in range(3):
        if b[i] > t[i]:
            b[i], t[i] = t[i], b[i]
    for i in range(3):
        if b[i] < -extent[i] * 0.5:
            b[i] = -extent[i] * 0.5
        if t[i] > extent[i] * 0.5:
            t[i] = extent[i] * 0.5
    dx = extent / n
    bv = np.array((b + extent * 0.5) / dx, dtype=np.int32)
    tv = np.array((t + extent * 0.5) / dx, dtype=np.int32)
    for i in range(3):
        if tv[i] >= n[i]:
            tv[i] = n[i] - 1
    for i in range(3):
        if bv[i] < 0:
            bv[i] = 0
    return b, t, bv, tv


def physical_to_voxel(pos, extent, n):
    """sources/sim_state.py:354-358 — (pos + L/2)/dx truncated to unsigned."""
    extent = np.asarray(extent, dtype=np.float64)
    dx = extent / np.asarray(n)
    return ((np.asarray(pos, dtype=np.float64) + extent * 0.5) / dx).astype(np.uint64).astype(np.int64)


def simpson_box_from_corners(bottom_bohr, top_bohr, extent, n):
    """Sample box of a volume probability: sources/measurement.py:92-116.

    Corners are flipped if inverted, converted with
    ``transform_physical_coordinate_to_voxel_3``; the top voxel gets +1
    (inclusive Simpson boundary) and an even sample count is truncated by one.
    Divergence: the count is also clipped so that the box stays inside the
    grid (the reference reads past the array there).
    """
    b = np.array(bottom_bohr, dtype=np.float64)
    t = np.array(top_bohr, dtype=np.float64)
    for i in range(3):
        if b[i] > t[i]:
            b[i], t[i] = t[i], b[i]
    bv = physical_to_voxel(b, extent, n)
    tv = physical_to_voxel(t, extent, n) + 1
    cnt = tv - bv
    n = np.asarray(n)
    for i in range(3):
        bv[i] = min(max(bv[i], 0), n[i] - 1)
        cnt[i] = min(cnt[i], n[i] - bv[i])
        if cnt[i] % 2 == 0:
            cnt[i] -= 1
        cnt[i] = max(cnt[i], 1)
    return bv.astype(np.int64), cnt.astype(np.int64)


def expected_location_box(obs_bottom_voxel, obs_top_voxel):
    """Sample box of ExpectedLocation: sources/measurement.py:318-329."""
    bv = np.array(obs_bottom_voxel, dtype=np.int64)
    tv = np.array(obs_top_voxel, dtype=np.int64) + 1
    cnt = tv - bv
    for i in range(3):
        if cnt[i] % 2 == 0:
            cnt[i] -= 1
    return bv, cnt


# ---------------------------------------------------------------------------
# Wave packet — sources/cuda_kernels/gaussian_wave_packet.cu:6-43,
#               sources/cuda_kernels/common.cu:569-605
# ---------------------------------------------------------------------------

def gaussian_wave_packet(n, dx, sigma, r0, k0, double_precision=False):
    """psi(r) = prod_d (2/(pi a_d^2))^(1/4) exp(-(r_d-r0_d)^2/a_d^2) * e^{i k0.r}.

    a = 2 sigma; r_d = dx_d * ((int)i - (int)N_d/2) (gaussian_wave_packet.cu:36-40).
    The phase uses absolute r, not r - r0 (common.cu:585).
    """
    R = real_dtype(double_precision)
    C = complex_dtype(double_precision)
    pi = R(math.pi)
    axes = []
    for d in range(3):
        i = np.arange(n[d], dtype=np.int64) - (int(n[d]) // 2)
        r = R(dx[d]) * i.astype(R)
        a = R(2.0) * R(sigma[d])
        norm = np.power(R(2.0) / pi / a / a, R(0.25))
        diff = r - R(r0[d])
        g = norm * np.exp((-diff) * diff / a / a)
        axes.append((r.astype(R), g.astype(R)))
    (rx, gx), (ry, gy), (rz, gz) = axes
    g = (gx[:, None, None] * gy[None, :, None]) * gz[None, None, :]
    phase = (R(k0[0]) * rx[:, None, None] + R(k0[1]) * ry[None, :, None]) + R(k0[2]) * rz[None, None, :]
    psi = g * (np.cos(phase) + 1j * np.sin(phase))
    return psi.astype(C)


# ---------------------------------------------------------------------------
# Potentials
# ---------------------------------------------------------------------------

def _f32(x):
    return np.float32(x)


def fma32(a, b, c):
    """Fused multiply-add in float32, correctly rounded: round(a*b + c) with one rounding.

    The reference's kernels are compiled with contraction on (NVRTC's default), so
    its compiler fuses a product into the add or subtract that consumes it. a*b is
    exact in float64; the float64 sum is corrected with an error-free transformation
    (TwoSum) where it lands exactly halfway between two float32 values.
    """
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    c = np.asarray(c, np.float32)
    p = a.astype(np.float64) * b.astype(np.float64)
    c64 = c.astype(np.float64)
    s = p + c64
    bb = s - p
    e = (p - (s - bb)) + (c64 - bb)
    r = s.astype(np.float32)
    r64 = r.astype(np.float64)
    other = np.where(s > r64, np.nextafter(r, np.float32(np.inf)), np.nextafter(r, np.float32(-np.inf)))
    mid = (r64 != s) & (np.abs(s - r64) == np.abs(other.astype(np.float64) - s)) & (e != 0)
    pick = np.where((e > 0) == (other > r), other, r)
    return np.where(mid, pick, r).astype(np.float32)


def _mul32(a, b):
    return (np.asarray(a, np.float32) * np.asarray(b, np.float32)).astype(np.float32)


def dot3_contracted(a, b):
    """a.x*b.x + a.y*b.y + a.z*b.z as the reference's compiled dot() evaluates it:
    the first product fused into the first sum, the third into the second,
    fma(a.z, b.z, fma(a.x, b.x, a.y*b.y)) (common.cu:65-68)."""
    return fma32(a[2], b[2], fma32(a[0], b[0], _mul32(a[1], b[1])))


def wall_frame(normal, slit_rotation_radian):
    """Float32 frame of a potential wall as the reference's device code computes it.

    Restates potential_wall.cu:39-45 with common.cu:70-77 (cross), :220-223
    (normalize) and :348-369 (rotate_vector), with the fused multiply-adds its
    compiler forms: in a sum or difference of two products the first product is
    fused (fma(x0, y0, +-x1*y1)); a product added to an earlier sum is fused
    into it. up = (0,1,0), or (0,1,1) when |n.up| > 0.99 (the reference sets
    up.x = 0 and up.z = 1); right = normalize(cross(n, up)) rotated by
    slit_rotation_radian around n; cos/sin of the half angle are the float32
    roundings of the exact values.

    The reference takes cosf/sinf on the device, and those are not correctly
    rounded at every argument: sinf(0.7853982f), the half angle of a pi/2 slit
    rotation, is 0.70710683 on the device against 0.70710677 correctly rounded.
    Such a one-ulp difference moves a slit edge by about 1e-7 Bohr, which changes
    only voxels that lie exactly on the edge in float32 arithmetic (a slit edge at
    |y| = 1 on a grid of spacing 0.5, for example). The engine calls the device
    functions and matches the reference's own kernels there
    (tests/test_gpu_refpath.py); tests against this oracle use geometries
    without such ties.
    """
    n = np.asarray(normal, dtype=np.float64)
    n = (n / math.sqrt(float(np.dot(n, n)))).astype(np.float32)  # sources/potential.py:180
    up = np.array([0.0, 1.0, 0.0], dtype=np.float32)
    if abs(float(dot3_contracted(n, up))) > 0.99:
        up = np.array([0.0, 1.0, 1.0], dtype=np.float32)
    c = np.array([
        fma32(n[1], up[2], -_mul32(n[2], up[1])),
        fma32(n[2], up[0], -_mul32(n[0], up[2])),
        fma32(n[0], up[1], -_mul32(n[1], up[0])),
    ], dtype=np.float32)
    ln = np.sqrt(dot3_contracted(c, c)).astype(np.float32)
    right = (c / ln).astype(np.float32)
    half = _f32(_f32(slit_rotation_radian) / _f32(2.0))
    q0 = _f32(math.cos(float(half)))
    s = _f32(math.sin(float(half)))
    q1, q2, q3 = _mul32(s, n[0]), _mul32(s, n[1]), _mul32(s, n[2])
    two = _f32(2.0)
    Q = np.zeros((3, 3), dtype=np.float32)
    Q[0, 0] = fma32(-q3, q3, fma32(-q2, q2, fma32(q0, q0, _mul32(q1, q1))))
    Q[0, 1] = _mul32(two, fma32(q1, q2, -_mul32(q0, q3)))
    Q[0, 2] = _mul32(two, fma32(q1, q3, _mul32(q0, q2)))
    Q[1, 0] = _mul32(two, fma32(q2, q1, _mul32(q0, q3)))
    Q[1, 1] = fma32(-q3, q3, fma32(q2, q2, fma32(q0, q0, -_mul32(q1, q1))))
    Q[1, 2] = _mul32(two, fma32(q2, q3, -_mul32(q0, q1)))
    Q[2, 0] = _mul32(two, fma32(q3, q1, -_mul32(q0, q2)))
    Q[2, 1] = _mul32(two, fma32(q3, q2, _mul32(q0, q1)))
    Q[2, 2] = fma32(q3, q3, fma32(-q2, q2, fma32(q0, q0, -_mul32(q1, q1))))
    rr = np.array([fma32(Q[i, 2], right[2], fma32(Q[i, 0], right[0], _mul32(Q[i, 1], right[1]))) for i in range(3)],
                  dtype=np.float32)
    return n, rr


@dataclass
class Wall:
    """Parameters of sources/potential.py:161-198 (PotentialWall)."""
    potential_hartree: float = 20.0
    center_bohr_radii_3: tuple = (0.0, 0.0, 0.0)
    normal_vector_3: tuple = (1.0, 0.0, 0.0)
    plateau_thickness_bohr_radii: float = 5.0
    slope_thickness_bohr_radii: float = 0.0
    slope_exponent: float = 1.0
    slit_count: int = 0
    slit_spacing_bohr_radii: float = 1.0
    slit_width_bohr_radii: float = 0.5
    slit_rotation_radian: float = 0.0


def add_potential_wall(V, dx, wall: Wall):
    """V += wall (real part), restating sources/cuda_kernels/potential_wall.cu:4-83.

    r = dx * (voxel - 0.5 N); d = |n.(r-c)|; dR = |right.(r-c)|; slits leave
    V untouched; plateau adds U, slope adds U*(1-(d-p/2)/s)^e. Float32
    arithmetic with the reference compiler's fused multiply-adds (the dot
    products as in ``dot3_contracted``; ``sp*1.5 -+ sw*0.5`` fuses the first
    product), which decide the voxels that lie exactly on a plateau or slit edge.
    """
    n = V.shape
    f = np.float32
    nrm, right = wall_frame(wall.normal_vector_3, wall.slit_rotation_radian)
    c = np.array(wall.center_bohr_radii_3, dtype=np.float32)
    d32 = np.array(dx, dtype=np.float32)
    coords = []
    for a in range(3):
        v = np.arange(n[a], dtype=np.float32)
        coords.append((d32[a] * (v - f(0.5) * f(n[a]))).astype(np.float32))
    shape = tuple(int(x) for x in n)
    ax = np.broadcast_to((coords[0] - c[0]).astype(np.float32)[:, None, None], shape)
    ay = np.broadcast_to((coords[1] - c[1]).astype(np.float32)[None, :, None], shape)
    az = np.broadcast_to((coords[2] - c[2]).astype(np.float32)[None, None, :], shape)
    d = np.abs(fma32(nrm[2], az, fma32(nrm[0], ax, _mul32(nrm[1], ay))))
    dR = np.abs(fma32(right[2], az, fma32(right[0], ax, _mul32(right[1], ay))))
    sw = f(wall.slit_width_bohr_radii)
    sp = f(wall.slit_spacing_bohr_radii)
    half = f(0.5)
    sc = int(wall.slit_count)
    if sc == 1:
        skip = dR < sw * half
    elif sc == 2:
        skip = (dR > (sp - sw) * half) & (dR < (sp + sw) * half)
    elif sc == 3:
        skip = (dR < sw * half) | ((dR > sp - sw * half) & (dR < sp + sw * half))
    elif sc == 4:
        skip = ((dR > (sp - sw) * half) & (dR < (sp + sw) * half)) | (
            (dR > fma32(sp, f(1.5), -_mul32(sw, half))) & (dR < fma32(sp, f(1.5), _mul32(sw, half))))
    else:
        skip = np.zeros(d.shape, dtype=bool)
    U = f(wall.potential_hartree)
    p2 = f(wall.plateau_thickness_bohr_radii) * half
    s = f(wall.slope_thickness_bohr_radii)
    add = np.zeros(d.shape, dtype=np.float32)
    plateau = d <= p2
    add[plateau] = U
    slope = (~plateau) & (d <= p2 + s)
    if np.any(slope):
        t = (f(1.0) - (d[slope] - p2) / s).astype(np.float32)
        add[slope] = U * np.power(t, f(wall.slope_exponent)).astype(np.float32)
    add[skip] = 0.0
    V += add.astype(np.complex64)
    return V


@dataclass
class Absorbing:
    """Parameters of sources/potential.py:57-106 (AbsorbingBoundaryCondition)."""
    bottom: tuple = (-25.0, -25.0, -25.0)
    top: tuple = (25.0, 25.0, 25.0)
    offset: float = 1.0
    potential_pos: tuple = (-100.0, -100.0, -100.0)
    potential_neg: tuple = (-100.0, -100.0, -100.0)
    exponent_pos: tuple = (2.0, 2.0, 2.0)
    exponent_neg: tuple = (2.0, 2.0, 2.0)


def _atan32(x):
    """float32 atan, correctly rounded (evaluated in float64)."""
    return np.arctan(np.asarray(x, np.float32).astype(np.float64)).astype(np.float32)


def _pow32(a, b):
    """float32 pow, correctly rounded (evaluated in float64)."""
    return np.power(np.asarray(a, np.float32).astype(np.float64), np.asarray(b, np.float32).astype(np.float64)).astype(
        np.float32)


def _mix(xyz, u, v):
    """common.cu:394-397 — xyz.z*v + (1-v)*(xyz.y*u + xyz.x*(1-u)), with the
    compiler's fusions: fma(z, v, (1-v)*fma(y, u, x*(1-u)))."""
    f = np.float32
    inner = fma32(xyz[1], u, _mul32(xyz[0], (f(1.0) - u)))
    return fma32(xyz[2], v, _mul32((f(1.0) - v), inner))


def absorbing_potential_imag(n, dx, ab: Absorbing):
    """Imaginary absorbing ramp, restating sources/cuda_kernels/absorbing_potential.cu:37-306.

    26 regions (8 corners, 12 edges, 6 faces) tested in the reference's order,
    first match wins; quirks kept (edges 10, 12 and 20 blend maxD with u=0).
    Returns the float32 ramp U(r) that the reference adds as V += i*U.
    Float32 arithmetic with the reference compiler's fused multiply-adds: the
    voxel position dx*v - (0.5 N) dx fuses the first product, sqrt(a*a + b*b) is
    sqrt(fma(a, a, b*b)), lengths follow ``dot3_contracted`` and blends ``_mix``.
    """
    f = np.float32
    d32 = np.array(dx, dtype=np.float32)
    N = np.array(n, dtype=np.float32)
    bottom = np.array(ab.bottom, dtype=np.float32)
    top = np.array(ab.top, dtype=np.float32)
    off = f(ab.offset)
    pp = np.array(ab.potential_pos, dtype=np.float32)
    pn = np.array(ab.potential_neg, dtype=np.float32)
    ep = np.array(ab.exponent_pos, dtype=np.float32)
    en = np.array(ab.exponent_neg, dtype=np.float32)
    box_half = ((f(0.5) * N) * d32).astype(np.float32)
    rr = []
    for a in range(3):
        v = np.arange(n[a], dtype=np.float32)
        rr.append(fma32(d32[a], v, -box_half[a]))
    rx = rr[0][:, None, None]
    ry = rr[1][None, :, None]
    rz = rr[2][None, None, :]
    shape = tuple(int(x) for x in n)
    Bx = np.broadcast_to(rx - bottom[0], shape).astype(np.float32)
    By = np.broadcast_to(ry - bottom[1], shape).astype(np.float32)
    Bz = np.broadcast_to(rz - bottom[2], shape).astype(np.float32)
    Tx = np.broadcast_to(rx - top[0], shape).astype(np.float32)
    Ty = np.broadcast_to(ry - top[1], shape).astype(np.float32)
    Tz = np.broadcast_to(rz - top[2], shape).astype(np.float32)
    zero = f(0.0)
    pi = f(math.pi)
    out = np.zeros(shape, dtype=np.float32)
    done = np.zeros(shape, dtype=bool)
    absb = np.abs(bottom)
    abst = np.abs(top)

    def L3(a, b, c):
        return np.sqrt(dot3_contracted((a, b, c), (a, b, c))).astype(np.float32)

    def ramp(mask, dist, maxD, expo, pot):
        val = _pow32(np.maximum(dist - off, zero) / maxD, expo).astype(np.float32) * pot
        out[mask] = val.astype(np.float32)

    def corner(cond, a_num, a_den, b_num, b_h1, b_h2, sel_abs, sel_e, sel_p, dvec):
        m = cond & ~done
        if not np.any(m):
            return m
        an = a_num[m]; ad = a_den[m]
        u = (_atan32(an / ad) / pi * f(2.0)).astype(np.float32)
        h1 = b_h1[m]; h2 = b_h2[m]
        v = (_atan32(b_num[m] / np.sqrt(fma32(h1, h1, _mul32(h2, h2)))) / pi * f(2.0)).astype(np.float32)
        maxd_xyz = [box_half[i] - (sel_abs[i] + off) for i in range(3)]
        maxD = _mix(maxd_xyz, u, v)
        expo = _mix(sel_e, u, v)
        pot = _mix(sel_p, u, v)
        ramp(m, L3(dvec[0][m], dvec[1][m], dvec[2][m]), maxD, expo, pot)
        done[m] = True
        return m

    # corners of the bottom plate (absorbing_potential.cu:59-106)
    corner((Bx < 0) & (By < 0) & (Bz < 0), By, Bx, -Bz, Bx, By,
           absb, en, pn, (Bx, By, Bz))
    corner((Bx < 0) & (By < 0) & (Tz > 0), By, Bx, Tz, Bx, By,
           [absb[0], absb[1], abst[2]], [en[0], en[1], ep[2]], [pn[0], pn[1], pp[2]], (Bx, By, Tz))
    corner((By < 0) & (Tx > 0) & (Tz > 0), -By, Tx, Tz, Tx, By,
           [abst[0], absb[1], abst[2]], [ep[0], en[1], ep[2]], [pp[0], pn[1], pp[2]], (Tx, By, Tz))
    corner((By < 0) & (Bz < 0) & (Tx > 0), -By, Tx, -Bz, Tx, By,
           [abst[0], absb[1], absb[2]], [ep[0], en[1], en[2]], [pp[0], pn[1], pn[2]], (Tx, By, Bz))
    # corners of the top plate (absorbing_potential.cu:108-155)
    corner((Tx > 0) & (Ty > 0) & (Tz > 0), Ty, Tx, Tz, Tx, Ty,
           abst, ep, pp, (Tx, Ty, Tz))
    corner((Bz < 0) & (Tx > 0) & (Ty > 0), Ty, Tx, -Bz, Tx, Ty,
           [abst[0], abst[1], absb[2]], [ep[0], ep[1], en[2]], [pp[0], pp[1], pn[2]], (Tx, Ty, Bz))
    corner((Bx < 0) & (Bz < 0) & (Ty > 0), Ty, -Bx, -Bz, Bx, Ty,
           [absb[0], abst[1], absb[2]], [en[0], ep[1], en[2]], [pn[0], pp[1], pn[2]], (Bx, Ty, Bz))
    corner((Bx < 0) & (Ty > 0) & (Tz > 0), Ty, -Bx, Tz, Bx, Ty,
           [absb[0], abst[1], abst[2]], [en[0], ep[1], ep[2]], [pn[0], pp[1], pp[2]], (Bx, Ty, Tz))

    def edge(cond, num, den, use_u, u_fix_maxd, u_fix_other, sel_abs, sel_off, sel_e, sel_p, dvec):
        """Edge regions: one blend angle; u_fix_* is the constant the reference passes."""
        m = cond & ~done
        if not np.any(m):
            return
        ang = (_atan32(num[m] / den[m]) / pi * f(2.0)).astype(np.float32)
        maxd_xyz = [box_half[i] - (sel_abs[i] + sel_off[i]) for i in range(3)]
        if use_u:   # blend in x/y with u = ang, v = 0
            maxD = _mix(maxd_xyz, ang, zero)
            expo = _mix(sel_e, ang, zero)
            pot = _mix(sel_p, ang, zero)
        else:       # blend with v = ang and the fixed u values used by the reference
            maxD = _mix(maxd_xyz, f(u_fix_maxd), ang)
            expo = _mix(sel_e, f(u_fix_other), ang)
            pot = _mix(sel_p, f(u_fix_other), ang)
        ramp(m, L3(dvec[0][m], dvec[1][m], dvec[2][m]), maxD, expo, pot)
        done[m] = True

    Z = np.zeros(shape, dtype=np.float32)
    z0 = f(0.0)
    # bottom edges (absorbing_potential.cu:156-196)
    edge((Bx < 0) & (By < 0) & (Bz > 0) & (Tz < 0), By, Bx, True, 0, 0,
         [absb[0], absb[1], z0], [off, off, z0], [en[0], en[1], z0], [pn[0], pn[1], z0], (Bx, By, Z))
    edge((Bx > 0) & (By < 0) & (Tx < 0) & (Tz > 0), Tz, -By, False, 0.0, 1.0,
         [z0, absb[1], abst[2]], [z0, off, off], [z0, en[1], ep[2]], [z0, pn[1], pp[2]], (Z, By, Tz))
    edge((By < 0) & (Bz > 0) & (Tx > 0) & (Tz < 0), -By, Tx, True, 0, 0,
         [abst[0], absb[1], z0], [off, off, z0], [ep[0], en[1], z0], [pp[0], pn[1], z0], (Tx, By, Z))
    edge((Bx > 0) & (By < 0) & (Bz < 0) & (Tx < 0), Bz, By, False, 0.0, 1.0,
         [z0, absb[1], absb[2]], [z0, off, off], [z0, en[1], en[2]], [z0, pn[1], pn[2]], (Z, By, Bz))
    # pillar edges (absorbing_potential.cu:197-237)
    edge((Bx < 0) & (By > 0) & (Bz < 0) & (Ty < 0), Bz, Bx, False, 0.0, 0.0,
         [absb[0], z0, absb[2]], [off, z0, off], [en[0], z0, en[2]], [pn[0], z0, pn[2]], (Bx, Z, Bz))
    edge((Bx < 0) & (By > 0) & (Ty < 0) & (Tz > 0), Tz, -Bx, False, 0.0, 0.0,
         [absb[0], z0, abst[2]], [off, z0, off], [en[0], z0, ep[2]], [pn[0], z0, pp[2]], (Bx, Z, Tz))
    edge((By > 0) & (Tx > 0) & (Ty < 0) & (Tz > 0), Tz, Tx, False, 0.0, 0.0,
         [abst[0], z0, abst[2]], [off, z0, off], [ep[0], z0, ep[2]], [pp[0], z0, pp[2]], (Tx, Z, Tz))
    edge((By > 0) & (Bz < 0) & (Tx > 0) & (Ty < 0), -Bz, Tx, False, 0.0, 0.0,
         [abst[0], z0, absb[2]], [off, z0, off], [ep[0], z0, en[2]], [pp[0], z0, pn[2]], (Tx, Z, Bz))
    # top plane edges (absorbing_potential.cu:238-278)
    edge((Bx < 0) & (Bz > 0) & (Ty > 0) & (Tz < 0), Ty, -Bx, True, 0, 0,
         [absb[0], abst[1], z0], [off, off, z0], [en[0], ep[1], z0], [pn[0], pp[1], z0], (Bx, Ty, Z))
    edge((Bx > 0) & (Tx < 0) & (Ty > 0) & (Tz > 0), Tz, Ty, False, 1.0, 1.0,
         [z0, abst[1], abst[2]], [z0, off, off], [z0, ep[1], ep[2]], [z0, pp[1], pp[2]], (Z, Ty, Tz))
    edge((Bz > 0) & (Tx > 0) & (Ty > 0) & (Tz < 0), Ty, Tx, True, 0, 0,
         [abst[0], abst[1], z0], [off, off, z0], [ep[0], ep[1], z0], [pp[0], pp[1], z0], (Tx, Ty, Z))
    edge((Bx > 0) & (Bz < 0) & (Tx < 0) & (Ty > 0), -Bz, Ty, False, 0.0, 0.0,
         [z0, abst[1], absb[2]], [z0, off, off], [z0, ep[1], en[2]], [z0, pp[1], pn[2]], (Z, Ty, Bz))

    # box sides (absorbing_potential.cu:279-303)
    def side(cond, dist, maxD, expo, pot):
        m = cond & ~done
        if not np.any(m):
            return
        val = _pow32(np.maximum(dist[m] - off, zero) / maxD, expo).astype(np.float32) * pot
        out[m] = val.astype(np.float32)
        done[m] = True

    side((Bx > 0) & (By < 0) & (Bz > 0) & (Tx < 0) & (Tz < 0), -By, box_half[1] - (absb[1] + off), en[1], pn[1])
    side((Bx > 0) & (By > 0) & (Tx < 0) & (Ty < 0) & (Tz > 0), Tz, box_half[2] - (abst[2] + off), ep[2], pp[2])
    side((By > 0) & (Bz > 0) & (Tx > 0) & (Ty < 0) & (Tz < 0), Tx, box_half[0] - (abst[0] + off), ep[0], pp[0])
    side((Bx > 0) & (By > 0) & (Bz < 0) & (Tx < 0) & (Ty < 0), -Bz, box_half[2] - (absb[2] + off), en[2], pn[2])
    side((Bx < 0) & (By > 0) & (Bz > 0) & (Ty < 0) & (Tz < 0), -Bx, box_half[0] - (absb[0] + off), en[0], pn[0])
    side((Bx > 0) & (Bz > 0) & (Tx < 0) & (Ty > 0) & (Tz < 0), Ty, box_half[1] - (abst[1] + off), ep[1], pp[1])
    return out


def add_absorbing_potential(V, dx, ab: Absorbing):
    """V += i*U(r): absorbing_potential.cu:305-306."""
    V += (1j * absorbing_potential_imag(V.shape, dx, ab)).astype(np.complex64)
    return V


def harmonic_oscillator(n, dx, omega, mass=1.0):
    """V = 1/2 m w^2 |r|^2 with r = voxel*dx - L/2: sources/potential.py:414-423.

    This is how the reference enters a harmonic oscillator (as a raw
    pre-initialised potential file, sources/potential.py:47-55).
    """
    const = 0.5 * mass * omega ** 2
    out = []
    for a in range(3):
        v = np.arange(n[a], dtype=np.float64)
        out.append(v * dx[a] - dx[a] * n[a] * 0.5)
    r2 = out[0][:, None, None] ** 2 + out[1][None, :, None] ** 2 + out[2][None, None, :] ** 2
    return (const * r2).astype(np.complex64)


# ---------------------------------------------------------------------------
# Split-operator Fourier step — sources/sim_state.py:641-697
# ---------------------------------------------------------------------------

def wave_numbers(n, dx):
    """sources/sim_state.py:275-278 — 2 pi fftfreq(n, d=dx) in float64."""
    return [2.0 * np.pi * np.fft.fftfreq(int(n[a]), d=float(dx[a])) for a in range(3)]


def kinetic_phase(n, dx, dt, mass, double_precision, fraction=0.25):
    """exp(i*angle), angle = -|k|^2 * dt * fraction / m.

    kinetic_operator.cu:16-23 with fraction = 1/4 (the half kinetic step
    exp(-i k^2 dt / (4 m))). k is cast to the working precision per component.
    """
    R = real_dtype(double_precision)
    kx, ky, kz = [k.astype(R) for k in wave_numbers(n, dx)]
    k2 = (kx[:, None, None] * kx[:, None, None] + ky[None, :, None] * ky[None, :, None]) + kz[None, None, :] * kz[None, None, :]
    angle = -k2 * R(1.0) * R(dt) / R(1.0 / fraction) / R(mass)
    return (np.cos(angle) + 1j * np.sin(angle)).astype(complex_dtype(double_precision))


def potential_phase(V, dt, double_precision):
    """cexp_i(-dt*V) = e^{-i dt ReV} e^{dt ImV}: potential_operator.cu:11-15, common.cu:98-111."""
    R = real_dtype(double_precision)
    re = (-R(dt)) * V.real.astype(R)
    im = (-R(dt)) * V.imag.astype(R)
    return ((np.cos(re) + 1j * np.sin(re)) * np.exp(-im)).astype(complex_dtype(double_precision))


def split_step(psi, V, dx, dt, mass, nsteps=1, double_precision=None, fft=None):
    """nsteps of the Strang split fftn -> K/2 -> ifftn -> V -> fftn -> K/2 -> ifftn.

    Follows sources/sim_state.py:641-697 op for op (norm="ortho" transforms).
    ``fft`` may supply (fftn, ifftn) callables (e.g. scipy.fft with workers);
    the default is numpy's pocketfft.
    """
    if double_precision is None:
        double_precision = psi.dtype == np.complex128
    C = complex_dtype(double_precision)
    psi = psi.astype(C, copy=True)
    n = psi.shape
    K = kinetic_phase(n, dx, dt, mass, double_precision)
    P = potential_phase(V, dt, double_precision)
    fftn, ifftn = fft if fft is not None else (np.fft.fftn, np.fft.ifftn)
    for _ in range(nsteps):
        psi = fftn(psi, norm="ortho").astype(C, copy=False)
        psi *= K
        psi = ifftn(psi, norm="ortho").astype(C, copy=False)
        psi *= P
        psi = fftn(psi, norm="ortho").astype(C, copy=False)
        psi *= K
        psi = ifftn(psi, norm="ortho").astype(C, copy=False)
    return psi


def advect_walls(walls, velocities, dt):
    """One update of the moving walls (sources/sim_state.py:470-473): centre += v dt in
    float64, then the x centre is clamped at 0. Returns new Wall objects."""
    import dataclasses

    out = []
    for w, v in zip(walls, velocities):
        c = np.asarray(w.center_bohr_radii_3, np.float64) + np.asarray(v, np.float64) * dt
        if c[0] < 0.0:
            c[0] = 0.0
        out.append(dataclasses.replace(w, center_bohr_radii_3=tuple(float(x) for x in c)))
    return out


def rebuild_potential(n, dx, walls, absorbing):
    """generate_potential_from_walls_and_drain (sources/potential.py:508-522): V.fill(0),
    every wall added, then the absorbing ramp."""
    V = np.zeros(n, np.complex64)
    for w in walls:
        add_potential_wall(V, dx, w)
    if absorbing is not None:
        add_absorbing_potential(V, dx, absorbing)
    return V


def dynamic_split_run(psi, V, dx, dt, mass, walls, velocities, absorbing, nsteps):
    """The reference's loop in dynamic potential mode (sources/core_sim.py:19-23):
    evolve one split step with the current V, then advect the walls and rebuild V.
    FP64 propagation; returns (psi, V, walls)."""
    for _ in range(nsteps):
        psi = split_step(psi, V, dx, dt, mass, nsteps=1, double_precision=True)
        walls = advect_walls(walls, velocities, dt)
        V = rebuild_potential(V.shape, dx, walls, absorbing)
    return psi, V, walls


# ---------------------------------------------------------------------------
# Power-series (Taylor) step — sources/sim_state.py:721-752,
#                               sources/cuda_kernels/power_series_operator.cu:3-65
# ---------------------------------------------------------------------------

def _shift_clamped(s, axis, k):
    """s at index i+k along axis; out-of-range neighbours replaced by the centre value
    (power_series_operator.cu:23-46)."""
    n = s.shape[axis]
    idx = np.arange(n) + k
    valid = (idx >= 0) & (idx < n)
    src = np.where(valid, idx, np.arange(n))
    return np.take(s, src, axis=axis)


def laplacian(s, dx, stencil_order=2, reference_quirk=True):
    """Discrete Laplacian of the power-series kernel.

    stencil_order=2: the reference's 7-point stencil, summed in its order and
    divided by dx_x^2 for every axis (power_series_operator.cu:50-58;
    ``reference_quirk`` keeps the dx_x-only division).
    stencil_order=4: 4th-order central difference (-1,16,-30,16,-1)/12 per axis
    with the same centre-clamp boundary rule, each axis divided by its own
    spacing squared.
    """
    R = s.real.dtype.type
    if stencil_order == 2:
        s_n00 = _shift_clamped(s, 0, -1); s_p00 = _shift_clamped(s, 0, 1)
        s_0n0 = _shift_clamped(s, 1, -1); s_0p0 = _shift_clamped(s, 1, 1)
        s_00n = _shift_clamped(s, 2, -1); s_00p = _shift_clamped(s, 2, 1)
        acc = s_n00 + s_p00
        acc = acc + s_0n0
        acc = acc - R(6.0) * s
        acc = acc + s_0p0
        acc = acc + s_00n
        acc = acc + s_00p
        if reference_quirk:
            return acc / R(dx[0]) / R(dx[0])
        raise ValueError("2nd-order stencil is only defined in the reference's form")
    if stencil_order == 4:
        out = np.zeros_like(s)
        for a in range(3):
            m2 = _shift_clamped(s, a, -2); m1 = _shift_clamped(s, a, -1)
            p1 = _shift_clamped(s, a, 1); p2 = _shift_clamped(s, a, 2)
            t = (R(16.0) * (m1 + p1) - (m2 + p2)) - R(30.0) * s
            out = out + t * R(1.0 / (12.0 * dx[a] * dx[a]))
        return out
    raise ValueError("stencil_order must be 2 or 4")


def taylor_step(psi, V, dx, dt, mass, order=10, stencil_order=2, nsteps=1):
    """psi += sum_{n=1..p} s_n, s_n = i (dt/n) (lap(s_{n-1})/(2m) - V s_{n-1}), s_0 = psi.

    Restates sources/sim_state.py:721-752 and power_series_operator.cu:60-64.
    The series terms are kept in the wave function's precision (the reference
    reinterprets complex128 ping-pong buffers as complex64 in double mode,
    which is not reproduced).
    """
    C = psi.dtype.type
    R = psi.real.dtype.type
    psi = psi.copy()
    Vc = V.astype(C)
    for _ in range(nsteps):
        s = psi.copy()
        for n in range(1, order + 1):
            lap = laplacian(s, dx, stencil_order)
            inner = C(complex(R(1.0) / R(2.0) / R(mass), 0.0)) * lap - Vc * s
            coef = C(1j) * C(complex(R(dt) / R(n), 0.0))
            s = (coef * inner).astype(C)
            psi += s
    return psi


# ---------------------------------------------------------------------------
# Observables — volume_probability.cu:4-47, expected_location.cu:3-73,
#               common.cu:466-520 (Simpson weights)
# ---------------------------------------------------------------------------

def simpson_weights_1d(count):
    """1,4,2,4,...,4,1 for an odd sample count (common.cu:470-476)."""
    w = np.ones(count, dtype=np.float64)
    if count > 2:
        idx = np.arange(1, count - 1)
        w[1:count - 1] = np.where(idx % 2 == 0, 2.0, 4.0)
    return w


def _box_weights(count):
    wx = simpson_weights_1d(int(count[0]))
    wy = simpson_weights_1d(int(count[1]))
    wz = simpson_weights_1d(int(count[2]))
    return wx[:, None, None] * wy[None, :, None] * wz[None, None, :] / 27.0


def volume_probability(psi, dx, bottom_voxel, sample_count):
    """sum |psi|^2 * simpson * dx dy dz over the box (FP64 accumulation)."""
    b = [int(x) for x in bottom_voxel]
    c = [int(x) for x in sample_count]
    sub = psi[b[0]:b[0] + c[0], b[1]:b[1] + c[1], b[2]:b[2] + c[2]].astype(np.complex128)
    p = (sub.real ** 2 + sub.imag ** 2)
    return float(np.sum(p * _box_weights(c)) * dx[0] * dx[1] * dx[2])


def expected_location(psi, dx, bottom_voxel, sample_count):
    """(<r>, <r^2>) per axis with Simpson weights (expected_location.cu:32-72).

    r_d = dx_d * ((int)v + bottom_d - N_d/2). Not normalised by the norm,
    as in the reference. The second-pass stale shared-memory quirk
    (expected_location.cu:61-66) is not reproduced.
    """
    n = psi.shape
    b = [int(x) for x in bottom_voxel]
    c = [int(x) for x in sample_count]
    sub = psi[b[0]:b[0] + c[0], b[1]:b[1] + c[1], b[2]:b[2] + c[2]].astype(np.complex128)
    p = (sub.real ** 2 + sub.imag ** 2) * _box_weights(c) * (dx[0] * dx[1] * dx[2])
    r = []
    for a in range(3):
        v = np.arange(c[a], dtype=np.int64) + b[a] - int(n[a]) // 2
        r.append(dx[a] * v.astype(np.float64))
    pe = [
        float(np.sum(p * r[0][:, None, None])),
        float(np.sum(p * r[1][None, :, None])),
        float(np.sum(p * r[2][None, None, :])),
    ]
    pe2 = [
        float(np.sum(p * (r[0] ** 2)[:, None, None])),
        float(np.sum(p * (r[1] ** 2)[None, :, None])),
        float(np.sum(p * (r[2] ** 2)[None, None, :])),
    ]
    return np.array(pe), np.array(pe2)


def standard_deviation(er, er2):
    """sources/measurement.py:394-399 — sqrt(<r^2> - <r>^2)."""
    return np.sqrt(np.asarray(er2) - np.asarray(er) ** 2)


# ---------------------------------------------------------------------------
# Analytic known answers and time-series helpers — sources/math_utils.py
# ---------------------------------------------------------------------------

def indefinite_simpson_integral(array, dt):
    """sources/math_utils.py:199-234 (restated)."""
    array = np.asarray(array)
    n = array.size
    if n == 0:
        return np.empty(0, dtype=array.dtype)
    if n == 1:
        return np.array([0.0], dtype=array.dtype)
    if n == 2:
        return np.array([0.0, (array[0] + array[1]) / 2.0], dtype=array.dtype)
    is_even = n % 2 == 0
    odd_section = n - 1 if is_even else n
    even_section = n if is_even else n - 1
    integral = np.zeros(n, dtype=np.float64)
    integral[1] = 3.0 * (array[0] + array[1]) / 2.0
    for i in range(2, odd_section, 2):
        integral[i] = integral[i - 2] + array[i - 2] + 4.0 * array[i - 1] + array[i]
    for i in range(3, even_section, 2):
        integral[i] = integral[i - 2] + array[i - 2] + 4.0 * array[i - 1] + array[i]
    return integral * dt / 3.0


def predict_free_space_standard_deviation(delta_t, sigma0, mass, step_count):
    """sources/math_utils.py:237-251 — sigma(t) = sqrt(a^2 + 4 t^2/(m^2 a^2))/2, a = 2 sigma0."""
    a = sigma0 * 2.0
    t = np.arange(step_count, dtype=np.float64) * delta_t
    return np.sqrt(a ** 2 + 4.0 * (1.0 / mass ** 2) * t ** 2 / a ** 2) / 2.0


def predict_free_space_expected_location(delta_t, x0, velocity, step_count):
    """sources/math_utils.py:254-267 — <x>(t) = x0 + v t."""
    return x0 + np.arange(step_count, dtype=np.float64) * delta_t * velocity


# ---------------------------------------------------------------------------
# Whole-scenario helpers used by tests and the CPU baseline
# ---------------------------------------------------------------------------

@dataclass
class Scenario:
    n: tuple
    extent: tuple
    sigma: tuple
    r0: tuple
    k0: tuple
    dt: float
    mass: float = 1.0
    double_precision: bool = False
    walls: list = field(default_factory=list)
    absorbing: Absorbing | None = None
    ho_omega: float | None = None

    @property
    def dx(self):
        return delta_x(self.extent, self.n)

    def psi0(self):
        return gaussian_wave_packet(self.n, self.dx, self.sigma, self.r0, self.k0, self.double_precision)

    def potential(self):
        V = np.zeros(self.n, dtype=np.complex64)
        if self.ho_omega is not None:
            V += harmonic_oscillator(self.n, self.dx, self.ho_omega, self.mass)
        if self.absorbing is not None:
            add_absorbing_potential(V, self.dx, self.absorbing)
        for w in self.walls:
            add_potential_wall(V, self.dx, w)
        return V


def config1_barrier_64():
    """64^3 over a 60-Bohr cube, complex128, sigma 2, r0 (-10,0,0), k0 (2,0,0);
    1 Ha barrier 2 Bohr wide at x=0, dt 0.01."""
    return Scenario(n=(64, 64, 64), extent=(60.0, 60.0, 60.0), sigma=(2.0, 2.0, 2.0),
                    r0=(-10.0, 0.0, 0.0), k0=(2.0, 0.0, 0.0), dt=0.01, double_precision=True,
                    walls=[Wall(potential_hartree=1.0, plateau_thickness_bohr_radii=2.0,
                                slope_thickness_bohr_radii=0.0)])


def config2_ho_128():
    """128^3 over a 40-Bohr cube, complex64, HO omega 0.5, sigma 1.5, r0 (5,0,0), k0 0, dt 0.005."""
    return Scenario(n=(128, 128, 128), extent=(40.0, 40.0, 40.0), sigma=(1.5, 1.5, 1.5),
                    r0=(5.0, 0.0, 0.0), k0=(0.0, 0.0, 0.0), dt=0.005, ho_omega=0.5)


def config3_double_slit(n=256, extent=80.0):
    """Double slit: wall at x=0, 1 Bohr thick, 20 Ha, two 2-Bohr slits at y=+-3 along z;
    sigma 3, r0 (-20,0,0), k0 (2.5,0,0); 16-cell quadratic absorber (-50 Ha), dt 0.01."""
    dxv = extent / n
    inner = extent * 0.5 - 16 * dxv
    return Scenario(n=(n, n, n), extent=(extent,) * 3, sigma=(3.0, 3.0, 3.0),
                    r0=(-20.0, 0.0, 0.0), k0=(2.5, 0.0, 0.0), dt=0.01,
                    walls=[Wall(potential_hartree=20.0, plateau_thickness_bohr_radii=1.0,
                                slope_thickness_bohr_radii=0.0, slit_count=2,
                                slit_spacing_bohr_radii=6.0, slit_width_bohr_radii=2.0,
                                slit_rotation_radian=math.pi / 2)],
                    absorbing=Absorbing(bottom=(-inner,) * 3, top=(inner,) * 3, offset=0.0,
                                        potential_pos=(-50.0,) * 3, potential_neg=(-50.0,) * 3,
                                        exponent_pos=(2.0,) * 3, exponent_neg=(2.0,) * 3))


# ---------------------------------------------------------------------------
# Plane probability current — sources/cuda_kernels/probability_current_density.cu:11-218,
#                              sources/measurement.py:207-289
# ---------------------------------------------------------------------------

def plane_frame(normal):
    """right/up of the sampling plane (probability_current_density.cu:41-49), float32:
    prefUp = (0,1,0), or (0,0,1) when |n.y| > 0.99; right = normalize(n x prefUp);
    up = normalize(right x n)."""
    f = np.float32
    n = np.asarray(normal, dtype=np.float64)
    n = (n / math.sqrt(float(np.dot(n, n)))).astype(np.float32)
    pu = np.array([0.0, 1.0, 0.0], dtype=np.float32)
    d = f(f(f(n[0] * pu[0]) + f(n[1] * pu[1])) + f(n[2] * pu[2]))
    if abs(float(d)) > 0.99:
        pu = np.array([0.0, 0.0, 1.0], dtype=np.float32)

    def cross(a, b):
        return np.array([f(a[1] * b[2]) - f(a[2] * b[1]), f(a[2] * b[0]) - f(a[0] * b[2]),
                         f(a[0] * b[1]) - f(a[1] * b[0])], dtype=np.float32)

    def normalize(a):
        dd = f(f(f(a[0] * a[0]) + f(a[1] * a[1])) + f(a[2] * a[2]))
        return (a / np.float32(math.sqrt(float(dd)))).astype(np.float32)

    right = normalize(cross(n, pu))
    up = normalize(cross(right, n))
    return n, right, up


def plane_probability_current(psi, dx, center, normal, size, sample_count, mass=1.0):
    """Flux of the probability current through a sampled plane.

    Sample point (px, py): r = c + right*dW*(px - sx/2) + up*dH*(py - sy/2), nearest
    voxel by truncation of r/dx + N/2 (clamped to the grid here; the reference reads
    out of bounds there), 6th-order central gradient with out-of-range neighbours
    replaced by the centre, j.n = Im(conj(psi) dpsi/dn) / m, 2D Simpson over the samples.
    """
    f = np.float32
    R = psi.real.dtype.type
    n_arr = np.asarray(psi.shape)
    nrm, right, up = plane_frame(normal)
    sx, sy = int(sample_count[0]), int(sample_count[1])
    dW = R(size[0]) / R(sx - 1)
    dH = R(size[1]) / R(sy - 1)
    px = (np.arange(sx) - sx // 2).astype(np.float32)
    py = (np.arange(sy) - sy // 2).astype(np.float32)
    c = np.asarray(center, dtype=np.float32)
    r = np.empty((sx, sy, 3), dtype=np.float32)
    for k in range(3):
        # center + (right*dW)*px + (up*dH)*py, each product rounded (probability_current_density.cu:56-57)
        a = (f(right[k] * f(dW)) * px).astype(np.float32)
        b = (f(up[k] * f(dH)) * py).astype(np.float32)
        r[:, :, k] = ((c[k] + a)[:, None] + b[None, :]).astype(np.float32)
    vox = np.empty((sx, sy, 3), dtype=np.int64)
    for k in range(3):
        fv = r[:, :, k].astype(R) / R(dx[k]) + R(0.5) * R(n_arr[k])
        v = np.trunc(fv).astype(np.int64)
        vox[:, :, k] = np.clip(v, 0, n_arr[k] - 1)
    psi_c = psi.astype(np.complex128)

    def at(ix, iy, iz):
        return psi_c[ix, iy, iz]

    ix, iy, iz = vox[:, :, 0], vox[:, :, 1], vox[:, :, 2]
    centre = at(ix, iy, iz)

    def nb(axis, k):
        idx = [ix.copy(), iy.copy(), iz.copy()]
        moved = idx[axis] + k
        ok = (moved >= 0) & (moved <= n_arr[axis] - 1)
        idx[axis] = np.where(ok, moved, idx[axis])
        return at(*idx)

    grads = []
    for axis in range(3):
        g = (nb(axis, 3) - 9.0 * nb(axis, 2) + 45.0 * nb(axis, 1) - 45.0 * nb(axis, -1)
             + 9.0 * nb(axis, -2) - nb(axis, -3)) / 60.0 / float(dx[axis])
        grads.append(g)
    dpsi = float(nrm[0]) * grads[0] + float(nrm[1]) * grads[1] + float(nrm[2]) * grads[2]
    density = (np.conj(centre) * dpsi).imag / mass
    wx = simpson_weights_1d(sx)
    wy = simpson_weights_1d(sy)
    return float(np.sum(density * wx[:, None] * wy[None, :]) / 9.0 * float(dW) * float(dH)), density
