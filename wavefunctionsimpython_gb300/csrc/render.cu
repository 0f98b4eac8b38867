// render.cu — headless volumetric ray march of psi (and V) into an image buffer.
//
// Restates the emission-absorption shader of the reference's volume view
// (sources/multi_volume_shaders.py:200-310 main loop, :335-390 per-volume
// shading; colormaps sources/volumetric_visualization.py:49-104; volume
// preparation :108-160) as a CUDA kernel with one thread per pixel:
//   * psi is normalised to [-1, 1] by the colour limit (0.005 in the reference)
//     and V by max |V| over its real and imaginary parts, both kept complex and padded by one
//     zero voxel like the reference's textures;
//   * rays of a turntable perspective camera march the padded box with the
//     relative step (0.1 voxel); each step samples both volumes trilinearly
//     (exact FP32 weights), shades them with the density gradient (central
//     differences, including the reference's z component NZ.NX), an optional
//     shadow march towards the light, and keeps the volume with the larger
//     opacity;
//   * colour and per-channel attenuation accumulate front to back with early
//     termination at 0.99; the result is tone mapped with the ACES fit the
//     shader uses (Hill's RRT+ODT approximation) over a white background.
// The math runs in FP32; the output is RGBA8 or RGBA float32.
#include <stdint.h>

#include <cmath>

#include "../../include/wfs.h"
#include "kernels.h"

namespace wfs {
namespace {

struct V3 {
    float x, y, z;
};
__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ V3 mulv(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float dot3(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 normalize3(V3 a) {
    const float l = sqrtf(dot3(a, a));
    return l > 0.f ? a * (1.f / l) : a;
}
__device__ __forceinline__ float clamp01(float v) { return fminf(fmaxf(v, 0.f), 1.f); }

// Trilinear sample of a padded [N0][N1][N2] volume at voxel coordinates (x = axis 2,
// y = axis 1, z = axis 0), clamped to the edge like a clamp-to-edge texture.
template <int C>
__device__ __forceinline__ void trilinear(const float* __restrict__ vol, const int* N, V3 p, float (&out)[C]) {
    const float cx = fminf(fmaxf(p.x, 0.f), float(N[2] - 1));
    const float cy = fminf(fmaxf(p.y, 0.f), float(N[1] - 1));
    const float cz = fminf(fmaxf(p.z, 0.f), float(N[0] - 1));
    const int x0 = min(int(cx), N[2] - 2), y0 = min(int(cy), N[1] - 2), z0 = min(int(cz), N[0] - 2);
    const float fx = cx - float(x0), fy = cy - float(y0), fz = cz - float(z0);
    const int64_t sy = N[2], sz = int64_t(N[1]) * N[2];
    const float* b = vol + (int64_t(z0) * sz + int64_t(y0) * sy + x0) * C;
#pragma unroll
    for (int c = 0; c < C; ++c) {
        const float c000 = b[c], c001 = b[C + c];
        const float c010 = b[sy * C + c], c011 = b[(sy + 1) * C + c];
        const float c100 = b[sz * C + c], c101 = b[(sz + 1) * C + c];
        const float c110 = b[(sz + sy) * C + c], c111 = b[(sz + sy + 1) * C + c];
        const float x00 = c000 * (1.f - fx) + c001 * fx, x01 = c010 * (1.f - fx) + c011 * fx;
        const float x10 = c100 * (1.f - fx) + c101 * fx, x11 = c110 * (1.f - fx) + c111 * fx;
        const float y0v = x00 * (1.f - fy) + x01 * fy, y1v = x10 * (1.f - fy) + x11 * fy;
        out[c] = y0v * (1.f - fz) + y1v * fz;
    }
}

struct Sample {
    float re, im;
    V3 grad;
};

// Value and density gradient in texture units (sources/multi_volume_shaders.py
// complexCentralDifferenceGradSample: the z component pairs the z and x neighbours).
template <int C>
__device__ __forceinline__ Sample shade_sample(const float* vol, const int* N, V3 p) {
    float s[C], nx[C], ny[C], nz[C], px[C], py[C], pz[C];
    trilinear<C>(vol, N, p, s);
    trilinear<C>(vol, N, p - v3(1.f, 0.f, 0.f), nx);
    trilinear<C>(vol, N, p - v3(0.f, 1.f, 0.f), ny);
    trilinear<C>(vol, N, p - v3(0.f, 0.f, 1.f), nz);
    trilinear<C>(vol, N, p + v3(1.f, 0.f, 0.f), px);
    trilinear<C>(vol, N, p + v3(0.f, 1.f, 0.f), py);
    trilinear<C>(vol, N, p + v3(0.f, 0.f, 1.f), pz);
    auto d2 = [](const float (&a)[C], const float (&b)[C]) {
        float r = a[0] * b[0];
        if constexpr (C > 1) r += a[1] * b[1];
        return r;
    };
    Sample o;
    o.re = s[0];
    o.im = C > 1 ? s[C - 1] : 0.f;
    const V3 sn = v3(d2(nx, nx), d2(ny, ny), d2(nz, nx));
    const V3 sp = v3(d2(px, px), d2(py, py), d2(pz, px));
    o.grad = mulv(sp - sn, v3(0.5f * float(N[2]), 0.5f * float(N[1]), 0.5f * float(N[0])));
    return o;
}

struct Rgba {
    float r, g, b, a;
};

// translucent_fire (sources/volumetric_visualization.py:49-86): phase -> cyclic colour, density -> opacity
__device__ __forceinline__ Rgba fire(float re, float im) {
    const float p = re * re + im * im;
    const float phase = atan2f(im, re) / 3.14159f * 0.5f + 0.5f;
    const float t = fminf((p - 0.01f) * 1.0f, 1.0f);
    if (t <= 0.f) return Rgba{0.f, 0.f, 0.f, 0.f};
    const V3 c0 = v3(10.f, 10.f, 255.f) * (1.f / 255.f), c1 = v3(10.f, 255.f, 10.f) * (1.f / 255.f);
    const V3 c2 = v3(255.f, 10.f, 10.f) * (1.f / 255.f), c3 = v3(255.f, 255.f, 5.f) * (1.f / 255.f);
    V3 c;
    if (phase < 0.25f) c = c0 * (1.f - phase / 0.25f) + c1 * (phase / 0.25f);
    else if (phase < 0.5f) c = c1 * (1.f - (phase - 0.25f) / 0.25f) + c2 * ((phase - 0.25f) / 0.25f);
    else if (phase < 0.75f) c = c2 * (1.f - (phase - 0.5f) / 0.25f) + c3 * ((phase - 0.5f) / 0.25f);
    else c = c3 * (1.f - (phase - 0.75f) / 0.25f) + c0 * ((phase - 0.75f) / 0.25f);
    return Rgba{c.x, c.y, c.z, t};
}
// translucent_green (sources/volumetric_visualization.py:88-98): the potential's real part
__device__ __forceinline__ Rgba green(float re) {
    const float t = fminf(re - 0.001f, 1.0f);
    if (t <= 0.f) return Rgba{0.f, 0.f, 0.f, 0.f};
    return Rgba{t, sqrtf(t), t * t, fmaxf(0.f, t * 1.001f - 0.001f) * 0.5f};
}

__device__ __forceinline__ V3 aces(V3 c) {
    // column-major GLSL matrices of the shader, applied as m * c
    const V3 v = v3(0.59719f * c.x + 0.35458f * c.y + 0.04823f * c.z, 0.07600f * c.x + 0.90834f * c.y + 0.01566f * c.z,
                    0.02840f * c.x + 0.13383f * c.y + 0.83777f * c.z);
    auto num = [](float x) { return x * (x + 0.0245786f) - 0.000090537f; };
    auto den = [](float x) { return x * (0.983729f * x + 0.4329510f) + 0.238081f; };
    const V3 r = v3(num(v.x) / den(v.x), num(v.y) / den(v.y), num(v.z) / den(v.z));
    const V3 m = v3(1.60475f * r.x - 0.53108f * r.y - 0.07367f * r.z, -0.10208f * r.x + 1.10813f * r.y - 0.00605f * r.z,
                    -0.00327f * r.x - 0.07276f * r.y + 1.07602f * r.z);
    const float g = 1.f / 2.2f;
    return v3(powf(clamp01(m.x), g), powf(clamp01(m.y), g), powf(clamp01(m.z), g));
}

__device__ __forceinline__ V3 radiance(const Rgba& al, const Sample& s, V3 shadow, V3 L, V3 view) {
    const float gl = sqrtf(dot3(s.grad, s.grad));
    if (!(gl > 0.000001f)) return v3(0.f, 0.f, 0.f);
    const V3 n = s.grad * (-1.f / gl);
    const V3 h = normalize3(view * -1.f + L);
    const V3 lp = v3(1.0f, 0.976f, 0.847f);
    const float shininess = 60.f, diffuse = 30.f, specular = 20.f, ambient = 0.03f;
    const float gt = fminf(fmaxf(gl, 0.f), 1.f);
    const float nl = fmaxf(0.f, dot3(n, L));
    const float sp = specular * gt * powf(fmaxf(0.f, dot3(n, h)), shininess);
    const V3 one_s = v3(1.f - shadow.x, 1.f - shadow.y, 1.f - shadow.z);
    const V3 dif = mulv(lp, one_s) * (diffuse * ((1.f - gt) + gt * nl));
    return v3(al.a * ((dif.x + ambient) * al.r + lp.x * one_s.x * sp), al.a * ((dif.y + ambient) * al.g + lp.y * one_s.y * sp),
              al.a * ((dif.z + ambient) * al.b + lp.z * one_s.z * sp));
}

__global__ void __launch_bounds__(128) render_kernel(const float* __restrict__ psi, const float* __restrict__ pot,
                                                     RenderArgs a) {
    const int px = blockIdx.x * blockDim.x + threadIdx.x;
    const int py = blockIdx.y * blockDim.y + threadIdx.y;
    if (px >= a.width || py >= a.height) return;
    const int* N = a.npad;
    const V3 eye = v3(a.eye[0], a.eye[1], a.eye[2]);
    const V3 fw = v3(a.forward[0], a.forward[1], a.forward[2]);
    const V3 rt = v3(a.right[0], a.right[1], a.right[2]);
    const V3 up = v3(a.up[0], a.up[1], a.up[2]);
    const float u = (2.f * (float(px) + 0.5f) / float(a.width) - 1.f) * a.tan_half_fov * a.aspect;
    const float v = (1.f - 2.f * (float(py) + 0.5f) / float(a.height)) * a.tan_half_fov;
    const V3 d = normalize3(fw + rt * u + up * v);
    // slab intersection with the padded box [-0.5, N - 0.5] (x = axis 2, y = axis 1, z = axis 0)
    const float lo[3] = {-0.5f, -0.5f, -0.5f};
    const float hi[3] = {float(N[2]) - 0.5f, float(N[1]) - 0.5f, float(N[0]) - 0.5f};
    const float e[3] = {eye.x, eye.y, eye.z}, dd[3] = {d.x, d.y, d.z};
    float t0 = 0.f, t1 = 3.0e38f;
    for (int k = 0; k < 3; ++k) {
        if (fabsf(dd[k]) < 1e-12f) {
            if (e[k] < lo[k] || e[k] > hi[k]) t1 = -1.f;
            continue;
        }
        float ta = (lo[k] - e[k]) / dd[k], tb = (hi[k] - e[k]) / dd[k];
        if (ta > tb) { const float tmp = ta; ta = tb; tb = tmp; }
        t0 = fmaxf(t0, ta);
        t1 = fminf(t1, tb);
    }
    V3 acc_c = v3(0.f, 0.f, 0.f), acc_a = v3(0.f, 0.f, 0.f);
    const int nsteps = t1 > t0 ? int((t1 - t0) / a.step + 0.5f) : 0;
    if (nsteps >= 1) {
        const float h = (t1 - t0) / float(nsteps);
        const V3 stepv = d * h;
        const V3 inv_n = v3(1.f / float(N[2]), 1.f / float(N[1]), 1.f / float(N[0]));
        const float step_size = sqrtf(dot3(mulv(stepv, inv_n), mulv(stepv, inv_n)));  // texture units
        const V3 L = v3(a.light[0], a.light[1], a.light[2]);                            // unit, texture space
        const V3 Lvox = mulv(L, v3(float(N[2]), float(N[1]), float(N[0])));
        V3 p = eye + d * t0;
        for (int it = 0; it < nsteps; ++it) {
            V3 shadow = v3(0.f, 0.f, 0.f);
            if (a.shadow_steps > 0) {
                float sstep = step_size * 3.0f;
                V3 sp = p + Lvox * sstep;
                float discont = 1.0f;
                const float satt = a.atten_density * 50.0f;
                for (int si = 0; si < a.shadow_steps; ++si) {
                    V3 s = v3(0.f, 0.f, 0.f);
                    float w[2];
                    trilinear<2>(psi, N, sp, w);
                    const Rgba f = fire(w[0], w[1]);
                    const float k = sstep * satt * discont;
                    s = v3(clamp01(s.x + f.a * (0.5f + 0.5f * (1.f - f.r)) * k), clamp01(s.y + f.a * (0.5f + 0.5f * (1.f - f.g)) * k),
                           clamp01(s.z + f.a * (0.5f + 0.5f * (1.f - f.b)) * k));
                    if (pot) {
                        float q[2];
                        trilinear<2>(pot, N, sp, q);
                        const Rgba g = green(q[0]);
                        s = v3(clamp01(s.x + g.a * (0.5f + 0.5f * (1.f - g.r)) * k), clamp01(s.y + g.a * (0.5f + 0.5f * (1.f - g.g)) * k),
                               clamp01(s.z + g.a * (0.5f + 0.5f * (1.f - g.b)) * k));
                    }
                    shadow = shadow + mulv(s, v3(1.f - shadow.x, 1.f - shadow.y, 1.f - shadow.z));
                    sp = sp + Lvox * sstep;
                    discont *= 0.96f;
                    sstep *= 1.0001f;
                }
            }
            Rgba color{0.f, 0.f, 0.f, 0.f};
            {
                const Sample s = shade_sample<2>(psi, N, p);
                const Rgba al = fire(s.re, s.im);
                const V3 rad = radiance(al, s, shadow, L, d);
                if (al.a > color.a) color = Rgba{rad.x, rad.y, rad.z, al.a};
            }
            if (pot) {
                const Sample s = shade_sample<2>(pot, N, p);
                const Rgba al = green(s.re);
                const V3 rad = radiance(al, s, shadow, L, d);
                if (al.a > color.a) color = Rgba{rad.x, rad.y, rad.z, al.a};
            }
            const float cs = a.color_density * step_size, as = a.atten_density * step_size;
            const V3 c = v3(fmaxf(cs * color.r, 0.f), fmaxf(cs * color.g, 0.f), fmaxf(cs * color.b, 0.f));
            const float tint = 0.75f;
            const V3 at = v3(clamp01(as * color.a * ((1.f - tint) + tint * fmaxf(1.f - color.r, 0.f))),
                             clamp01(as * color.a * ((1.f - tint) + tint * fmaxf(1.f - color.g, 0.f))),
                             clamp01(as * color.a * ((1.f - tint) + tint * fmaxf(1.f - color.b, 0.f))));
            acc_c = acc_c + mulv(c, v3(1.f - acc_a.x, 1.f - acc_a.y, 1.f - acc_a.z));
            acc_a = acc_a + mulv(at, v3(1.f - acc_a.x, 1.f - acc_a.y, 1.f - acc_a.z));
            if (acc_a.x > 0.99f && acc_a.y > 0.99f && acc_a.z > 0.99f) {
                acc_a = v3(1.f, 1.f, 1.f);
                break;
            }
            p = p + stepv;
        }
    }
    const V3 col = aces(acc_c + v3(1.f - acc_a.x, 1.f - acc_a.y, 1.f - acc_a.z));
    const int64_t o = int64_t(py) * a.width + px;
    if (a.format == 1) {
        reinterpret_cast<float4*>(a.out)[o] = make_float4(col.x, col.y, col.z, 1.f);
    } else {
        auto q = [](float x) { return (unsigned char)(fminf(fmaxf(x * 255.f + 0.5f, 0.f), 255.f)); };
        reinterpret_cast<uchar4*>(a.out)[o] = make_uchar4(q(col.x), q(col.y), q(col.z), 255);
    }
}

// Padded, normalised psi (float2) and V (real part, float) volumes.
template <typename R>
__global__ void normalise_psi_kernel(const Cx<R>* __restrict__ psi, int n0, int n1, int n2, float inv_scale,
                                     float2* __restrict__ out) {
    const int64_t N1 = n1 + 2, N2 = n2 + 2, total = int64_t(n0 + 2) * N1 * N2;
    for (int64_t g = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; g < total; g += int64_t(gridDim.x) * blockDim.x) {
        const int k = int(g % N2) - 1, j = int((g / N2) % N1) - 1, i = int(g / (N1 * N2)) - 1;
        float2 v = make_float2(0.f, 0.f);
        if (i >= 0 && i < n0 && j >= 0 && j < n1 && k >= 0 && k < n2) {
            const Cx<R> z = psi[(int64_t(i) * n1 + j) * n2 + k];
            v = make_float2(fminf(fmaxf(float(z.x) * inv_scale, -1.f), 1.f), fminf(fmaxf(float(z.y) * inv_scale, -1.f), 1.f));
        }
        out[g] = v;
    }
}
__global__ void max_abs_kernel(const float* __restrict__ v, int64_t count, unsigned int* __restrict__ out_bits) {
    float m = 0.f;
    for (int64_t g = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; g < count; g += int64_t(gridDim.x) * blockDim.x)
        m = fmaxf(m, fabsf(v[g]));
    for (int off = 16; off > 0; off >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, off));
    if ((threadIdx.x & 31) == 0) atomicMax(out_bits, __float_as_uint(m));  // non-negative floats order as integers
}
__global__ void normalise_pot_kernel(const float2* __restrict__ V, int n0, int n1, int n2, const unsigned int* max_bits,
                                     float fixed_scale, float2* __restrict__ out) {
    const float mx = fixed_scale > 0.f ? fixed_scale : __uint_as_float(*max_bits);
    const float inv = mx > 0.f ? 1.f / mx : 0.f;
    const int64_t N1 = n1 + 2, N2 = n2 + 2, total = int64_t(n0 + 2) * N1 * N2;
    for (int64_t g = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; g < total; g += int64_t(gridDim.x) * blockDim.x) {
        const int k = int(g % N2) - 1, j = int((g / N2) % N1) - 1, i = int(g / (N1 * N2)) - 1;
        float2 v = make_float2(0.f, 0.f);
        if (i >= 0 && i < n0 && j >= 0 && j < n1 && k >= 0 && k < n2) {
            const float2 z = V[(int64_t(i) * n1 + j) * n2 + k];
            v = make_float2(fminf(fmaxf(z.x * inv, -1.f), 1.f), fminf(fmaxf(z.y * inv, -1.f), 1.f));
        }
        out[g] = v;
    }
}

int grid_of(int64_t n) {
    int64_t g = (n + 255) / 256;
    return int(g > 152 * 8 ? 152 * 8 : (g < 1 ? 1 : g));
}

}  // namespace

// Camera of a turntable view around the padded volume's centre (world x = array axis 2,
// y = axis 1 (up), z = axis 0), as the reference's TurntableCamera with fov and elevation.
bool render_camera(const int npad[3], const wfs_render_desc& d, RenderArgs& a) {
    // steps below 0.05 voxel are refused (the reference refuses below 0.1) so a ray's step count stays bounded
    if (d.width < 1 || d.height < 1 || !(d.fov_deg > 0.0 && d.fov_deg < 179.0) || !(d.relative_step >= 0.05)) return false;
    const double c[3] = {0.5 * (npad[2] - 1), 0.5 * (npad[1] - 1), 0.5 * (npad[0] - 1)};
    const double half = 0.5 * d.fov_deg * M_PI / 180.0;
    const double rad = 0.5 * std::sqrt(double(npad[0]) * npad[0] + double(npad[1]) * npad[1] + double(npad[2]) * npad[2]);
    const double dist = d.distance > 0.0 ? d.distance : 1.05 * rad / std::sin(half);
    const double az = d.azimuth_deg * M_PI / 180.0, el = d.elevation_deg * M_PI / 180.0;
    const double dir[3] = {std::cos(el) * std::sin(az), std::sin(el), std::cos(el) * std::cos(az)};
    double eye[3], fw[3], rt[3], up[3];
    for (int k = 0; k < 3; ++k) {
        eye[k] = c[k] + dist * dir[k];
        fw[k] = -dir[k];
    }
    // right = forward x (0, 1, 0), up = right x forward
    rt[0] = -fw[2];
    rt[1] = 0.0;
    rt[2] = fw[0];
    double rl = std::sqrt(rt[0] * rt[0] + rt[2] * rt[2]);
    if (rl < 1e-9) {
        rt[0] = 1.0;
        rt[2] = 0.0;
        rl = 1.0;
    }
    rt[0] /= rl;
    rt[2] /= rl;
    up[0] = rt[1] * fw[2] - rt[2] * fw[1];
    up[1] = rt[2] * fw[0] - rt[0] * fw[2];
    up[2] = rt[0] * fw[1] - rt[1] * fw[0];
    double L[3] = {d.light[0], d.light[1], d.light[2]};
    const double ll = std::sqrt(L[0] * L[0] + L[1] * L[1] + L[2] * L[2]);
    if (!(ll > 0.0)) return false;
    for (int k = 0; k < 3; ++k) {
        a.eye[k] = float(eye[k]);
        a.forward[k] = float(fw[k]);
        a.right[k] = float(rt[k]);
        a.up[k] = float(up[k]);
        a.light[k] = float(L[k] / ll);
        a.npad[k] = npad[k];
    }
    a.tan_half_fov = float(std::tan(half));
    a.aspect = float(double(d.width) / double(d.height));
    a.width = d.width;
    a.height = d.height;
    a.step = float(d.relative_step);
    a.color_density = 6000.f;
    a.atten_density = 500.f;
    a.shadow_steps = d.shadow_steps;
    a.format = d.format;
    return true;
}

template <typename R>
cudaError_t launch_render(const Cx<R>* psi, const float2* V, const int n[3], const wfs_render_desc& d, void* out,
                          cudaStream_t s) {
    RenderArgs a{};
    const int npad[3] = {n[0] + 2, n[1] + 2, n[2] + 2};
    if (!render_camera(npad, d, a)) return cudaErrorInvalidValue;
    a.out = out;
    const int64_t vox = int64_t(npad[0]) * npad[1] * npad[2];
    float2* vol = nullptr;
    float2* pot = nullptr;
    unsigned int* mx = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&vol, vox * sizeof(float2), s);
    if (e != cudaSuccess) return e;
    const float scale = d.wave_function_scale > 0.0 ? float(d.wave_function_scale) : 0.005f;
    normalise_psi_kernel<R><<<grid_of(vox), 256, 0, s>>>(psi, n[0], n[1], n[2], 1.f / scale, vol);
    if (V && d.show_potential) {
        e = cudaMallocAsync((void**)&pot, vox * sizeof(float2) + 256, s);
        if (e == cudaSuccess) {
            mx = reinterpret_cast<unsigned int*>(pot + vox);  // one word after the volume
            e = cudaMemsetAsync(mx, 0, sizeof(unsigned int), s);
        }
        if (e == cudaSuccess) {
            const int64_t nf = int64_t(n[0]) * n[1] * n[2] * 2;
            max_abs_kernel<<<grid_of(nf), 256, 0, s>>>(reinterpret_cast<const float*>(V), nf, mx);
            normalise_pot_kernel<<<grid_of(vox), 256, 0, s>>>(V, n[0], n[1], n[2], mx, float(d.potential_scale), pot);
        }
    }
    if (e == cudaSuccess) {
        dim3 blk(16, 8), grd((d.width + 15) / 16, (d.height + 7) / 8);
        render_kernel<<<grd, blk, 0, s>>>(reinterpret_cast<const float*>(vol), reinterpret_cast<const float*>(pot), a);
        e = cudaGetLastError();
    }
    if (pot) cudaFreeAsync(pot, s);
    cudaFreeAsync(vol, s);
    return e;
}

template cudaError_t launch_render<float>(const Cx<float>*, const float2*, const int*, const wfs_render_desc&, void*,
                                          cudaStream_t);
template cudaError_t launch_render<double>(const Cx<double>*, const float2*, const int*, const wfs_render_desc&, void*,
                                           cudaStream_t);

}  // namespace wfs

extern "C" int wfs_render_volume(const void* psi_device, int32_t dtype, const int32_t n[3], const void* potential_device,
                                 const wfs_render_desc* desc, void* out_device, void* stream) {
    if (!psi_device || !n || !desc || !out_device || (dtype != WFS_C64 && dtype != WFS_C128)) return WFS_ERR_ARG;
    if (n[0] < 2 || n[1] < 2 || n[2] < 2 || (desc->format != 0 && desc->format != 1) || desc->shadow_steps < 0 ||
        desc->shadow_steps > 1000 || desc->width < 1 || desc->height < 1 ||
        int64_t(desc->width) * desc->height > (int64_t(1) << 28))
        return WFS_ERR_ARG;
    const int nn[3] = {n[0], n[1], n[2]};
    cudaError_t e;
    if (dtype == WFS_C64)
        e = wfs::launch_render<float>(static_cast<const wfs::Cx<float>*>(psi_device),
                                      static_cast<const float2*>(potential_device), nn, *desc, out_device,
                                      static_cast<cudaStream_t>(stream));
    else
        e = wfs::launch_render<double>(static_cast<const wfs::Cx<double>*>(psi_device),
                                       static_cast<const float2*>(potential_device), nn, *desc, out_device,
                                       static_cast<cudaStream_t>(stream));
    if (e == cudaErrorInvalidValue) return WFS_ERR_ARG;
    return e == cudaSuccess ? WFS_OK : WFS_ERR_CUDA;
}
