// kernels.h — launch interface between the host engine (engine.cu) and the
// device kernels. Plain structs; every launcher returns a cudaError_t.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

// Resident blocks per SM the FFT pass kernels and the fused plane kernel are
// register-budgeted for (build-time tuning knobs). Measured at 256^3 complex64
// on GB300: 2 for the pass kernels (x pass 75 us vs 84 us at 3) and 3 for the
// plane kernel (162 us vs 175 us at 2 and 258 us unconstrained).
#ifndef WFS_MINB_PASS
#define WFS_MINB_PASS 2
#endif
#ifndef WFS_MINB_PIPE
#define WFS_MINB_PIPE 2
#endif
#ifndef WFS_MINB_PLANE
#define WFS_MINB_PLANE 3
#endif
// The copy-staged strided pass computes no per-thread copy addresses and fits 80
// registers without spilling, so it is budgeted for 3 resident blocks per SM.
#ifndef WFS_MINB_STAGED
#define WFS_MINB_STAGED 3
#endif

namespace wfs {

// Two-stage plans (L = P * Q) of the supported FFT lengths.
#define WFS_PLAN_LIST(M)                                                                                      \
    M(2, 2, 1) M(3, 3, 1) M(4, 2, 2) M(6, 3, 2) M(8, 4, 2) M(12, 4, 3) M(16, 4, 4) M(24, 6, 4) M(32, 8, 4)      \
    M(48, 8, 6) M(64, 8, 8) M(96, 12, 8) M(128, 16, 8) M(192, 16, 12) M(256, 16, 16) M(384, 24, 16)            \
    M(512, 32, 16) M(768, 32, 24) M(1024, 32, 32)

// (P, Q) of the two-stage plan of length L on the host; false for unsupported lengths.
inline bool plan_pq(int L, int& P, int& Q) {
    switch (L) {
#define WFS_PLAN(L_, P_, Q_) case L_: P = P_; Q = Q_; return true;
        WFS_PLAN_LIST(WFS_PLAN)
#undef WFS_PLAN
        default: return false;
    }
}


constexpr int kMaxBox = 8;      // volume-probability boxes per fused observation
constexpr int kLocQ = 7;        // location box sums: S, Sx, Sy, Sz, Sxx, Syy, Szz
constexpr int kObsRowsPerCta = 8;  // (x, y) rows per CTA of observe_real_kernel: one warp per row

enum PassOp { OP_PLAIN = 0, OP_KIN = 1, OP_VPH = 2, OP_OBS = 3 };

struct ObsBox {
    int b[3];
    int c[3];
};

struct ObsArgs {
    int nbox;
    int has_loc;
    ObsBox box[kMaxBox];
    ObsBox loc;
    int n[3];
    double dx[3];
    double* partials;   // [grid][nq] per-CTA sums (scratch)
    int nq;             // nbox + (has_loc ? kLocQ : 0)
};

// One FFT pass over pencils of length L along one axis.
// Strided kernels: element (outer o, row r, column c) lives at
//   data + o*outer_stride + r*row_stride + c,   c < ncols (contiguous columns).
// Contiguous kernels: row q (q < nrows) is data + q*L .. + L - 1.
template <typename R>
struct PassArgs {
    Cx<R>* data;
    const Cx<R>* tw;        // twiddle table of the axis (two_stage_roots: 3L entries)
    int64_t outer_stride;
    int64_t row_stride;
    int32_t ncols;          // strided: columns per outer slab
    int32_t tiles;          // strided: column tiles per outer slab
    int64_t nrows;          // contiguous: number of rows
    int32_t dir;            // OP_PLAIN: -1 forward, +1 inverse
    R scale;                // applied to the pass output
    // OP_KIN (strided): out = F^-1( k_row[k] * k_c1[c / c2n] * k_c2[c % c2n] * F(x) ) * scale
    const Cx<R>* k_row;
    const Cx<R>* k_c1;
    const Cx<R>* k_c2;
    int32_t c2n;
    // OP_VPH (contiguous): out = F( e[q*L + z] * F^-1(x) ) * scale
    const Cx<R>* ephase;
    // OP_OBS (contiguous, read-only): observe scale * F^-1(x); rows are (x, y) = (q / ny, q % ny)
    ObsArgs obs;
    int* status;            // copy-staged passes: bit 0 set when a bounded wait gave up (may be null)
    uint64_t wait_ns;       // copy-staged passes: limit of the wait for a staged tile (0: the default, 1: give up at once)
};

template <typename R>
cudaError_t launch_fft_strided(int L, int op, const PassArgs<R>& a, int64_t outer_count, cudaStream_t s);
template <typename R>
cudaError_t launch_fft_contig(int L, int op, const PassArgs<R>& a, cudaStream_t s, int* grid_out);
bool fft_length_supported(int L, bool dbl);
int fft_contig_rows_per_cta(int L, bool dbl);
int fft_strided_cols_per_cta(int L, bool dbl);

// ---- fused yz-plane pass (plane_f32.cu / plane_f64.cu) ----
template <typename R>
struct PlaneArgs;
template <typename R>
cudaError_t launch_plane(int ny, int nz, const PlaneArgs<R>& a, int64_t nplanes, cudaStream_t s);
bool plane_pass_supported(int ny, int nz);

// ---- field kernels (field_kernels.cu) ----
struct WallDev {
    float U, cx, cy, cz, nx, ny, nz, rot;  // rot: slit rotation (radian); the frame is formed on the device
    float plateau, slope, slope_exp, slit_spacing, slit_width;
    int slit_count;
};
struct AbsorbDev {
    float bottom[3], top[3], offset, pp[3], pn[3], ep[3], en[3];
};

cudaError_t launch_wall(float2* V, const int n[3], const float dx[3], const WallDev& w, cudaStream_t s);

// Moving walls of the dynamic potential mode: every wall at its current centre, plus the
// previous centres of the walls that move. frames[3 * i] is wall i's rotated slit axis
// (wall_right), formed once on the device by launch_wall_frames.
constexpr int kMaxDynWalls = 8;
struct DynWallsDev {
    int nwall;
    WallDev w[kMaxDynWalls];          // centre = the centre after this step's advection
    float old_c[kMaxDynWalls][3];     // centre before it
    int moving[kMaxDynWalls];         // 1 when the wall moved this step
    int lo[3], hi[3];                 // voxel box (inclusive) that holds every moving wall's band
    const float* frames;
};
cudaError_t launch_wall_frames(float* frames, const WallDev* walls, int nwall, cudaStream_t s);
// Rewrites V.x (the sum of all walls, in order, from zero) and the phase table e at the
// voxels that a moving wall covered before or covers after this step; other voxels keep
// their values, which the walls' new positions do not change. e may be null (no table).
template <typename R>
cudaError_t launch_wall_band(float2* V, Cx<R>* e, double dt, const int n[3], const float dx[3], const DynWallsDev& d,
                             cudaStream_t s);
cudaError_t launch_absorbing(float2* V, const int n[3], const float dx[3], const AbsorbDev& a, cudaStream_t s);
cudaError_t launch_add_raw(float2* V, const void* src, int raw_type, int64_t count, cudaStream_t s);
template <typename R>
cudaError_t launch_gaussian(Cx<R>* psi, const int n[3], const R* gx, const R* gy, const R* gz,
                            const R* rx, const R* ry, const R* rz, R kx, R ky, R kz, cudaStream_t s);
template <typename R>
cudaError_t launch_vphase(Cx<R>* e, const float2* V, double dt, int64_t count, cudaStream_t s);
template <typename R>
cudaError_t launch_kin_product(Cx<R>* out, const Cx<R>* kx, const Cx<R>* ky, const Cx<R>* kz,
                               const int n[3], cudaStream_t s);
template <typename R>
cudaError_t launch_mul_inplace(Cx<R>* inout, const Cx<R>* f, int64_t count, cudaStream_t s);
template <typename R>
cudaError_t launch_observe_real(const Cx<R>* psi, const ObsArgs& o, cudaStream_t s, int* grid_out);
cudaError_t launch_reduce_partials(const double* partials, int nblocks, int nq, double* out, cudaStream_t s);
template <typename R>
cudaError_t launch_norm(const Cx<R>* psi, int64_t count, double* partials, int* nblocks, int* flag, cudaStream_t s);

// ---- plane probability current (current.cu) ----
struct PlaneCurrentArgs {
    int n[3];
    double dx[3];
    float center[3], right[3], up[3], normal[3];  // float32 frame, as the reference computes it
    float dWf, dHf;                                 // sample spacings on the plane
    int sx, sy;                                     // odd sample counts
    double mass;
};
template <typename R>
cudaError_t launch_plane_current(const Cx<R>* psi, const PlaneCurrentArgs& a, double* partials, int max_blocks,
                                 R* density, cudaStream_t s, int* grid_out);

// ---- headless volume rendering (render.cu) ----
struct RenderArgs {
    float eye[3], forward[3], right[3], up[3], light[3];
    int npad[3];          // padded volume dimensions (axis 0, 1, 2)
    float tan_half_fov, aspect, step, color_density, atten_density;
    int width, height, shadow_steps, format;
    void* out;
};
}  // namespace wfs
struct wfs_render_desc;
namespace wfs {
template <typename R>
cudaError_t launch_render(const Cx<R>* psi, const float2* V, const int n[3], const wfs_render_desc& d, void* out,
                          cudaStream_t s);

// ---- power series (taylor.cu) ----
template <typename R>
struct TaylorArgs {
    const Cx<R>* s_prev;
    Cx<R>* s_next;        // may be null on the last term
    const float2* V;
    const Cx<R>* acc_in;  // psi (term 1) or the accumulator
    Cx<R>* acc_out;       // accumulator
    int n[3];
    R dxq;                // 2nd order: every axis divided by dx_x twice
    R c4[3];              // 4th order: 1 / (12 dx_a^2)
    R inv2m;              // 1 / 2 / m
    R a;                  // dt / n
};
template <typename R>
cudaError_t launch_taylor_term(int stencil_order, const TaylorArgs<R>& t, cudaStream_t s);

}  // namespace wfs
