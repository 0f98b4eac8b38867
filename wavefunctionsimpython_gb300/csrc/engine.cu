// engine.cu — host side of the C ABI declared in include/wfs.h.
//
// Split-operator schedule. The reference step (sources/sim_state.py:641-697)
// is S = P V P with P = F^-1 K/2 F. With F = Fx Fy Fz applied as one pencil
// pass per axis and the kinetic factor K = Kx Ky Kz separable, the engine
// keeps psi in one of four representations and applies S as
//   X[Fx K Fx^-1]  Y[Fy^-1]  Z[Fz^-1 E Fz]  Y[Fy]      (E = exp(-i dt V))
// per step, merging the trailing K/2 of one step with the leading K/2 of the
// next (Strang merging). Representations of the stored array:
//   REAL    psi_n                      (x, y, z)
//   G       Fz psi_n                   (x, y, kz)
//   H       Fy Fz psi_n                (x, ky, kz)
//   PENDING Fy Fz V P psi_{n-1}; psi_n = X[Fx K/2 Fx^-1] of it, in H form.
// Reading psi or observing materialises what is needed; observation from
// PENDING costs X[K/2] + Y[Fy^-1] + a read-only Z[Fz^-1 observe] pass.
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/wfs.h"
#include "kernels.h"
#include "plane_kernels.cuh"
#include "host_helpers.h"

using namespace wfs;

namespace {

thread_local std::string g_error;

enum Rep { REP_REAL = 0, REP_G = 1, REP_H = 2, REP_PENDING = 3 };

struct KinTables {
    double dt = std::nan(""), mass = std::nan(""), frac = std::nan(""), amp = std::nan("");
    void* k[3] = {nullptr, nullptr, nullptr};
};

// Dynamic potential mode (wfs_set_dynamic_walls): the walls with their current centres and
// velocities, the absorbing ramp the rebuild adds, and the walls' slit axes on the device.
struct DynWalls {
    int nwall = 0;
    wfs_wall walls[wfs::kMaxDynWalls];
    double vel[wfs::kMaxDynWalls][3];
    bool has_abs = false;
    wfs_absorbing abs;
    bool rebuilt = false;  // the first update rebuilds V whole, as the reference does every step
    float* frames = nullptr;
    wfs::WallDev* dwalls = nullptr;
};

}  // namespace

namespace wfs {
// Lets entry points without a handle report through wfs_global_error().
void record_global_error(const std::string& m) { g_error = m; }
}  // namespace wfs

struct wfs_handle {
    int n[3];
    double extent[3];
    double dx[3];
    int dtype;
    int device;
    cudaStream_t stream;
    bool own_stream;
    int64_t count;
    size_t elem;          // bytes per psi element
    void* psi;            // live psi buffer
    void* scratch[2];     // Taylor buffers (allocated on first use)
    float2* V;
    void* ephase;         // exp(-i dt V) in psi precision
    double ephase_dt;
    bool ephase_valid;
    void* tw[3];          // twiddle tables per axis
    KinTables kin_half, kin_full;
    DynWalls dyn;
    Rep rep;
    double pend_dt, pend_mass;
    double* partials;     // observation scratch, per-CTA FP64 sums
    size_t partials_cap;  // doubles
    double* series;       // device observation series of wfs_run_split
    size_t series_cap;    // doubles
    double* dres;         // device results
    double* hres;         // pinned host results
    int* dflag;
    uint64_t copy_wait_ns;  // limit of a copy-staged pass's wait for a tile (wfs_set_copy_wait_limit)
    std::string err;
    // per-pass CUDA-event profile (wfs_profile_enable / wfs_profile_read)
    bool prof_on;
    int prof_stride;      // bracket the launches of every prof_stride-th step
    int64_t steps_done;   // steps (split or power series) since creation
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> prof_live;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> prof_pool;
    double prof_ms[WFS_NPASS];
    int64_t prof_count[WFS_NPASS];
    int64_t launches;
    int schedule;         // WFS_SCHEDULE_*
    // amplitude folded into the x factor of the stepping kinetic tables: the inverse of
    // the transforms' mean gain from rounded constants (split_step_gains), one step's
    // worth in the full table and half of the y/z part in the half table
    double amp_full, amp_half;
};

namespace {

int set_err(wfs_handle* h, int code, const std::string& msg) {
    if (h) h->err = msg;
    g_error = msg;
    return code;
}

#define CK(call)                                                                                  \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess)                                                                    \
            return set_err(h, WFS_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

bool is_dbl(const wfs_handle* h) { return h->dtype == WFS_C128; }

// Brackets one kernel launch with CUDA events when profiling is on and counts launches.
struct PassScope {
    wfs_handle* h;
    int kind;
    cudaEvent_t e1 = nullptr, e2 = nullptr;
    PassScope(wfs_handle* hh, int k) : h(hh), kind(k) {
        h->launches += 1;
        if (!h->prof_on || (h->steps_done % h->prof_stride) != 0) return;
        if (h->prof_pool.empty()) {
            cudaEvent_t a, b;
            if (cudaEventCreate(&a) != cudaSuccess) return;
            if (cudaEventCreate(&b) != cudaSuccess) { cudaEventDestroy(a); return; }
            h->prof_pool.push_back({a, b});
        }
        e1 = h->prof_pool.back().first;
        e2 = h->prof_pool.back().second;
        h->prof_pool.pop_back();
        cudaEventRecord(e1, h->stream);
    }
    ~PassScope() {
        if (!e1) return;
        cudaEventRecord(e2, h->stream);
        h->prof_live.push_back({kind, {e1, e2}});
    }
};

// The device wait-status word (dflag[1]) is queued into pinned memory before a host sync and
// read after it, so checking it adds no synchronisation.
cudaError_t queue_status(wfs_handle* h) {
    return cudaMemcpyAsync(h->hres + 255, h->dflag + 1, sizeof(int), cudaMemcpyDeviceToHost, h->stream);
}
// After the sync that followed queue_status: WFS_ERR_TIMEOUT when a bounded device-side wait
// gave up since the last check (the word is then cleared).
int take_status(wfs_handle* h) {
    int* s = reinterpret_cast<int*>(h->hres + 255);
    if (*s == 0) return WFS_OK;
    *s = 0;
    cudaMemsetAsync(h->dflag + 1, 0, sizeof(int), h->stream);
    return set_err(h, WFS_ERR_TIMEOUT, "a bounded device-side wait of a copy-staged pass gave up");
}

int ensure_partials(wfs_handle* h, size_t need) {
    if (need <= h->partials_cap) return WFS_OK;
    if (h->partials) cudaFree(h->partials);
    h->partials = nullptr;
    h->partials_cap = 0;
    CK(cudaMalloc(&h->partials, need * sizeof(double)));
    h->partials_cap = need;
    return WFS_OK;
}

template <typename R>
int upload_roots(wfs_handle* h, int axis) {
    const int L = h->n[axis];
    std::vector<Cx<R>> t(3 * size_t(L));
    if (!two_stage_roots<R>(L, t.data())) return WFS_ERR_UNSUPPORTED;
    CK(cudaMalloc(&h->tw[axis], t.size() * sizeof(Cx<R>)));
    CK(cudaMemcpy(h->tw[axis], t.data(), t.size() * sizeof(Cx<R>), cudaMemcpyHostToDevice));
    return WFS_OK;
}

// Per-axis kinetic factors exp(-i k^2 dt frac / m), k = 2 pi fftfreq(N, dx)
// (sources/sim_state.py:275-278, kinetic_operator.cu:20-23). The x factor is scaled by
// amp before rounding (1 for the kinetic operator itself; the engine's gain compensation
// for the tables of the split step).
template <typename R>
int ensure_kin(wfs_handle* h, KinTables& kt, double dt, double mass, double frac, double amp = 1.0) {
    if (kt.dt == dt && kt.mass == mass && kt.frac == frac && kt.amp == amp && kt.k[0]) return WFS_OK;
    // kernels already queued on the engine's stream may still read the old table
    if (kt.k[0]) CK(cudaStreamSynchronize(h->stream));
    for (int a = 0; a < 3; ++a) {
        const int L = h->n[a];
        std::vector<Cx<R>> v(L);
        for (int i = 0; i < L; ++i) {
            const int fi = (i < (L + 1) / 2) ? i : i - L;  // fftfreq ordering
            const double k = 2.0 * M_PI * double(fi) / (double(L) * h->dx[a]);
            const double ang = -k * k * dt * frac / mass;
            const double m = (a == 0) ? amp : 1.0;
            v[i] = mk<R>(R(m * std::cos(ang)), R(m * std::sin(ang)));
        }
        if (!kt.k[a]) CK(cudaMalloc(&kt.k[a], L * sizeof(Cx<R>)));
        CK(cudaMemcpy(kt.k[a], v.data(), L * sizeof(Cx<R>), cudaMemcpyHostToDevice));
    }
    kt.dt = dt;
    kt.mass = mass;
    kt.frac = frac;
    kt.amp = amp;
    return WFS_OK;
}

template <typename R>
int ensure_ephase(wfs_handle* h, double dt) {
    if (h->ephase_valid && h->ephase_dt == dt) return WFS_OK;
    if (!h->ephase) CK(cudaMalloc(&h->ephase, h->count * sizeof(Cx<R>)));
    PassScope ps(h, WFS_PASS_OTHER);
    CK(launch_vphase<R>(reinterpret_cast<Cx<R>*>(h->ephase), h->V, dt, h->count, h->stream));
    h->ephase_dt = dt;
    h->ephase_valid = true;
    return WFS_OK;
}

// ---- single passes --------------------------------------------------------
template <typename R>
PassArgs<R> base_args(wfs_handle* h, int axis) {
    PassArgs<R> a;
    std::memset(&a, 0, sizeof(a));
    a.data = reinterpret_cast<Cx<R>*>(h->psi);
    a.tw = reinterpret_cast<const Cx<R>*>(h->tw[axis]);
    a.scale = R(1);
    a.status = h->dflag + 1;
    a.wait_ns = h->copy_wait_ns;
    return a;
}

template <typename R>
int pass_x_kin(wfs_handle* h, KinTables& kt) {
    PassArgs<R> a = base_args<R>(h, 0);
    const int64_t plane = int64_t(h->n[1]) * h->n[2];
    a.outer_stride = 0;
    a.row_stride = plane;
    a.ncols = int32_t(plane);
    a.k_row = reinterpret_cast<const Cx<R>*>(kt.k[0]);
    a.k_c1 = reinterpret_cast<const Cx<R>*>(kt.k[1]);
    a.k_c2 = reinterpret_cast<const Cx<R>*>(kt.k[2]);
    a.c2n = h->n[2];
    a.scale = R(1.0 / double(h->n[0]));
    PassScope ps(h, WFS_PASS_X_KIN);
    CK(launch_fft_strided<R>(h->n[0], OP_KIN, a, 1, h->stream));
    return WFS_OK;
}

template <typename R>
int pass_y(wfs_handle* h, int dir) {
    PassArgs<R> a = base_args<R>(h, 1);
    a.outer_stride = int64_t(h->n[1]) * h->n[2];
    a.row_stride = h->n[2];
    a.ncols = h->n[2];
    a.dir = dir;
    a.scale = R(1.0 / std::sqrt(double(h->n[1])));
    PassScope ps(h, WFS_PASS_Y);
    CK(launch_fft_strided<R>(h->n[1], OP_PLAIN, a, h->n[0], h->stream));
    return WFS_OK;
}

template <typename R>
int pass_z(wfs_handle* h, int dir) {
    PassArgs<R> a = base_args<R>(h, 2);
    a.nrows = int64_t(h->n[0]) * h->n[1];
    a.dir = dir;
    a.scale = R(1.0 / std::sqrt(double(h->n[2])));
    PassScope ps(h, WFS_PASS_Z);
    CK(launch_fft_contig<R>(h->n[2], OP_PLAIN, a, h->stream, nullptr));
    return WFS_OK;
}

template <typename R>
int pass_z_vph(wfs_handle* h) {
    PassArgs<R> a = base_args<R>(h, 2);
    a.nrows = int64_t(h->n[0]) * h->n[1];
    a.ephase = reinterpret_cast<const Cx<R>*>(h->ephase);
    a.scale = R(1.0 / double(h->n[2]));
    PassScope ps(h, WFS_PASS_Z_VPH);
    CK(launch_fft_contig<R>(h->n[2], OP_VPH, a, h->stream, nullptr));
    return WFS_OK;
}

// Y[Fy^-1] Z[Fz^-1 E Fz] Y[Fy] in one launch (one cluster per yz-plane).
template <typename R>
int pass_plane(wfs_handle* h) {
    PlaneArgs<R> a;
    a.data = reinterpret_cast<Cx<R>*>(h->psi);
    a.tw_y = reinterpret_cast<const Cx<R>*>(h->tw[1]);
    a.tw_z = reinterpret_cast<const Cx<R>*>(h->tw[2]);
    a.ephase = reinterpret_cast<const Cx<R>*>(h->ephase);
    a.plane_elems = int64_t(h->n[1]) * h->n[2];
    a.scale_y = R(1.0 / std::sqrt(double(h->n[1])));
    a.scale_z = R(1.0 / double(h->n[2]));
    PassScope ps(h, WFS_PASS_PLANE);
    CK(launch_plane<R>(h->n[1], h->n[2], a, h->n[0], h->stream));
    return WFS_OK;
}

bool use_plane(const wfs_handle* h) {
    if (h->schedule == WFS_SCHEDULE_AXIS) return false;
    return plane_pass_supported(h->n[1], h->n[2]);
}

// ---- representation changes ----------------------------------------------
template <typename R>
int finish_pending(wfs_handle* h) {
    if (h->rep != REP_PENDING) return WFS_OK;
    int rc = ensure_kin<R>(h, h->kin_half, h->pend_dt, h->pend_mass, 0.25, h->amp_half);
    if (rc) return rc;
    rc = pass_x_kin<R>(h, h->kin_half);
    if (rc) return rc;
    h->rep = REP_H;
    return WFS_OK;
}

template <typename R>
int to_H(wfs_handle* h) {
    int rc = WFS_OK;
    if (h->rep == REP_PENDING) return finish_pending<R>(h);
    if (h->rep == REP_REAL) {
        if ((rc = pass_z<R>(h, -1))) return rc;
        h->rep = REP_G;
    }
    if (h->rep == REP_G) {
        if ((rc = pass_y<R>(h, -1))) return rc;
        h->rep = REP_H;
    }
    return WFS_OK;
}

template <typename R>
int to_real(wfs_handle* h) {
    int rc = finish_pending<R>(h);
    if (rc) return rc;
    if (h->rep == REP_H) {
        if ((rc = pass_y<R>(h, +1))) return rc;
        h->rep = REP_G;
    }
    if (h->rep == REP_G) {
        if ((rc = pass_z<R>(h, +1))) return rc;
        h->rep = REP_REAL;
    }
    return WFS_OK;
}

bool fft_ready(wfs_handle* h) {
    if (h->count >= (int64_t(1) << 31)) {  // the pass kernels index psi with 32-bit element offsets
        set_err(h, WFS_ERR_UNSUPPORTED, "split-step: grids of 2^31 sites or more are not supported");
        return false;
    }
    for (int a = 0; a < 3; ++a)
        if (!fft_length_supported(h->n[a], is_dbl(h))) {
            set_err(h, WFS_ERR_UNSUPPORTED, "split-step: axis length " + std::to_string(h->n[a]) +
                                                " not supported (2^a * 3^b with b <= 1, 2..1024)");
            return false;
        }
    return true;
}

// One update of the dynamic potential after a step (sources/sim_state.py:466-509): every
// wall advects by v dt with its x centre clamped at 0, then V is rebuilt from the walls and
// the absorbing ramp (sources/potential.py:508-522). The first update rebuilds V whole
// (any pre-initialised potential is dropped, as in the reference); later ones rewrite only
// the voxels a moving wall reached before or reaches after the move, together with their
// phase-table entries, which gives the same V as a whole rebuild.
template <typename R>
int dyn_update(wfs_handle* h, double dt) {
    DynWalls& d = h->dyn;
    DynWallsDev dd;
    std::memset(&dd, 0, sizeof(dd));
    dd.nwall = d.nwall;
    dd.frames = d.frames;
    bool any = false;
    for (int i = 0; i < d.nwall; ++i) {
        wfs_wall& w = d.walls[i];
        for (int k = 0; k < 3; ++k) dd.old_c[i][k] = float(w.center[k]);
        for (int k = 0; k < 3; ++k) w.center[k] = w.center[k] + d.vel[i][k] * dt;
        if (w.center[0] < 0.0) w.center[0] = 0.0;
        if (!wall_frame(&w, dd.w[i])) return set_err(h, WFS_ERR_ARG, "invalid moving wall");
        dd.moving[i] = (dd.w[i].cx != dd.old_c[i][0] || dd.w[i].cy != dd.old_c[i][1] || dd.w[i].cz != dd.old_c[i][2]);
        any = any || dd.moving[i];
    }
    const float dx[3] = {float(h->dx[0]), float(h->dx[1]), float(h->dx[2])};
    if (!d.rebuilt) {
        PassScope ps(h, WFS_PASS_OTHER);
        CK(cudaMemsetAsync(h->V, 0, h->count * sizeof(float2), h->stream));
        for (int i = 0; i < d.nwall; ++i) CK(launch_wall(h->V, h->n, dx, dd.w[i], h->stream));
        if (d.has_abs) {
            AbsorbDev ad;
            for (int k = 0; k < 3; ++k) {
                ad.bottom[k] = float(d.abs.bottom[k]);
                ad.top[k] = float(d.abs.top[k]);
                ad.pp[k] = float(d.abs.potential_pos[k]);
                ad.pn[k] = float(d.abs.potential_neg[k]);
                ad.ep[k] = float(d.abs.exponent_pos[k]);
                ad.en[k] = float(d.abs.exponent_neg[k]);
            }
            ad.offset = float(d.abs.offset);
            CK(launch_absorbing(h->V, h->n, dx, ad, h->stream));
        }
        h->ephase_valid = false;
        d.rebuilt = true;
        return WFS_OK;
    }
    if (!any) return WFS_OK;
    // the box the moving walls' bands lie in: along the normal of an axis-aligned wall the
    // voxels within its reach of the old or new centre (one voxel of margin each side),
    // the whole axis otherwise
    for (int k = 0; k < 3; ++k) {
        dd.lo[k] = h->n[k];
        dd.hi[k] = -1;
    }
    for (int i = 0; i < d.nwall; ++i) {
        if (!dd.moving[i]) continue;
        const WallDev& w = dd.w[i];
        const float nv[3] = {w.nx, w.ny, w.nz};
        const float cn[3] = {w.cx, w.cy, w.cz};
        const double reach = std::max(0.5 * w.plateau, 0.5 * w.plateau + double(w.slope));
        for (int k = 0; k < 3; ++k) {
            const bool aligned = nv[(k + 1) % 3] == 0.0f && nv[(k + 2) % 3] == 0.0f;
            int lo = 0, hi = h->n[k] - 1;
            if (aligned) {
                const double c0 = std::min(double(cn[k]), double(dd.old_c[i][k]));
                const double c1 = std::max(double(cn[k]), double(dd.old_c[i][k]));
                const double v0 = std::floor((c0 - reach) / h->dx[k] + 0.5 * h->n[k]) - 1.0;
                const double v1 = std::ceil((c1 + reach) / h->dx[k] + 0.5 * h->n[k]) + 1.0;
                lo = int(std::max(0.0, std::min(v0, double(h->n[k] - 1))));
                hi = int(std::max(0.0, std::min(v1, double(h->n[k] - 1))));
            }
            dd.lo[k] = std::min(dd.lo[k], lo);
            dd.hi[k] = std::max(dd.hi[k], hi);
        }
    }
    Cx<R>* e = (h->ephase_valid && h->ephase) ? reinterpret_cast<Cx<R>*>(h->ephase) : nullptr;
    PassScope ps(h, WFS_PASS_OTHER);
    CK(launch_wall_band<R>(h->V, e, h->ephase_dt, h->n, dx, dd, h->stream));
    return WFS_OK;
}

template <typename R>
int split_steps(wfs_handle* h, int nsteps, double dt, double mass) {
    if (nsteps <= 0) return WFS_OK;
    if (!fft_ready(h)) return WFS_ERR_UNSUPPORTED;
    int rc;
    if (h->rep == REP_PENDING && (h->pend_dt != dt || h->pend_mass != mass)) {
        if ((rc = finish_pending<R>(h))) return rc;
    }
    if ((rc = ensure_ephase<R>(h, dt))) return rc;
    if ((rc = ensure_kin<R>(h, h->kin_half, dt, mass, 0.25, h->amp_half))) return rc;
    if ((rc = ensure_kin<R>(h, h->kin_full, dt, mass, 0.5, h->amp_full))) return rc;
    bool merged = (h->rep == REP_PENDING);
    if (!merged && (rc = to_H<R>(h))) return rc;
    const bool plane = use_plane(h);
    for (int s = 0; s < nsteps; ++s, ++h->steps_done) {
        if ((rc = pass_x_kin<R>(h, merged ? h->kin_full : h->kin_half))) return rc;
        if (plane) {
            if ((rc = pass_plane<R>(h))) return rc;
        } else {
            if ((rc = pass_y<R>(h, +1))) return rc;
            if ((rc = pass_z_vph<R>(h))) return rc;
            if ((rc = pass_y<R>(h, -1))) return rc;
        }
        merged = true;
        if (h->dyn.nwall) {  // the potential of the next step (update_potential after evolve_state)
            if ((rc = dyn_update<R>(h, dt))) return rc;
            if ((rc = ensure_ephase<R>(h, dt))) return rc;
        }
    }
    h->rep = REP_PENDING;
    h->pend_dt = dt;
    h->pend_mass = mass;
    return WFS_OK;
}

// ---- observation ----------------------------------------------------------
int fill_obs(wfs_handle* h, const wfs_box* boxes, int nbox, const wfs_box* loc, ObsArgs& o) {
    if (nbox < 0 || nbox > kMaxBox) return set_err(h, WFS_ERR_ARG, "nbox must be in [0, 8]");
    if (nbox > 0 && !boxes) return set_err(h, WFS_ERR_ARG, "boxes is null");
    std::memset(&o, 0, sizeof(o));
    o.nbox = nbox;
    auto cp = [&](const wfs_box& b, ObsBox& d) -> bool {
        for (int a = 0; a < 3; ++a) {
            if (b.count[a] < 1 || b.bottom[a] < 0 || b.bottom[a] + b.count[a] > h->n[a]) return false;
            d.b[a] = b.bottom[a];
            d.c[a] = b.count[a];
        }
        return true;
    };
    for (int b = 0; b < nbox; ++b)
        if (!cp(boxes[b], o.box[b])) return set_err(h, WFS_ERR_ARG, "observation box outside the grid");
    o.has_loc = loc ? 1 : 0;
    if (loc && !cp(*loc, o.loc)) return set_err(h, WFS_ERR_ARG, "location box outside the grid");
    for (int a = 0; a < 3; ++a) {
        o.n[a] = h->n[a];
        o.dx[a] = h->dx[a];
    }
    o.nq = nbox + (loc ? kLocQ : 0);
    return WFS_OK;
}

// Launches the observation reduction for the current psi without changing the
// represented state; results (raw Simpson sums) land in dres[0..nq).
template <typename R>
int observe_launch(wfs_handle* h, ObsArgs& o, double* dout) {
    int rc = finish_pending<R>(h);
    if (rc) return rc;
    if (o.nq == 0) return WFS_OK;
    if (h->rep == REP_H) {
        if ((rc = pass_y<R>(h, +1))) return rc;
        h->rep = REP_G;
    }
    int grid = 0;
    if (h->rep == REP_G) {
        const int rows = fft_contig_rows_per_cta(h->n[2], is_dbl(h));
        const int64_t nrows = int64_t(h->n[0]) * h->n[1];
        const int64_t g = (nrows + rows - 1) / rows;
        if ((rc = ensure_partials(h, size_t(g) * o.nq))) return rc;
        o.partials = h->partials;
        PassArgs<R> a = base_args<R>(h, 2);
        a.nrows = nrows;
        a.scale = R(1.0 / std::sqrt(double(h->n[2])));
        a.obs = o;
        PassScope ps(h, WFS_PASS_OBSERVE);
        CK(launch_fft_contig<R>(h->n[2], OP_OBS, a, h->stream, &grid));
    } else {
        const int64_t nrows = int64_t(h->n[0]) * h->n[1];
        const int64_t g = (nrows + 7) / 8;
        if ((rc = ensure_partials(h, size_t(g) * o.nq))) return rc;
        o.partials = h->partials;
        PassScope ps(h, WFS_PASS_OBSERVE);
        CK(launch_observe_real<R>(reinterpret_cast<const Cx<R>*>(h->psi), o, h->stream, &grid));
    }
    PassScope ps(h, WFS_PASS_OTHER);
    CK(launch_reduce_partials(h->partials, grid, o.nq, dout, h->stream));
    return WFS_OK;
}

// Converts raw sums to the reference's quantities.
void finish_obs(const wfs_handle* h, const ObsArgs& o, const double* raw, double* prob, double* r, double* r2) {
    const double dv = h->dx[0] * h->dx[1] * h->dx[2] / 27.0;
    for (int b = 0; b < o.nbox; ++b)
        if (prob) prob[b] = raw[b] * dv;
    if (o.has_loc) {
        const double* l = raw + o.nbox;  // sums of w (v - N/2) and w (v - N/2)^2 per axis
        for (int a = 0; a < 3; ++a) {
            if (r) r[a] = l[1 + a] * h->dx[a] * dv;
            if (r2) r2[a] = l[4 + a] * (h->dx[a] * h->dx[a]) * dv;
        }
    }
}

template <typename R>
int do_observe(wfs_handle* h, const wfs_box* boxes, int nbox, const wfs_box* loc, double* prob, double* r, double* r2) {
    ObsArgs o;
    int rc = fill_obs(h, boxes, nbox, loc, o);
    if (rc) return rc;
    if ((rc = observe_launch<R>(h, o, h->dres))) return rc;
    if (o.nq) {
        CK(cudaMemcpyAsync(h->hres, h->dres, o.nq * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        CK(queue_status(h));
        CK(cudaStreamSynchronize(h->stream));
        if ((rc = take_status(h))) return rc;
    }
    finish_obs(h, o, h->hres, prob, r, r2);
    return WFS_OK;
}

// Sampling plane of PlaneProbabilityCurrent (sources/measurement.py:207-289): frame, sample
// grid and the sample spacings dW, dH the flux is scaled by.
int fill_plane(wfs_handle* h, const double* center, const double* normal, const double* size, const int32_t* count,
               double mass, PlaneCurrentArgs& a, double* dW, double* dH) {
    if (!center || !normal || !size || !count || !(mass > 0)) return set_err(h, WFS_ERR_ARG, "invalid plane argument");
    if (count[0] < 3 || count[1] < 3 || (count[0] % 2) == 0 || (count[1] % 2) == 0)
        return set_err(h, WFS_ERR_ARG, "sample counts must be odd and >= 3 (Simpson)");
    std::memset(&a, 0, sizeof(a));
    if (!plane_frame(normal, a.normal, a.right, a.up)) return set_err(h, WFS_ERR_ARG, "degenerate plane normal");
    for (int k = 0; k < 3; ++k) {
        a.n[k] = h->n[k];
        a.dx[k] = h->dx[k];
        a.center[k] = float(center[k]);
    }
    a.sx = count[0];
    a.sy = count[1];
    a.mass = mass;
    *dW = is_dbl(h) ? size[0] / double(a.sx - 1) : double(float(size[0]) / float(a.sx - 1));
    *dH = is_dbl(h) ? size[1] / double(a.sy - 1) : double(float(size[1]) / float(a.sy - 1));
    a.dWf = float(*dW);
    a.dHf = float(*dH);
    return WFS_OK;
}

// Arguments of every plane and the factor dW dH / 9 that turns its raw Simpson sum into a flux.
int fill_planes(wfs_handle* h, const wfs_plane* planes, int nplane, double mass, std::vector<PlaneCurrentArgs>& pa,
                std::vector<double>& pscale) {
    pa.resize(size_t(nplane));
    pscale.resize(size_t(nplane));
    for (int i = 0; i < nplane; ++i) {
        const wfs_plane& pl = planes[i];
        double dW = 0, dH = 0;
        const int rc = fill_plane(h, pl.center, pl.normal, pl.size, pl.count, mass, pa[size_t(i)], &dW, &dH);
        if (rc) return rc;
        pscale[size_t(i)] = dW * dH / 9.0;
    }
    return WFS_OK;
}

constexpr int kPlaneCurrentBlocks = 1024;  // CTAs (and FP64 partial sums) of a plane-current launch

template <typename R>
int do_run_split(wfs_handle* h, int nsteps, double dt, double mass, int interval, const wfs_box* boxes, int nbox,
                 const wfs_box* loc, double* prob_series, double* loc_series, const wfs_plane* planes = nullptr,
                 int nplane = 0, double* flux_series = nullptr) {
    if (interval < 1) return set_err(h, WFS_ERR_ARG, "interval must be >= 1");
    ObsArgs o;
    int rc = fill_obs(h, boxes, nbox, loc, o);
    if (rc) return rc;
    if (nplane < 0 || (nplane > 0 && !planes)) return set_err(h, WFS_ERR_ARG, "invalid planes");
    std::vector<PlaneCurrentArgs> pa;
    std::vector<double> pscale;
    if ((rc = fill_planes(h, planes, nplane, mass, pa, pscale))) return rc;
    if (nplane && (rc = ensure_partials(h, kPlaneCurrentBlocks))) return rc;
    const int stride = o.nq + nplane;  // doubles per record
    const int nrec = stride ? (nsteps + interval - 1) / interval : 0;
    const size_t need = size_t(nrec) * stride;
    if (need > h->series_cap) {  // kept across calls so repeated runs allocate nothing
        if (h->series) cudaFree(h->series);
        h->series = nullptr;
        h->series_cap = 0;
        CK(cudaMalloc(&h->series, need * sizeof(double)));
        h->series_cap = need;
    }
    double* dser = h->series;
    int rec = 0;
    for (int i = 0; i < nsteps && rc == WFS_OK; i += interval) {
        double* slot = dser + size_t(rec++) * stride;
        // plane currents read real-space psi: observe from it too (no fused transform)
        if (nplane) rc = to_real<R>(h);
        if (rc == WFS_OK && o.nq) rc = observe_launch<R>(h, o, slot);
        for (int p = 0; p < nplane && rc == WFS_OK; ++p) {
            int grid = 0;
            {
                PassScope ps(h, WFS_PASS_OBSERVE);
                CK(launch_plane_current<R>(reinterpret_cast<const Cx<R>*>(h->psi), pa[p], h->partials,
                                           kPlaneCurrentBlocks, nullptr, h->stream, &grid));
            }
            PassScope ps(h, WFS_PASS_OTHER);
            CK(launch_reduce_partials(h->partials, grid, 1, slot + o.nq + p, h->stream));
        }
        if (rc == WFS_OK) rc = split_steps<R>(h, (i + interval <= nsteps) ? interval : nsteps - i, dt, mass);
    }
    if (rc == WFS_OK && nrec) {
        std::vector<double> raw(size_t(nrec) * stride);
        cudaError_t e = cudaMemcpyAsync(raw.data(), dser, raw.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
        if (e == cudaSuccess) e = queue_status(h);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
        if (e != cudaSuccess) rc = set_err(h, WFS_ERR_CUDA, std::string("series copy: ") + cudaGetErrorString(e));
        if (rc == WFS_OK) rc = take_status(h);
        for (int k = 0; k < nrec && rc == WFS_OK; ++k) {
            double rr[3], rr2[3];
            const double* rk = raw.data() + size_t(k) * stride;
            finish_obs(h, o, rk, prob_series ? prob_series + size_t(k) * nbox : nullptr, rr, rr2);
            if (loc && loc_series)
                for (int a = 0; a < 3; ++a) {
                    loc_series[k * 6 + a] = rr[a];
                    loc_series[k * 6 + 3 + a] = rr2[a];
                }
            if (flux_series)
                for (int p = 0; p < nplane; ++p) flux_series[size_t(k) * nplane + p] = rk[o.nq + p] * pscale[p];
        }
    }
    return rc;
}

template <typename R>
int taylor_steps(wfs_handle* h, int nsteps, double dt, double mass, int order, int stencil) {
    int rc = to_real<R>(h);
    if (rc) return rc;
    for (int i = 0; i < 2; ++i)
        if (!h->scratch[i]) CK(cudaMalloc(&h->scratch[i], h->count * sizeof(Cx<R>)));
    TaylorArgs<R> t;
    std::memset(&t, 0, sizeof(t));
    for (int a = 0; a < 3; ++a) {
        t.n[a] = h->n[a];
        t.c4[a] = R(1.0 / (12.0 * h->dx[a] * h->dx[a]));
    }
    t.dxq = R(float(h->dx[0]));
    t.inv2m = R(1) / R(2) / R(mass);
    t.V = h->V;
    for (int s = 0; s < nsteps; ++s, ++h->steps_done) {
        Cx<R>* psi = reinterpret_cast<Cx<R>*>(h->psi);
        Cx<R>* A = reinterpret_cast<Cx<R>*>(h->scratch[0]);
        Cx<R>* B = reinterpret_cast<Cx<R>*>(h->scratch[1]);
        // buffers: s ping-pongs between A and psi (psi is free after term 1); acc lives in B
        Cx<R>* sp = psi;
        Cx<R>* sn = A;
        for (int n = 1; n <= order; ++n) {
            t.s_prev = sp;
            t.s_next = (n == order) ? nullptr : sn;
            t.acc_in = (n == 1) ? psi : B;
            t.acc_out = B;
            t.a = R(dt) / R(n);
            PassScope ps(h, WFS_PASS_TAYLOR);
            CK(launch_taylor_term<R>(stencil, t, h->stream));
            Cx<R>* tmp = sp;
            sp = sn;
            sn = tmp;
        }
        // new psi = B; old psi and A become scratch
        h->scratch[1] = h->psi;
        h->psi = B;
        if (h->dyn.nwall && (rc = dyn_update<R>(h, dt))) return rc;
    }
    return WFS_OK;
}

int dispatch_err(wfs_handle* h) { return set_err(h, WFS_ERR_ARG, "null handle"); }

}  // namespace

// ===========================================================================
extern "C" {

int wfs_abi_version(void) { return WFS_ABI_VERSION; }
const char* wfs_global_error(void) { return g_error.c_str(); }

int wfs_create(const wfs_grid_desc* d, wfs_handle** out) {
    wfs_handle* h = nullptr;
    if (!d || !out) return set_err(nullptr, WFS_ERR_ARG, "null descriptor or output");
    *out = nullptr;
    if (d->dtype != WFS_C64 && d->dtype != WFS_C128) return set_err(nullptr, WFS_ERR_ARG, "dtype must be WFS_C64 or WFS_C128");
    for (int a = 0; a < 3; ++a) {
        if (d->n[a] < 1 || d->n[a] > (1 << 16)) return set_err(nullptr, WFS_ERR_ARG, "axis length out of range");
        if (!(d->extent[a] > 0)) return set_err(nullptr, WFS_ERR_ARG, "extent must be positive");
    }
    if (int64_t(d->n[0]) * d->n[1] * d->n[2] > (int64_t(1) << 34)) return set_err(nullptr, WFS_ERR_ARG, "grid too large");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return set_err(nullptr, WFS_ERR_CUDA, "no CUDA device available");
    if (d->device < 0 || d->device >= ndev) return set_err(nullptr, WFS_ERR_ARG, "device ordinal out of range");
    h = new wfs_handle();
    std::memset(h->tw, 0, sizeof(h->tw));
    h->scratch[0] = h->scratch[1] = nullptr;
    h->psi = nullptr;
    h->V = nullptr;
    h->ephase = nullptr;
    h->ephase_valid = false;
    h->partials = nullptr;
    h->partials_cap = 0;
    h->series = nullptr;
    h->series_cap = 0;
    h->dres = nullptr;
    h->hres = nullptr;
    h->dflag = nullptr;
    h->rep = REP_REAL;
    h->prof_on = false;
    h->prof_stride = 1;
    h->copy_wait_ns = kWaitLimitNs;
    h->steps_done = 0;
    h->launches = 0;
    h->schedule = WFS_SCHEDULE_AUTO;
    h->amp_full = h->amp_half = 1.0;
    for (int k = 0; k < WFS_NPASS; ++k) { h->prof_ms[k] = 0.0; h->prof_count[k] = 0; }
    h->dtype = d->dtype;
    h->device = d->device;
    for (int a = 0; a < 3; ++a) {
        h->n[a] = d->n[a];
        h->extent[a] = d->extent[a];
        h->dx[a] = d->extent[a] / double(d->n[a]);
    }
    h->count = int64_t(h->n[0]) * h->n[1] * h->n[2];
    h->elem = is_dbl(h) ? 16 : 8;
    auto fail = [&](int rc) {
        std::string m = h->err;
        wfs_destroy(h);
        g_error = m;
        return rc;
    };
    if (cudaSetDevice(h->device) != cudaSuccess) return fail(set_err(h, WFS_ERR_CUDA, "cudaSetDevice failed"));
    if (d->stream) {
        h->stream = reinterpret_cast<cudaStream_t>(d->stream);
        h->own_stream = false;
    } else {
        if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess)
            return fail(set_err(h, WFS_ERR_CUDA, "cudaStreamCreate failed"));
        h->own_stream = true;
    }
    cudaError_t e = cudaMalloc(&h->psi, h->count * h->elem);
    if (e == cudaSuccess) e = cudaMalloc(&h->V, h->count * sizeof(float2));
    if (e == cudaSuccess) e = cudaMalloc(&h->dres, 256 * sizeof(double));
    if (e == cudaSuccess) e = cudaMallocHost(&h->hres, 256 * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&h->dflag, 2 * sizeof(int));  // [0] non-finite, [1] wait status
    if (e == cudaSuccess) e = cudaMemsetAsync(h->dflag, 0, 2 * sizeof(int), h->stream);
    if (e == cudaSuccess) std::memset(h->hres, 0, 256 * sizeof(double));
    if (e == cudaSuccess) e = cudaMemsetAsync(h->psi, 0, h->count * h->elem, h->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(h->V, 0, h->count * sizeof(float2), h->stream);
    if (e != cudaSuccess) return fail(set_err(h, WFS_ERR_CUDA, std::string("allocation: ") + cudaGetErrorString(e)));
    int rc = WFS_OK;
    for (int a = 0; a < 3 && rc == WFS_OK; ++a)
        if (fft_length_supported(h->n[a], is_dbl(h))) rc = is_dbl(h) ? upload_roots<double>(h, a) : upload_roots<float>(h, a);
    if (rc) return fail(rc);
    bool all_fft = true;
    for (int a = 0; a < 3; ++a) all_fft = all_fft && fft_length_supported(h->n[a], is_dbl(h));
    if (all_fft) {
        // per x pass: its own two x transforms; per step: one set of y/z transforms, whose
        // correction the full table carries whole and each of the two half tables by half
        double gx = 1.0, gyz = 1.0;
        if (is_dbl(h)) split_step_gains<double>(h->n, &gx, &gyz);
        else split_step_gains<float>(h->n, &gx, &gyz);
        h->amp_full = 1.0 / std::sqrt(gx * gyz);
        h->amp_half = 1.0 / std::sqrt(gx * std::sqrt(gyz));
    }
    *out = h;
    return WFS_OK;
}

int wfs_destroy(wfs_handle* h) {
    if (!h) return WFS_OK;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    void* bufs[] = {h->psi, h->scratch[0], h->scratch[1], h->V, h->ephase, h->partials, h->series, h->dres, h->dflag,
                    h->tw[0], h->tw[1], h->tw[2], h->kin_half.k[0], h->kin_half.k[1], h->kin_half.k[2],
                    h->kin_full.k[0], h->kin_full.k[1], h->kin_full.k[2], h->dyn.frames, h->dyn.dwalls};
    for (void* b : bufs)
        if (b) cudaFree(b);
    if (h->hres) cudaFreeHost(h->hres);
    for (auto& pe : h->prof_live) { cudaEventDestroy(pe.second.first); cudaEventDestroy(pe.second.second); }
    for (auto& pe : h->prof_pool) { cudaEventDestroy(pe.first); cudaEventDestroy(pe.second); }
    if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return WFS_OK;
}

const char* wfs_last_error(const wfs_handle* h) { return h ? h->err.c_str() : g_error.c_str(); }

int wfs_synchronize(wfs_handle* h) {
    if (!h) return dispatch_err(h);
    CK(queue_status(h));
    CK(cudaStreamSynchronize(h->stream));
    return take_status(h);
}

int wfs_set_copy_wait_limit(wfs_handle* h, double seconds) {
    if (!h) return dispatch_err(h);
    if (!(seconds >= 0.0) || seconds > 60.0) return set_err(h, WFS_ERR_ARG, "wait limit must lie in [0, 60] seconds");
    const double ns = seconds * 1e9;
    h->copy_wait_ns = ns <= 1.0 ? 1 : uint64_t(ns);
    return WFS_OK;
}

int wfs_potential_clear(wfs_handle* h) {
    if (!h) return dispatch_err(h);
    CK(cudaMemsetAsync(h->V, 0, h->count * sizeof(float2), h->stream));
    h->ephase_valid = false;
    return WFS_OK;
}

int wfs_potential_add_wall(wfs_handle* h, const wfs_wall* w) {
    if (!h) return dispatch_err(h);
    if (!w) return set_err(h, WFS_ERR_ARG, "null wall");
    WallDev wd;
    if (!wall_frame(w, wd)) return set_err(h, WFS_ERR_ARG, "wall normal has zero length or a value is not finite");
    float dx[3] = {float(h->dx[0]), float(h->dx[1]), float(h->dx[2])};
    CK(launch_wall(h->V, h->n, dx, wd, h->stream));
    h->ephase_valid = false;
    return WFS_OK;
}

int wfs_potential_add_absorbing(wfs_handle* h, const wfs_absorbing* a) {
    if (!h) return dispatch_err(h);
    if (!a) return set_err(h, WFS_ERR_ARG, "null absorbing description");
    AbsorbDev ad;
    for (int i = 0; i < 3; ++i) {
        ad.bottom[i] = float(a->bottom[i]);
        ad.top[i] = float(a->top[i]);
        ad.pp[i] = float(a->potential_pos[i]);
        ad.pn[i] = float(a->potential_neg[i]);
        ad.ep[i] = float(a->exponent_pos[i]);
        ad.en[i] = float(a->exponent_neg[i]);
    }
    ad.offset = float(a->offset);
    float dx[3] = {float(h->dx[0]), float(h->dx[1]), float(h->dx[2])};
    CK(launch_absorbing(h->V, h->n, dx, ad, h->stream));
    h->ephase_valid = false;
    return WFS_OK;
}

int wfs_set_dynamic_walls(wfs_handle* h, const wfs_wall* walls, const double* velocity, int32_t nwall,
                          const wfs_absorbing* absorbing) {
    if (!h) return dispatch_err(h);
    if (nwall < 0 || nwall > kMaxDynWalls)
        return set_err(h, WFS_ERR_ARG, "nwall must be in [0, " + std::to_string(kMaxDynWalls) + "]");
    if (nwall > 0 && (!walls || !velocity)) return set_err(h, WFS_ERR_ARG, "null walls or velocities");
    DynWalls& d = h->dyn;
    WallDev wd[kMaxDynWalls];
    for (int i = 0; i < nwall; ++i)
        if (!wall_frame(&walls[i], wd[i])) return set_err(h, WFS_ERR_ARG, "invalid wall " + std::to_string(i));
    d.nwall = 0;
    d.rebuilt = false;
    if (nwall == 0) return WFS_OK;
    if (!d.frames) CK(cudaMalloc(&d.frames, 3 * kMaxDynWalls * sizeof(float)));
    if (!d.dwalls) CK(cudaMalloc(&d.dwalls, kMaxDynWalls * sizeof(WallDev)));
    CK(cudaMemcpyAsync(d.dwalls, wd, nwall * sizeof(WallDev), cudaMemcpyHostToDevice, h->stream));
    CK(launch_wall_frames(d.frames, d.dwalls, nwall, h->stream));
    CK(cudaStreamSynchronize(h->stream));  // wd lives on this stack frame
    for (int i = 0; i < nwall; ++i) {
        d.walls[i] = walls[i];
        for (int k = 0; k < 3; ++k) d.vel[i][k] = velocity[3 * i + k];
    }
    d.has_abs = absorbing != nullptr;
    if (absorbing) d.abs = *absorbing;
    d.nwall = nwall;
    return WFS_OK;
}

int wfs_get_dynamic_walls(wfs_handle* h, double* centers, int32_t nwall) {
    if (!h) return dispatch_err(h);
    if (!centers || nwall != h->dyn.nwall) return set_err(h, WFS_ERR_ARG, "centers must hold 3 values per dynamic wall");
    for (int i = 0; i < nwall; ++i)
        for (int k = 0; k < 3; ++k) centers[3 * i + k] = h->dyn.walls[i].center[k];
    return WFS_OK;
}

int wfs_potential_add_raw(wfs_handle* h, const void* data, int32_t raw_type, int32_t on_device) {
    if (!h) return dispatch_err(h);
    if (!data) return set_err(h, WFS_ERR_ARG, "null data");
    static const size_t sz[] = {4, 8, 8, 16};
    if (raw_type < 0 || raw_type > 3) return set_err(h, WFS_ERR_ARG, "raw_type out of range");
    const size_t bytes = size_t(h->count) * sz[raw_type];
    const void* src = data;
    void* tmp = nullptr;
    if (!on_device) {
        CK(cudaMalloc(&tmp, bytes));
        CK(cudaMemcpyAsync(tmp, data, bytes, cudaMemcpyHostToDevice, h->stream));
        src = tmp;
    }
    cudaError_t e = launch_add_raw(h->V, src, raw_type, h->count, h->stream);
    if (tmp) {
        cudaStreamSynchronize(h->stream);
        cudaFree(tmp);
    }
    if (e != cudaSuccess) return set_err(h, WFS_ERR_CUDA, std::string("add_raw: ") + cudaGetErrorString(e));
    h->ephase_valid = false;
    return WFS_OK;
}

int wfs_set_potential(wfs_handle* h, const void* v, int32_t on_device) {
    if (!h) return dispatch_err(h);
    if (!v) return set_err(h, WFS_ERR_ARG, "null potential");
    CK(cudaMemcpyAsync(h->V, v, h->count * sizeof(float2), on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, h->stream));
    if (!on_device) CK(cudaStreamSynchronize(h->stream));
    h->ephase_valid = false;
    return WFS_OK;
}

int wfs_get_potential(wfs_handle* h, void* v, int32_t to_device) {
    if (!h) return dispatch_err(h);
    if (!v) return set_err(h, WFS_ERR_ARG, "null output");
    CK(cudaMemcpyAsync(v, h->V, h->count * sizeof(float2), to_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return WFS_OK;
}

int wfs_init_gaussian(wfs_handle* h, const double sigma[3], const double r0[3], const double k0[3]) {
    if (!h) return dispatch_err(h);
    if (!sigma || !r0 || !k0) return set_err(h, WFS_ERR_ARG, "null packet parameter");
    const bool dbl = is_dbl(h);
    // per-axis envelope and coordinate (common.cu:569-586, gaussian_wave_packet.cu:36-40)
    int total = h->n[0] + h->n[1] + h->n[2];
    std::vector<double> gd(total), rd(total);
    std::vector<float> gf(total), rf(total);
    int off[3] = {0, h->n[0], h->n[0] + h->n[1]};
    for (int a = 0; a < 3; ++a) {
        for (int i = 0; i < h->n[a]; ++i) {
            const int iv = i - h->n[a] / 2;
            if (dbl) {
                const double r = h->dx[a] * double(iv);
                const double aa = 2.0 * sigma[a];
                const double norm = std::pow(2.0 / M_PI / aa / aa, 0.25);
                const double d = r - r0[a];
                gd[off[a] + i] = norm * std::exp(-d * d / aa / aa);
                rd[off[a] + i] = r;
            } else {
                volatile float r = float(h->dx[a]) * float(iv);
                const float aa = 2.0f * float(sigma[a]);
                volatile float q = 2.0f / float(M_PI);
                q = q / aa;
                q = q / aa;
                const float norm = std::pow(float(q), 0.25f);
                volatile float d = float(r) - float(r0[a]);
                volatile float ex = -float(d) * float(d);
                ex = ex / aa;
                ex = ex / aa;
                volatile float g = norm * std::exp(float(ex));
                gf[off[a] + i] = g;
                rf[off[a] + i] = r;
            }
        }
    }
    const size_t rb = dbl ? sizeof(double) : sizeof(float);
    void* dbuf = nullptr;
    CK(cudaMalloc(&dbuf, 2 * total * rb));
    CK(cudaMemcpyAsync(dbuf, dbl ? (void*)gd.data() : (void*)gf.data(), total * rb, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync((char*)dbuf + total * rb, dbl ? (void*)rd.data() : (void*)rf.data(), total * rb, cudaMemcpyHostToDevice, h->stream));
    cudaError_t e;
    if (dbl) {
        const double* g = reinterpret_cast<const double*>(dbuf);
        const double* r = g + total;
        e = launch_gaussian<double>(reinterpret_cast<Cx<double>*>(h->psi), h->n, g, g + off[1], g + off[2], r, r + off[1], r + off[2],
                                    k0[0], k0[1], k0[2], h->stream);
    } else {
        const float* g = reinterpret_cast<const float*>(dbuf);
        const float* r = g + total;
        e = launch_gaussian<float>(reinterpret_cast<Cx<float>*>(h->psi), h->n, g, g + off[1], g + off[2], r, r + off[1], r + off[2],
                                   float(k0[0]), float(k0[1]), float(k0[2]), h->stream);
    }
    cudaStreamSynchronize(h->stream);
    cudaFree(dbuf);
    if (e != cudaSuccess) return set_err(h, WFS_ERR_CUDA, std::string("gaussian: ") + cudaGetErrorString(e));
    h->rep = REP_REAL;
    return WFS_OK;
}

int wfs_set_psi(wfs_handle* h, const void* psi, int32_t on_device) {
    if (!h) return dispatch_err(h);
    if (!psi) return set_err(h, WFS_ERR_ARG, "null psi");
    CK(cudaMemcpyAsync(h->psi, psi, h->count * h->elem, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, h->stream));
    if (!on_device) CK(cudaStreamSynchronize(h->stream));
    h->rep = REP_REAL;
    return WFS_OK;
}

int wfs_get_psi(wfs_handle* h, void* psi, int32_t to_device) {
    if (!h) return dispatch_err(h);
    if (!psi) return set_err(h, WFS_ERR_ARG, "null output");
    int rc = is_dbl(h) ? to_real<double>(h) : to_real<float>(h);
    if (rc) return rc;
    CK(cudaMemcpyAsync(psi, h->psi, h->count * h->elem, to_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, h->stream));
    CK(queue_status(h));
    CK(cudaStreamSynchronize(h->stream));
    return take_status(h);
}

int wfs_psi_device_ptr(wfs_handle* h, void** ptr) {
    if (!h) return dispatch_err(h);
    if (!ptr) return set_err(h, WFS_ERR_ARG, "null output");
    int rc = is_dbl(h) ? to_real<double>(h) : to_real<float>(h);
    if (rc) return rc;
    *ptr = h->psi;
    return WFS_OK;
}

int wfs_step_split(wfs_handle* h, int32_t nsteps, double dt, double mass) {
    if (!h) return dispatch_err(h);
    if (nsteps < 0 || !(mass > 0) || !std::isfinite(dt)) return set_err(h, WFS_ERR_ARG, "invalid nsteps, dt or mass");
    return is_dbl(h) ? split_steps<double>(h, nsteps, dt, mass) : split_steps<float>(h, nsteps, dt, mass);
}

int wfs_step_taylor(wfs_handle* h, int32_t nsteps, double dt, double mass, int32_t order, int32_t stencil_order) {
    if (!h) return dispatch_err(h);
    if (nsteps < 0 || order < 1 || !(mass > 0) || !std::isfinite(dt)) return set_err(h, WFS_ERR_ARG, "invalid nsteps, order, dt or mass");
    if (stencil_order != 2 && stencil_order != 4) return set_err(h, WFS_ERR_ARG, "stencil_order must be 2 or 4");
    return is_dbl(h) ? taylor_steps<double>(h, nsteps, dt, mass, order, stencil_order)
                     : taylor_steps<float>(h, nsteps, dt, mass, order, stencil_order);
}

int wfs_kinetic_operator(wfs_handle* h, double dt, double mass, double fraction, void* out, int32_t to_device) {
    if (!h) return dispatch_err(h);
    if (!out || !(mass > 0)) return set_err(h, WFS_ERR_ARG, "null output or invalid mass");
    KinTables kt;
    int rc;
    void* dev = out;
    if (!to_device) CK(cudaMalloc(&dev, h->count * h->elem));
    if (is_dbl(h)) {
        rc = ensure_kin<double>(h, kt, dt, mass, fraction);
        if (!rc) CK(launch_kin_product<double>(reinterpret_cast<Cx<double>*>(dev), (Cx<double>*)kt.k[0], (Cx<double>*)kt.k[1], (Cx<double>*)kt.k[2], h->n, h->stream));
    } else {
        rc = ensure_kin<float>(h, kt, dt, mass, fraction);
        if (!rc) CK(launch_kin_product<float>(reinterpret_cast<Cx<float>*>(dev), (Cx<float>*)kt.k[0], (Cx<float>*)kt.k[1], (Cx<float>*)kt.k[2], h->n, h->stream));
    }
    if (!to_device && !rc) CK(cudaMemcpyAsync(out, dev, h->count * h->elem, cudaMemcpyDeviceToHost, h->stream));
    cudaStreamSynchronize(h->stream);
    for (int a = 0; a < 3; ++a)
        if (kt.k[a]) cudaFree(kt.k[a]);
    if (!to_device) cudaFree(dev);
    return rc;
}

int wfs_potential_operator(wfs_handle* h, double dt, void* inout, int32_t on_device) {
    if (!h) return dispatch_err(h);
    if (!inout) return set_err(h, WFS_ERR_ARG, "null buffer");
    int rc = is_dbl(h) ? ensure_ephase<double>(h, dt) : ensure_ephase<float>(h, dt);
    if (rc) return rc;
    void* dev = inout;
    if (!on_device) {
        CK(cudaMalloc(&dev, h->count * h->elem));
        CK(cudaMemcpyAsync(dev, inout, h->count * h->elem, cudaMemcpyHostToDevice, h->stream));
    }
    cudaError_t e = is_dbl(h) ? launch_mul_inplace<double>((Cx<double>*)dev, (const Cx<double>*)h->ephase, h->count, h->stream)
                              : launch_mul_inplace<float>((Cx<float>*)dev, (const Cx<float>*)h->ephase, h->count, h->stream);
    if (e == cudaSuccess && !on_device) e = cudaMemcpyAsync(inout, dev, h->count * h->elem, cudaMemcpyDeviceToHost, h->stream);
    cudaStreamSynchronize(h->stream);
    if (!on_device) cudaFree(dev);
    if (e != cudaSuccess) return set_err(h, WFS_ERR_CUDA, std::string("potential_operator: ") + cudaGetErrorString(e));
    return WFS_OK;
}

int wfs_observe(wfs_handle* h, const wfs_box* boxes, int32_t nbox, const wfs_box* loc, double* prob_out, double* r_out, double* r2_out) {
    if (!h) return dispatch_err(h);
    return is_dbl(h) ? do_observe<double>(h, boxes, nbox, loc, prob_out, r_out, r2_out)
                     : do_observe<float>(h, boxes, nbox, loc, prob_out, r_out, r2_out);
}

int wfs_run_split_planes(wfs_handle* h, int32_t nsteps, double dt, double mass, int32_t interval, const wfs_box* boxes,
                         int32_t nbox, const wfs_box* loc, const wfs_plane* planes, int32_t nplane, double* prob_series,
                         double* loc_series, double* flux_series) {
    if (!h) return dispatch_err(h);
    return is_dbl(h) ? do_run_split<double>(h, nsteps, dt, mass, interval, boxes, nbox, loc, prob_series, loc_series,
                                            planes, nplane, flux_series)
                     : do_run_split<float>(h, nsteps, dt, mass, interval, boxes, nbox, loc, prob_series, loc_series,
                                           planes, nplane, flux_series);
}

int wfs_run_split(wfs_handle* h, int32_t nsteps, double dt, double mass, int32_t interval, const wfs_box* boxes, int32_t nbox,
                  const wfs_box* loc, double* prob_series, double* loc_series) {
    if (!h) return dispatch_err(h);
    if (nsteps < 0 || !(mass > 0) || !std::isfinite(dt)) return set_err(h, WFS_ERR_ARG, "invalid nsteps, dt or mass");
    return is_dbl(h) ? do_run_split<double>(h, nsteps, dt, mass, interval, boxes, nbox, loc, prob_series, loc_series)
                     : do_run_split<float>(h, nsteps, dt, mass, interval, boxes, nbox, loc, prob_series, loc_series);
}

int wfs_profile_enable(wfs_handle* h, int32_t stride) {
    if (!h) return dispatch_err(h);
    if (stride < 0) return set_err(h, WFS_ERR_ARG, "stride must be >= 0");
    h->prof_on = stride != 0;
    h->prof_stride = stride > 0 ? stride : 1;
    // event pairs are created here, outside any timed region
    while (h->prof_on && h->prof_pool.size() < 4096) {
        cudaEvent_t a, b;
        CK(cudaEventCreate(&a));
        CK(cudaEventCreate(&b));
        h->prof_pool.push_back({a, b});
    }
    return WFS_OK;
}

int wfs_profile_read(wfs_handle* h, double* ms_out, int64_t* count_out, int32_t reset) {
    if (!h) return dispatch_err(h);
    CK(cudaStreamSynchronize(h->stream));
    for (auto& pe : h->prof_live) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, pe.second.first, pe.second.second) == cudaSuccess) {
            h->prof_ms[pe.first] += ms;
            h->prof_count[pe.first] += 1;
        }
        h->prof_pool.push_back(pe.second);
    }
    h->prof_live.clear();
    for (int k = 0; k < WFS_NPASS; ++k) {
        if (ms_out) ms_out[k] = h->prof_ms[k];
        if (count_out) count_out[k] = h->prof_count[k];
        if (reset) { h->prof_ms[k] = 0.0; h->prof_count[k] = 0; }
    }
    return WFS_OK;
}

int wfs_set_schedule(wfs_handle* h, int32_t schedule) {
    if (!h) return dispatch_err(h);
    if (schedule < WFS_SCHEDULE_AUTO || schedule > WFS_SCHEDULE_PLANE) return set_err(h, WFS_ERR_ARG, "unknown schedule");
    if (schedule == WFS_SCHEDULE_PLANE && !plane_pass_supported(h->n[1], h->n[2]))
        return set_err(h, WFS_ERR_UNSUPPORTED, "plane schedule needs ny == nz in {32,48,64,96,128,192,256,384,512}");
    h->schedule = schedule;
    return WFS_OK;
}

int wfs_launch_count(wfs_handle* h, int64_t* out) {
    if (!h) return dispatch_err(h);
    if (!out) return set_err(h, WFS_ERR_ARG, "null output");
    *out = h->launches;
    return WFS_OK;
}

int wfs_split_step_gain(const int32_t n[3], int32_t dtype, double* g_x, double* g_yz) {
    if (!n || !g_x || !g_yz) return set_err(nullptr, WFS_ERR_ARG, "null argument");
    if (dtype != WFS_C64 && dtype != WFS_C128) return set_err(nullptr, WFS_ERR_ARG, "dtype must be WFS_C64 or WFS_C128");
    int nn[3];
    for (int a = 0; a < 3; ++a) {
        if (!fft_length_supported(n[a], dtype == WFS_C128))
            return set_err(nullptr, WFS_ERR_UNSUPPORTED, "axis length not supported by the split step");
        nn[a] = n[a];
    }
    if (dtype == WFS_C128) split_step_gains<double>(nn, g_x, g_yz);
    else split_step_gains<float>(nn, g_x, g_yz);
    return WFS_OK;
}

int wfs_plane_current(wfs_handle* h, const double center[3], const double normal[3], const double size[2],
                      const int32_t count[2], double mass, double* flux_out, void* density_out, int32_t to_device) {
    if (!h) return dispatch_err(h);
    if (!flux_out) return set_err(h, WFS_ERR_ARG, "null flux output");
    PlaneCurrentArgs a;
    double dW = 0, dH = 0;
    int rc = fill_plane(h, center, normal, size, count, mass, a, &dW, &dH);
    if (rc) return rc;
    rc = is_dbl(h) ? to_real<double>(h) : to_real<float>(h);
    if (rc) return rc;
    const int max_blocks = kPlaneCurrentBlocks;
    if ((rc = ensure_partials(h, max_blocks))) return rc;
    const size_t dbytes = size_t(a.sx) * a.sy * (is_dbl(h) ? sizeof(double) : sizeof(float));
    void* dens = nullptr;
    if (density_out) {
        if (to_device) dens = density_out;
        else CK(cudaMalloc(&dens, dbytes));
    }
    int grid = 0;
    cudaError_t e;
    {
        PassScope ps(h, WFS_PASS_OBSERVE);
        e = is_dbl(h) ? launch_plane_current<double>((const Cx<double>*)h->psi, a, h->partials, max_blocks, (double*)dens, h->stream, &grid)
                      : launch_plane_current<float>((const Cx<float>*)h->psi, a, h->partials, max_blocks, (float*)dens, h->stream, &grid);
    }
    if (e == cudaSuccess) e = launch_reduce_partials(h->partials, grid, 1, h->dres, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h->hres, h->dres, sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess && density_out && !to_device) e = cudaMemcpyAsync(density_out, dens, dbytes, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (density_out && !to_device && dens) cudaFree(dens);
    if (e != cudaSuccess) return set_err(h, WFS_ERR_CUDA, std::string("plane current: ") + cudaGetErrorString(e));
    *flux_out = h->hres[0] * dW * dH / 9.0;
    return WFS_OK;
}

int wfs_render(wfs_handle* h, const wfs_render_desc* desc, void* image, int32_t to_device) {
    if (!h) return dispatch_err(h);
    if (!desc || !image) return set_err(h, WFS_ERR_ARG, "invalid argument");
    if (desc->format != 0 && desc->format != 1) return set_err(h, WFS_ERR_ARG, "format must be 0 (RGBA8) or 1 (float)");
    if (desc->width < 1 || desc->height < 1 || int64_t(desc->width) * desc->height > (int64_t(1) << 28))
        return set_err(h, WFS_ERR_ARG, "invalid image size");
    if (desc->shadow_steps < 0 || desc->shadow_steps > 1000) return set_err(h, WFS_ERR_ARG, "shadow_steps must be in 0..1000");
    int rc = is_dbl(h) ? to_real<double>(h) : to_real<float>(h);
    if (rc) return rc;
    const size_t bytes = size_t(desc->width) * desc->height * (desc->format == 1 ? 16 : 4);
    void* dst = image;
    if (!to_device) CK(cudaMalloc(&dst, bytes));
    const int n[3] = {h->n[0], h->n[1], h->n[2]};
    cudaError_t e = is_dbl(h) ? launch_render<double>((const Cx<double>*)h->psi, (const float2*)h->V, n, *desc, dst, h->stream)
                              : launch_render<float>((const Cx<float>*)h->psi, (const float2*)h->V, n, *desc, dst, h->stream);
    if (e == cudaSuccess && !to_device) e = cudaMemcpyAsync(image, dst, bytes, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (!to_device) cudaFree(dst);
    if (e == cudaErrorInvalidValue) return set_err(h, WFS_ERR_ARG, "invalid camera or step");
    if (e != cudaSuccess) return set_err(h, WFS_ERR_CUDA, std::string("render: ") + cudaGetErrorString(e));
    return WFS_OK;
}

int wfs_norm(wfs_handle* h, double* norm_out) {
    if (!h) return dispatch_err(h);
    if (!norm_out) return set_err(h, WFS_ERR_ARG, "null output");
    int rc = is_dbl(h) ? to_real<double>(h) : to_real<float>(h);
    if (rc) return rc;
    if ((rc = ensure_partials(h, 152 * 8))) return rc;
    int nb = 0;
    CK(cudaMemsetAsync(h->dflag, 0, sizeof(int), h->stream));
    if (is_dbl(h)) CK(launch_norm<double>((const Cx<double>*)h->psi, h->count, h->partials, &nb, h->dflag, h->stream));
    else CK(launch_norm<float>((const Cx<float>*)h->psi, h->count, h->partials, &nb, h->dflag, h->stream));
    CK(launch_reduce_partials(h->partials, nb, 1, h->dres, h->stream));
    CK(cudaMemcpyAsync(h->hres, h->dres, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    int flag = 0;
    CK(cudaMemcpyAsync(&flag, h->dflag, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    *norm_out = h->hres[0] * h->dx[0] * h->dx[1] * h->dx[2];
    if (flag || !std::isfinite(*norm_out)) return set_err(h, WFS_ERR_NONFINITE, "psi holds NaN or Inf");
    return WFS_OK;
}

}  // extern "C"
