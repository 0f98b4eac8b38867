/*
 * wfs.h — C ABI of the GB300-native wave-function propagation engine.
 *
 * Plain C: pointers, sizes and status codes only. One handle owns one grid
 * (psi, the complex64 potential, phase tables and scratch) on one CUDA
 * device and one stream. Handles are not thread-safe; use one per host
 * thread. Every entry point returns 0 (WFS_OK) or a WFS_ERR_* code; the
 * message is read with wfs_last_error(h) (or wfs_global_error() when no
 * handle exists yet).
 *
 * Each declaration names the reference interface it replaces (paths are
 * relative to the WaveFunctionSimPython project root). The reference has no
 * native FFI; its Python call surface (SimState, operators,
 * MeasurementTools, core_sim) binds these through ctypes.
 */
#ifndef WFS_H
#define WFS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define WFS_ABI_VERSION 1

typedef struct wfs_handle wfs_handle;

enum wfs_status {
    WFS_OK = 0,
    WFS_ERR_ARG = 1,          /* invalid argument (shape, size, null pointer) */
    WFS_ERR_CUDA = 2,         /* a CUDA runtime call failed */
    WFS_ERR_TIMEOUT = 3,      /* a bounded device-side wait gave up */
    WFS_ERR_NONFINITE = 4,    /* NaN/Inf or norm blow-up detected in psi */
    WFS_ERR_UNSUPPORTED = 5,  /* axis length or configuration not supported */
    WFS_ERR_STATE = 6         /* call made in a state that does not allow it */
};

enum wfs_dtype { WFS_C64 = 0, WFS_C128 = 1 };

/* Element types accepted by wfs_potential_add_raw
 * (sources/potential.py:26-39: float32, float64, complex64, complex128). */
enum wfs_raw_type { WFS_RAW_F32 = 0, WFS_RAW_F64 = 1, WFS_RAW_C64 = 2, WFS_RAW_C128 = 3 };

/* Grid description. Replaces the volume/precision part of SimState.__init__
 * (sources/sim_state.py:83-94): number_of_voxels_3, simulated_volume_dimensions_bohr_radii_3,
 * double_precision_calculation. psi is C-ordered [x][y][z]. */
typedef struct {
    int32_t n[3];       /* voxels per axis; each a product of 2s and 3s, 2..1024 */
    double extent[3];   /* simulated volume in Bohr radii (delta_x = extent / n) */
    int32_t dtype;      /* WFS_C64 or WFS_C128 */
    int32_t device;     /* CUDA device ordinal */
    void* stream;       /* cudaStream_t to launch on, or NULL for an engine-owned stream */
} wfs_grid_desc;

/* One potential wall: sources/potential.py:161-198 (PotentialWall). */
typedef struct {
    double potential_hartree;
    double center[3];
    double normal[3];             /* need not be normalised */
    double plateau_thickness;
    double slope_thickness;
    double slope_exponent;
    int32_t slit_count;           /* 0..4 */
    double slit_spacing;
    double slit_width;
    double slit_rotation;         /* radians */
} wfs_wall;

/* Absorbing boundary: sources/potential.py:57-106 (AbsorbingBoundaryCondition). */
typedef struct {
    double bottom[3];             /* inner box corners in Bohr radii */
    double top[3];
    double offset;                /* start_offset */
    double potential_pos[3];      /* outer_potential_in_positive_xyz_direction_hartree_3 */
    double potential_neg[3];
    double exponent_pos[3];       /* slope_exponent_in_positive_xyz_direction_3 */
    double exponent_neg[3];
} wfs_absorbing;

/* Simpson sample box in voxels: first voxel and (odd) sample count per axis.
 * Built the way sources/measurement.py:101-116 and :320-329 build it. */
typedef struct {
    int32_t bottom[3];
    int32_t count[3];
} wfs_box;

int wfs_abi_version(void);
const char* wfs_global_error(void);

/* SimState(config) allocation of psi and V (sources/sim_state.py:63-183, :222-227). */
int wfs_create(const wfs_grid_desc* desc, wfs_handle** out);
int wfs_destroy(wfs_handle* h);
const char* wfs_last_error(const wfs_handle* h);
/* Waits for the handle's stream. Propagation calls are asynchronous; a copy-staged
 * pass whose bounded wait for a tile copy gave up is reported here, by wfs_get_psi
 * and by the observation calls as WFS_ERR_TIMEOUT (the status is then cleared). */
int wfs_synchronize(wfs_handle* h);
/* Limit of a copy-staged pass's wait for a staged tile, in seconds (default 1; at most
 * 60). A limit of zero makes every such wait give up at once: the pass then stops
 * without storing, and the next wfs_synchronize reports WFS_ERR_TIMEOUT once. This is
 * the test hook for the expiry path; it has no counterpart in the reference, whose
 * transforms are library calls. */
int wfs_set_copy_wait_limit(wfs_handle* h, double seconds);

/* Potential construction (sources/sim_state.py:210-255). */
int wfs_potential_clear(wfs_handle* h);                                   /* V.fill(0): sources/potential.py:510 */
int wfs_potential_add_wall(wfs_handle* h, const wfs_wall* w);              /* PotentialWall.add_potential: sources/potential.py:201-242 */
int wfs_potential_add_absorbing(wfs_handle* h, const wfs_absorbing* a);    /* AbsorbingBoundaryCondition.add_potential: sources/potential.py:108-158 */
int wfs_potential_add_raw(wfs_handle* h, const void* data, int32_t raw_type, int32_t on_device); /* PreInitializedPotential.add_potential: sources/potential.py:47-55 */
/* Dynamic potential mode: SimState.update_potential (sources/sim_state.py:466-509) with
 * generate_potential_from_walls_and_drain (sources/potential.py:508-522). After every
 * later step (split or power series) each wall's centre moves by velocity * dt (3 values
 * per wall, Bohr per hbar/Hartree) with its x clamped at 0, and V becomes the walls plus
 * the absorbing ramp (NULL: none). The first update rebuilds V whole, dropping any
 * pre-initialised potential as the reference's rebuild does; later updates rewrite only
 * the voxels a moving wall covered before or covers after the move (V and the phase
 * table), so the step loop stays on the device. nwall = 0 ends the mode; at most 8 walls. */
int wfs_set_dynamic_walls(wfs_handle* h, const wfs_wall* walls, const double* velocity, int32_t nwall,
                          const wfs_absorbing* absorbing);
/* Current centres of the dynamic walls, 3 per wall (nwall must equal the number set). */
int wfs_get_dynamic_walls(wfs_handle* h, double* centers, int32_t nwall);
int wfs_set_potential(wfs_handle* h, const void* v_c64, int32_t on_device);
int wfs_get_potential(wfs_handle* h, void* v_c64, int32_t to_device);

/* Wave function (sources/sim_state.py:185-208, :309-313; sources/wave_packet.py:217-271). */
int wfs_init_gaussian(wfs_handle* h, const double sigma[3], const double r0[3], const double k0[3]);
int wfs_set_psi(wfs_handle* h, const void* psi, int32_t on_device);
int wfs_get_psi(wfs_handle* h, void* psi, int32_t to_device);
/* Device pointer of psi in real space (materialises any pending split-step
 * state first). Valid until the next propagation call. */
int wfs_psi_device_ptr(wfs_handle* h, void** ptr);

/* Propagators: SimState.evolve_state (sources/sim_state.py:754-762). */
/* nsteps Strang steps: SimState._fft_time_evolution (sources/sim_state.py:641-697). */
int wfs_step_split(wfs_handle* h, int32_t nsteps, double dt, double mass);
/* nsteps power-series steps: SimState._power_series_time_evolution (sources/sim_state.py:721-752).
 * stencil_order 2 reproduces power_series_operator.cu:50-58; 4 is the 4th-order Laplacian. */
int wfs_step_taylor(wfs_handle* h, int32_t nsteps, double dt, double mass, int32_t order, int32_t stencil_order);

/* Operators module (sources/operators.py:9-55). */
/* Writes exp(-i |k|^2 dt fraction / m) (fraction 0.25 = the reference's half step,
 * kinetic_operator.cu:21-23) into out (psi dtype, N elements). */
int wfs_kinetic_operator(wfs_handle* h, double dt, double mass, double fraction, void* out, int32_t to_device);
/* inout *= cexp_i(-dt V) (potential_operator.cu:11-15); inout has psi dtype. */
int wfs_potential_operator(wfs_handle* h, double dt, void* inout, int32_t on_device);

/* Observables (sources/measurement.py:153-188 VolumeProbability, :354-400 ExpectedLocation).
 * prob_out[nbox]; loc may be NULL, else r_out[3] = <r>, r2_out[3] = <r^2>. FP64 accumulation. */
int wfs_observe(wfs_handle* h, const wfs_box* boxes, int32_t nbox, const wfs_box* loc,
                double* prob_out, double* r_out, double* r2_out);

/* Driver loop fused on the device: core_sim.run_iteration (sources/core_sim.py:26-65)
 * for the split-step method. Before step i (i = 0, interval, 2*interval, ... < nsteps)
 * the observables are recorded, as time_step does (sources/core_sim.py:19-24):
 * prob_series[rec*nbox + b], loc_series[rec*6 + (0..2 = <r>, 3..5 = <r^2>)].
 * The series arrays hold ceil(nsteps / interval) records. */
int wfs_run_split(wfs_handle* h, int32_t nsteps, double dt, double mass, int32_t interval,
                  const wfs_box* boxes, int32_t nbox, const wfs_box* loc,
                  double* prob_series, double* loc_series);

/* Sampling plane of a probability current (PlaneProbabilityCurrent,
 * sources/measurement.py:190-256): centre and normal in Bohr radii, extent
 * size[2] and odd Simpson sample counts count[2]. */
typedef struct {
    double center[3];
    double normal[3];
    double size[2];
    int32_t count[2];
} wfs_plane;

/* wfs_run_split plus plane probability currents: before every interval-th step
 * the flux through each plane is recorded too, flux_series[rec*nplane + p], all
 * on the device (MeasurementTools.measure_and_render with plane currents,
 * sources/measurement.py:644-705). With planes, the observables are taken from
 * real-space psi. */
int wfs_run_split_planes(wfs_handle* h, int32_t nsteps, double dt, double mass, int32_t interval,
                         const wfs_box* boxes, int32_t nbox, const wfs_box* loc, const wfs_plane* planes,
                         int32_t nplane, double* prob_series, double* loc_series, double* flux_series);

/* Probability flux through a sampled plane: PlaneProbabilityCurrent.calculate
 * (sources/measurement.py:258-289, probability_current_density.cu:11-218).
 * count[2] are the (odd) Simpson sample counts, size[2] the plane's extent in
 * Bohr radii. flux_out = integral of j.n over the plane; density_out (optional,
 * count[0]*count[1] values in psi's real precision, to host or device memory)
 * receives the sampled current density. */
int wfs_plane_current(wfs_handle* h, const double center[3], const double normal[3], const double size[2],
                      const int32_t count[2], double mass, double* flux_out, void* density_out, int32_t to_device);

/* FP64 norm sum |psi|^2 dV over the whole grid; WFS_ERR_NONFINITE when psi holds NaN/Inf. */
int wfs_norm(wfs_handle* h, double* norm_out);

/* Instrumentation (no counterpart in the reference, which only times the host
 * loop, sources/core_sim.py:43-49). When enabled, every kernel launch of the
 * engine is bracketed by CUDA events on the engine's stream; wfs_profile_read
 * synchronises and returns the accumulated device milliseconds and launch
 * counts per pass kind (WFS_NPASS entries each). */
enum wfs_pass_kind {
    WFS_PASS_X_KIN = 0,     /* x pencils: Fx, kinetic factor, Fx^-1 */
    WFS_PASS_Y = 1,         /* y pencils: Fy or Fy^-1 */
    WFS_PASS_Z_VPH = 2,     /* z rows: Fz^-1, potential phase, Fz */
    WFS_PASS_Z = 3,         /* z rows: Fz or Fz^-1 */
    WFS_PASS_OBSERVE = 4,   /* fused or standalone observation reduction */
    WFS_PASS_TAYLOR = 5,    /* one power-series term */
    WFS_PASS_OTHER = 6,     /* reductions, phase tables */
    WFS_PASS_PLANE = 7,     /* yz planes: Fy^-1, Fz^-1, potential phase, Fz, Fy */
    WFS_NPASS = 8
};
/* stride: 0 off; k >= 1 brackets the launches of every k-th step (and the
 * launches outside steps made while that step count is current). */
int wfs_profile_enable(wfs_handle* h, int32_t stride);
int wfs_profile_read(wfs_handle* h, double* ms_out, int64_t* count_out, int32_t reset);
/* Split-step schedule (no counterpart in the reference). AUTO uses the fused
 * yz-plane pass (2 HBM round trips per step) where the plane shape allows it,
 * else one pass per axis (4 round trips); AXIS forces the per-axis passes. */
enum wfs_schedule { WFS_SCHEDULE_AUTO = 0, WFS_SCHEDULE_AXIS = 1, WFS_SCHEDULE_PLANE = 2 };
int wfs_set_schedule(wfs_handle* h, int32_t schedule);
/* Number of kernels the engine has launched since creation. */
int wfs_launch_count(wfs_handle* h, int64_t* out);
/* Mean energy gain of one split step's transforms on an n[0] x n[1] x n[2] grid of dtype
 * (WFS_C64 or WFS_C128), as built from rounded constants: *g_x for the x pass (two x
 * transforms), *g_yz for the y/z work (two y and two z transforms). The engine divides
 * its kinetic x factors by their square roots (one x pass and one y/z set per step).
 * No counterpart in the reference: it reports the compensation of complex64 rounding
 * that keeps long runs on the complex128 trajectory. Host-only; needs no GPU. */
int wfs_split_step_gain(const int32_t n[3], int32_t dtype, double* g_x, double* g_yz);

/* ------------------------------------------------------------------------
 * Batched sweep: many independent packets on uneven cubic grids advanced
 * together (no counterpart in the reference, which runs one simulation per
 * process, sources/core_sim.py:26-65; each instance follows the same split
 * step as wfs_step_split). complex64 only; sizes 32, 48, 64, 96, 128. One
 * kernel launch per step advances every instance; runs can be captured in a
 * CUDA graph. Instance builders mirror the single-grid ones.
 * ---------------------------------------------------------------------- */
typedef struct wfs_batch wfs_batch;
typedef struct {
    int32_t ninst;
    const int32_t* n;        /* ninst cube edge lengths */
    const double* extent;    /* ninst cube edge lengths in Bohr radii */
    int32_t device;
    void* stream;            /* cudaStream_t or NULL */
} wfs_batch_desc;

int wfs_batch_create(const wfs_batch_desc* desc, wfs_batch** out);
int wfs_batch_destroy(wfs_batch* b);
const char* wfs_batch_last_error(const wfs_batch* b);
int wfs_batch_synchronize(wfs_batch* b);
int wfs_batch_init_gaussian(wfs_batch* b, int32_t i, const double sigma[3], const double r0[3], const double k0[3]);
int wfs_batch_add_wall(wfs_batch* b, int32_t i, const wfs_wall* w);
int wfs_batch_add_absorbing(wfs_batch* b, int32_t i, const wfs_absorbing* a);
int wfs_batch_set_potential(wfs_batch* b, int32_t i, const void* v_c64, int32_t on_device);
int wfs_batch_set_psi(wfs_batch* b, int32_t i, const void* psi_c64, int32_t on_device);
int wfs_batch_get_psi(wfs_batch* b, int32_t i, void* psi_c64, int32_t to_device);
/* nsteps Strang steps of every instance; use_graph != 0 replays a captured CUDA graph. */
int wfs_batch_run(wfs_batch* b, int32_t nsteps, double dt, double mass, int32_t use_graph);
/* One Simpson volume probability per instance: boxes[i] -> prob_out[i]. */
int wfs_batch_observe(wfs_batch* b, const wfs_box* boxes, double* prob_out);
/* Step schedule and radix orientation (0: P >= Q, 1: swapped). cluster 0 (the
 * default): two passes per step and size class, an x pass and a plane pass that holds
 * each yz-plane whole in one CTA's shared memory; cluster 1, 2, 4, 8 or 16: one launch
 * per step, one cluster of that many CTAs per instance, stages through L2. */
int wfs_batch_set_config(wfs_batch* b, int32_t cluster, int32_t swap);
/* Times every configuration over `steps` steps and keeps the fastest (psi is restored);
 * ms_out (optional, 12 entries) receives ms per step for cluster {0,1,2,4,8,16} x swap {0,1},
 * -1 where a configuration cannot be scheduled. */
int wfs_batch_autotune(wfs_batch* b, double dt, double mass, int32_t steps, int32_t* cluster_out, int32_t* swap_out,
                       double* ms_out);
int wfs_batch_launch_count(wfs_batch* b, int64_t* out);

/* ------------------------------------------------------------------------
 * Allocation-free observation. No counterpart in the reference: it exists for
 * callers that may not allocate device memory (a host application whose own
 * allocator owns the GPU, real-time loops that must not take allocator locks,
 * plugins that only receive device pointers) and so cannot create a handle.
 * Same results as wfs_observe for a real-space psi the caller owns on the
 * current device: out_device[0..nbox) = volume probabilities, and when loc is
 * not NULL out_device[nbox..nbox+3) = <r>, out_device[nbox+3..nbox+6) = <r^2>.
 * Asynchronous on `stream` (NULL = legacy default stream); calls no
 * allocating routine. Scratch is one fixed device array of
 * WFS_NOALLOC_SCRATCH_DOUBLES doubles (1 MiB per GPU, held until exit):
 * grids with ceil(nx*ny/8) * (nbox + (loc ? 7 : 0)) > WFS_NOALLOC_SCRATCH_DOUBLES - 16
 * are rejected with WFS_ERR_UNSUPPORTED. The first call in each CUDA context
 * (once per device for runtime-API callers) looks up the array's address and
 * caches it under the context's unique ID, so a context created after
 * cudaDeviceReset or a non-primary context gets its own lookup; make that
 * first call before any stream capture. Calls share the array: calls that
 * overlap on the GPU race. Message: wfs_global_error().
 * ---------------------------------------------------------------------- */
#define WFS_NOALLOC_SCRATCH_DOUBLES 131072
int wfs_observe_noalloc(const void* psi_device, int32_t dtype, const int32_t n[3], const double extent[3],
                        const wfs_box* boxes, int32_t nbox, const wfs_box* loc, double* out_device, void* stream);

/* ------------------------------------------------------------------------
 * Headless volume rendering of psi and V (replaces the vispy/GLSL view of
 * sources/volumetric_visualization.py:38-200 and
 * sources/multi_volume_shaders.py:200-390 with a CUDA ray march into an image
 * buffer; no graphics API). Row-major image, height x width pixels.
 * ---------------------------------------------------------------------- */
typedef struct wfs_render_desc {
    int32_t width, height;        /* image size (the reference's canvas: 1024 x 768) */
    double azimuth_deg;           /* turntable camera around the +y axis (array axis 1) */
    double elevation_deg;         /* the reference's default: 45 */
    double fov_deg;               /* the reference's default: 45 */
    double distance;              /* camera distance in voxels; <= 0 fits the volume */
    double relative_step;         /* ray step in voxels (the reference: 0.1) */
    double wave_function_scale;   /* |Re psi|, |Im psi| mapped to [-1, 1]; <= 0 means 0.005 */
    double potential_scale;       /* <= 0: max |V| over its real and imaginary parts */
    double light[3];              /* direction towards the light (the reference: 1, 1, -1) */
    int32_t shadow_steps;         /* 0: no shadows; the reference marches 50 (0..1000) */
    int32_t show_potential;       /* 1: render V's volume too */
    int32_t format;               /* 0: RGBA8 (4 bytes per pixel), 1: RGBA float32 */
} wfs_render_desc;

/* Renders the handle's psi (materialised first) and V into `image`
 * (width * height * 4 bytes for RGBA8, 16 for float; host or device memory). */
int wfs_render(wfs_handle* h, const wfs_render_desc* desc, void* image, int32_t to_device);

/* The same for caller-owned device arrays: psi (complex64/complex128, [n0][n1][n2])
 * and V (complex64, may be NULL); asynchronous on `stream`. */
int wfs_render_volume(const void* psi_device, int32_t dtype, const int32_t n[3], const void* potential_device,
                      const wfs_render_desc* desc, void* image_device, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* WFS_H */
