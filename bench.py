"""Benchmark: split-operator propagation, 256^3 complex64 double slit.

Workload (one "step" = one Strang split step): 256^3 grid over an 80-Bohr
cube, complex64; wall at x = 0, 1 Bohr thick, 20 Ha, two 2-Bohr slits at
y = +-3 along z; packet sigma 3, centre (-20, 0, 0), k0 (2.5, 0, 0);
16-cell quadratic absorber (-50 Ha); dt 0.01; the transmitted probability
P(x > 1) is recorded every 20 steps on the device (fused observation).
Synthetic, seeded, nothing is downloaded.

Printed JSON line (rank 0):
  value      site-steps/s, device-timed (CUDA events on the engine's stream),
             psi and the phase table resident in HBM (256 MiB > 129 MB L2, so
             no explicit L2 flush is needed between steps);
  e2e        the same metric through the public API with host buffers: psi0 and
             V uploaded from pinned host memory, the run, the series and psi read back;
  roofline   dominant pass (by device time, per-launch CUDA events in a separate
             untimed run of the same schedule, so no events sit in the timed
             region): algorithmic bytes per launch / mean launch time vs the
             measured HBM copy bandwidth;
  cpu_baseline  the NumPy oracle on one host core, on a bounded sample of steps.

--impl reference: the same workload on the host with the oracle split step
(scipy.fft with all host threads), each step a full 256^3 step; a bounded
number of steps is run so the arm ends within a few minutes.
Multi-GPU (torchrun): every rank propagates its own replica (the path does not
shard; replicas only); value = total site-steps / max rank time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N = 256
EXTENT = 80.0
DT = 0.01
OBS_INTERVAL = 20
SIGMA, R0, K0 = (3.0, 3.0, 3.0), (-20.0, 0.0, 0.0), (2.5, 0.0, 0.0)
ABS_CELLS = 16
ABS_POT = -50.0
METRIC = "site-steps/s at 256^3 c64 (split-step, double slit)"
PROFILE_STEPS = 40  # steps of the separate, untimed run that measures each pass


def engine_stream(torch):
    """A dedicated (non-default) stream shared by the engine and the timing events."""
    s = torch.cuda.Stream()
    torch.cuda.set_stream(s)
    return s


def workload_config():
    return {"workload": "double-slit split-step 256^3 complex64, 80 Bohr, dt 0.01, P(x>1) every 20 steps",
            "grid": [N, N, N], "dtype": "complex64", "obs_interval": OBS_INTERVAL,
            "l2": "working set psi 128 MiB + phase table 128 MiB > 129 MB L2 (no flush needed)"}


def transmitted_box():
    """P(x > 1) box as VolumeProbability builds it for corners (1,-35,-35)..(35,35,35)."""
    dx = EXTENT / N
    inner = EXTENT / 2 - ABS_CELLS * dx
    b = np.array([1.0, -inner, -inner])
    t = np.array([inner, inner, inner])
    bv = ((b + EXTENT / 2) / dx).astype(np.int64)
    tv = ((t + EXTENT / 2) / dx).astype(np.int64) + 1
    cnt = np.minimum(tv - bv, N - bv)
    cnt = np.where(cnt % 2 == 0, cnt - 1, cnt)
    return tuple(int(x) for x in bv), tuple(int(x) for x in cnt)


def build_engine(device=0, stream=None):
    from wavefunctionsimpython_gb300 import Engine

    dx = EXTENT / N
    inner = EXTENT / 2 - ABS_CELLS * dx
    e = Engine((N, N, N), (EXTENT,) * 3, double_precision=False, device=device, stream=stream)
    e.add_absorbing((-inner,) * 3, (inner,) * 3, 0.0, (ABS_POT,) * 3, (ABS_POT,) * 3, (2.0,) * 3, (2.0,) * 3)
    e.add_wall(20.0, (0.0, 0.0, 0.0), (1.0, 0.0, 0.0), 1.0, 0.0, 1.0, 2, 6.0, 2.0, math.pi / 2)
    e.init_gaussian(SIGMA, R0, K0)
    return e


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def ncu_traffic(kernel, table="bytes_per_launch"):
    """DRAM bytes (read + write) per launch of `kernel` from one ncu capture (or, with
    table="warp_instructions_per_launch", its warp instructions), or None."""
    tp = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if not os.path.exists(tp):
        return None
    with open(tp) as f:
        return json.load(f).get(table, {}).get(kernel)


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.file = None

    def __enter__(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.25)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            time.sleep(0.15)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or self.file is None:
            return None
        self.file.flush()
        rows = []
        with open(self.file.name) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.file.name)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "", 1).isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "", 1).isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        backend = "nccl" if args.impl == "own" else "gloo"
        if backend == "nccl":
            import torch

            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
        pg = dist
    return world, rank, local, pg


def max_over_ranks(pg, value, device=None):
    if pg is None:
        return value
    import torch

    t = torch.tensor([value], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def barrier(pg):
    if pg is not None:
        pg.barrier()


def cpu_split_sample(steps, workers=None):
    """Oracle split step at the full 256^3 c64 workload; returns (site-steps/s, seconds, steps)."""
    from oracle import wfs_oracle as orc

    dx = orc.delta_x((EXTENT,) * 3, (N, N, N))
    sc = orc.config3_double_slit(N, EXTENT)
    psi = sc.psi0()
    V = sc.potential()
    fft = None
    if workers is not None:
        import scipy.fft as sf

        fft = (lambda a, norm: sf.fftn(a, norm=norm, workers=workers),
               lambda a, norm: sf.ifftn(a, norm=norm, workers=workers))
    t0 = time.perf_counter()
    for _ in range(steps):
        psi = orc.split_step(psi, V, dx, DT, 1.0, nsteps=1, double_precision=False, fft=fft)
    t = time.perf_counter() - t0
    return N ** 3 * steps / t, t, steps


def run_reference(args):
    world, rank, local, pg = dist_setup(args)
    if rank != 0:
        return 0
    workers = os.cpu_count() or 1
    # bounded sample: at most ~90 s of CPU time in the timed part
    _, t1, _ = cpu_split_sample(1, workers)
    for _ in range(max(0, min(args.warmup, 1) - 1)):
        cpu_split_sample(1, workers)
    steps = max(1, min(args.steps, int(90.0 / max(t1, 1e-3))))
    value, t, steps = cpu_split_sample(steps, workers)
    line = {"metric": METRIC, "value": value, "unit": "site-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t / steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c64", "data": "synthetic", "config": workload_config(),
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "site-steps/s", "cores": workers, "kind": "port",
                             "sample": f"{steps} full 256^3 steps of the NumPy/SciPy oracle split step "
                                       f"(scipy.fft, workers={workers})"},
            "e2e": {"value": value, "unit": "site-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    gpu = reference_gpu_path(args)
    if gpu is not None:
        line["reference_gpu_path"] = gpu
    print(json.dumps(line))
    return 0


def reference_gpu_path(args):
    """The reference's own GPU path for this workload on this GPU, when its kernels were
    compiled (oracle/_ref): its kinetic and potential kernels and its packet and potential
    builders, launched on its own call sequence, with cuFFT (torch.fft, norm="ortho") for
    the transforms CuPy makes (sources/sim_state.py:641-697). Device-timed full 256^3
    steps; the P(x > 1) observation the reference makes every 20 steps is included."""
    try:
        import torch

        if not torch.cuda.is_available():
            return None
        from oracle import ref_gpu
        from oracle import wfs_oracle as orc

        if not ref_gpu.available():
            return None
    except Exception:  # noqa: BLE001 - the extra figure is optional
        return None
    torch.cuda.set_device(args.device)
    sc = orc.config3_double_slit(N, EXTENT)
    sim = ref_gpu.RefSim(sc.n, sc.extent, False, device=args.device)
    sim.build_scenario(sc)
    box = transmitted_box()
    steps = max(20, min(args.steps, 200))
    steps -= steps % OBS_INTERVAL

    def run(k):
        for i in range(k):
            if i % OBS_INTERVAL == 0:
                sim.volume_probability(*box)
            sim.split_step(DT, 1.0, 1, host_sync=True)

    run(max(args.warmup, 3))
    torch.cuda.synchronize()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record()
    run(steps)
    stop.record()
    torch.cuda.synchronize()
    ms = start.elapsed_time(stop) / steps
    return {"value": N ** 3 / (ms * 1e-3), "unit": "site-steps/s", "ms_per_step": ms, "steps": steps,
            "what": "the reference's own CUDA kernels (compiled unchanged) on its call sequence with its "
                    "per-step host synchronisation, cuFFT via torch.fft for its transforms, one GPU, complex64"}


def run_own(args):
    import torch

    world, rank, local, pg = dist_setup(args)
    dev = local if world > 1 else args.device
    torch.cuda.set_device(dev)
    stream = engine_stream(torch)
    box = transmitted_box()
    e = build_engine(dev, stream.cuda_stream)
    e.set_schedule(args.schedule)

    # warm-up (also allocates the observation buffers)
    e.run_split(max(args.warmup, 1), DT, 1.0, OBS_INTERVAL, [box], None)
    torch.cuda.synchronize()
    e.profile_enable(False)
    launches0 = e.launch_count()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev) as clk:
        barrier(pg)
        torch.cuda.synchronize()
        start.record(stream)
        probs, _ = e.run_split(args.steps, DT, 1.0, OBS_INTERVAL, [box], None)
        stop.record(stream)
        torch.cuda.synchronize()
        barrier(pg)
    ms = start.elapsed_time(stop)
    launches = e.launch_count() - launches0
    ms = max_over_ranks(pg, ms, device=f"cuda:{dev}" if world > 1 else None)
    # per-pass device times for the roofline: a separate, untimed run of the same
    # schedule with CUDA events around every launch (kept out of the timed region)
    e.profile_read(reset=True)
    e.profile_enable(True, stride=1)
    e.run_split(PROFILE_STEPS, DT, 1.0, OBS_INTERVAL, [box], None)
    torch.cuda.synchronize()
    prof = e.profile_read(reset=True)
    e.profile_enable(False)
    value = world * N ** 3 * args.steps / (ms * 1e-3)

    # roofline of the dominant pass
    peak, peak_kind = load_peaks()
    site_bytes = {"x_kin": 16, "y": 16, "z": 16, "z_vph": 24, "observe": 8, "plane": 24}
    dom = max((k for k in prof if k in site_bytes), key=lambda k: prof[k][0])
    dom_ms, dom_n = prof[dom]
    alg_bytes = site_bytes[dom] * N ** 3
    achieved = alg_bytes / (dom_ms / dom_n * 1e-3) / 1e9
    traffic = ncu_traffic(dom)
    passes = {k: {"ms_total": round(v[0], 4), "launches": v[1], "ms_mean": round(v[0] / v[1], 5)} for k, v in prof.items()}

    # end-to-end through the public API with pinned host buffers
    pinned_psi = torch.empty((N, N, N), dtype=torch.complex64, pin_memory=True)
    pinned_v = torch.empty((N, N, N), dtype=torch.complex64, pin_memory=True)
    psi0 = e.get_psi()
    v0 = e.get_potential()
    pinned_psi.numpy()[...] = psi0
    pinned_v.numpy()[...] = v0
    out_psi = torch.empty((N, N, N), dtype=torch.complex64, pin_memory=True)
    torch.cuda.synchronize()
    barrier(pg)
    t0 = time.perf_counter()
    e.set_potential(pinned_v.numpy())
    e.set_psi(pinned_psi.numpy())
    probs_e2e, _ = e.run_split(args.steps, DT, 1.0, OBS_INTERVAL, [box], None)
    e.get_psi(out=out_psi.numpy())
    t_e2e = time.perf_counter() - t0
    t_e2e = max_over_ranks(pg, t_e2e, device=f"cuda:{dev}" if world > 1 else None)
    e2e_value = world * N ** 3 * args.steps / t_e2e
    h2d = 2 * N ** 3 * 8 / args.steps
    d2h = (N ** 3 * 8 + probs_e2e.size * 8) / args.steps

    line = {"metric": METRIC, "value": value, "unit": "site-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c64", "data": "synthetic",
            "config": dict(workload_config(), schedule=args.schedule), "clocks": clk.summary(),
            "e2e": {"value": e2e_value, "unit": "site-steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": int(launches),
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_kind, "traffic": traffic,
                         "alg_bytes_per_launch": alg_bytes},
            "step_roofline_40B": {"achieved_gbs": value / world * 40 / 1e9, "frac": value / world * 40 / 1e9 / peak},
            "passes": passes,
            "transmitted_probability_last": float(probs[-1, 0]) if probs.size else None}
    if rank == 0 and not args.no_cpu_baseline:
        steps = 2
        v_cpu, t_cpu, steps = cpu_split_sample(steps)
        line["cpu_baseline"] = {"value": v_cpu, "unit": "site-steps/s", "cores": 1, "kind": "port",
                                "sample": f"{steps} full 256^3 steps of the NumPy oracle split step (pocketfft, 1 thread), {t_cpu:.1f} s"}
    if rank == 0:
        print(json.dumps(line))
    e.close()
    if pg is not None:
        pg.destroy_process_group()
    return 0


def run_taylor(args):
    """Power-series workload: 128^3 c64 over a 40-Bohr cube, harmonic oscillator
    w = 0.5, packet sigma 1.5 at (5,0,0), order 10, 4th-order Laplacian, dt 0.005."""
    import torch
    from wavefunctionsimpython_gb300 import Engine

    n, L, order = 128, 40.0, 10
    dx = L / n
    r = np.arange(n) * dx - L / 2
    V = (0.5 * 0.25 * (r[:, None, None] ** 2 + r[None, :, None] ** 2 + r[None, None, :] ** 2)).astype(np.complex64)
    torch.cuda.set_device(args.device)
    stream = engine_stream(torch)
    e = Engine((n, n, n), (L,) * 3, device=args.device, stream=stream.cuda_stream)
    e.set_potential(V)
    e.init_gaussian((1.5,) * 3, (5.0, 0.0, 0.0), (0.0, 0.0, 0.0))
    e.step_taylor(max(args.warmup, 1), 0.005, 1.0, order, 4)
    torch.cuda.synchronize()
    e.profile_enable(False)
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(args.device) as clk:
        torch.cuda.synchronize()
        start.record(stream)
        e.step_taylor(args.steps, 0.005, 1.0, order, 4)
        stop.record(stream)
        torch.cuda.synchronize()
    ms = start.elapsed_time(stop)
    # per-term device time from a separate, untimed run with events around each launch
    e.profile_read(reset=True)
    e.profile_enable(True, stride=1)
    e.step_taylor(min(args.steps, 20), 0.005, 1.0, order, 4)
    torch.cuda.synchronize()
    prof = e.profile_read(reset=True)
    e.profile_enable(False)
    peak, peak_kind = load_peaks()
    t_ms, t_n = prof["taylor"]
    achieved = 40 * n ** 3 / (t_ms / t_n * 1e-3) / 1e9
    hbm_view = {"achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                "alg_bytes_per_launch": 40 * n ** 3, "traffic": ncu_traffic("taylor"),
                "note": "DRAM bytes per launch from ncu: the 5 x 16 MiB working set stays in L2, so HBM is not "
                        "the bound"}
    # the kernel is issue bound while SMs are active: its warp instructions per launch (ncu)
    # over the live launch time, against one issue per scheduler per SM clock
    clocks = clk.summary()
    csum = clocks or {}
    mhz = csum.get("sm_mhz") or csum.get("sm_max_mhz") or 2070.0
    sms = torch.cuda.get_device_properties(args.device).multi_processor_count
    winst = ncu_traffic("taylor", "warp_instructions_per_launch")
    roof = {"bound": "issue", "kernel": "taylor", "unit": "G warp-instructions/s",
            "peak": sms * 4 * mhz * 1e6 / 1e9, "peak_source": f"{sms} SMs x 4 schedulers x {mhz:.0f} MHz (sampled)",
            "warp_instructions_per_launch": winst, "hbm_view": hbm_view}
    if winst:
        roof["achieved"] = winst / (t_ms / t_n * 1e-3) / 1e9
        roof["frac"] = roof["achieved"] / roof["peak"]
    line = {"metric": "site-steps/s at 128^3 c64 (power series, order 10, 4th-order Laplacian)",
            "value": n ** 3 * args.steps / (ms * 1e-3), "unit": "site-steps/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c64", "data": "synthetic",
            "config": {"workload": "harmonic oscillator power series 128^3 c64, p=10, 4th-order stencil, dt 0.005",
                       "l2": "working set 4 x 16 MiB fits in L2; term-to-term reuse is part of the design"},
            "clocks": clocks, "site_terms_per_s": n ** 3 * args.steps * order / (ms * 1e-3),
            "roofline": roof,
            "norm_after": e.norm()}
    print(json.dumps(line))
    return 0


BATCH_MIX = [(32, 128), (48, 64), (64, 48), (96, 16)]


def run_batch(args):
    """Batched sweep: 128x32^3, 64x48^3, 48x64^3, 16x96^3 over 40-Bohr cubes, complex64;
    per instance (seeded): barrier U[0.2,2] Ha, width U[1,4] Bohr, k0x U[0.5,3], sigma U[1,3],
    x0 U[-12,-6]; dt 0.01; one solve = 500 steps of every instance."""
    import torch
    from wavefunctionsimpython_gb300._lib import Batch

    rng = np.random.default_rng(2024)
    sizes = [n for n, cnt in BATCH_MIX for _ in range(cnt)]
    torch.cuda.set_device(args.device)
    stream = engine_stream(torch)
    b = Batch(sizes, [40.0] * len(sizes), device=args.device, stream=stream.cuda_stream)
    for i, n in enumerate(sizes):
        U, w = rng.uniform(0.2, 2.0), rng.uniform(1.0, 4.0)
        k0, sig, x0 = rng.uniform(0.5, 3.0), rng.uniform(1.0, 3.0), rng.uniform(-12.0, -6.0)
        b.add_wall(i, U, (0, 0, 0), (1, 0, 0), w)
        b.init_gaussian(i, (sig,) * 3, (x0, 0, 0), (k0, 0, 0))
    cl, sw, table = b.autotune(0.01, 1.0, steps=10)
    sites = sum(n ** 3 for n in sizes)
    steps = args.steps
    b.run(max(args.warmup, 3), 0.01, 1.0, graph=True)
    torch.cuda.synchronize()
    l0 = b.launch_count()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(args.device) as clk:
        torch.cuda.synchronize()
        start.record(stream)
        b.run(steps, 0.01, 1.0, graph=True)
        stop.record(stream)
        torch.cuda.synchronize()
    ms = start.elapsed_time(stop)
    launches = b.launch_count() - l0
    peak, peak_kind = load_peaks()
    value = sites * steps / (ms * 1e-3)
    # algorithmic HBM bytes per site-step of the tuned schedule: two passes per size class
    # (x pass 16 B, shared-memory plane pass 24 B) or one cluster launch (24 B, stages in L2)
    site_bytes = 40 if cl == 0 else 24
    achieved = site_bytes * sites / (ms / steps * 1e-3) / 1e9
    boxes = [((n // 2 + 1, 0, 0), (n // 2 - 1, n - 1, n - 1)) for n in sizes]
    probs = b.observe(boxes)
    line = {"metric": "batched site-steps/s (256 uneven instances, split step, c64)", "value": value,
            "unit": "site-steps/s", "n_gpus": 1, "steps": steps, "warmup": args.warmup, "ms_per_step": ms / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c64", "data": "synthetic",
            "config": {"workload": "batched sweep 128x32^3 + 64x48^3 + 48x64^3 + 16x96^3, 40 Bohr, dt 0.01",
                       "sites_per_step": sites, "cluster": cl, "radix_swap": sw, "graph": True,
                       "l2": "290 MiB of psi + 290 MiB of phase tables > 129 MB L2"},
            "solves_per_s": len(sizes) * 1000.0 / (ms / steps * 500),
            "autotune_ms_per_step": {f"cl{c}_swap{s}": v for (c, s), v in table.items()},
            "clocks": clk.summary(), "gpu_launches": int(launches),
            "roofline": {"bound": "hbm", "kernel": "batch step" if cl == 0 else "batch_kernel", "achieved": achieved,
                         "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                         "alg_bytes_per_step": site_bytes * sites,
                         "traffic": ncu_traffic("batch_two_pass" if cl == 0 else "batch"),
                         "traffic_note": "DRAM bytes per step from ncu"},
            "transmitted_probability_mean": float(np.mean(probs))}
    print(json.dumps(line))
    return 0


def surrogate_distribution(args, dist, stream):
    """Trains the FNO surrogate (64^3, width 32, 12 modes, 4 layers) on pairs from the plain
    split step of one scenario distribution, then measures held-out jumps of K = 50 steps
    against the exact propagator, the acceptance rate at the 1e-2 tolerance, and the
    effective speedup plain / (surrogate + rejected * plain + verified * plain). Inference
    (acceptance and timing) runs the kept-mode BF16 pass (FNO.forward_fast); the training
    forward's errors on the same seeds are reported beside it."""
    import ctypes

    import torch
    from wavefunctionsimpython_gb300 import fno as F

    if dist == "inband":
        # oscillators whose packets stay inside the 12 kept modes of a 24-Bohr box
        cfg = F.FnoConfig(extent=24.0, prior_steps=1)
        ranges = F.ScenarioRanges(p_wall=0.0, p_ho=1.0, omega=(0.2, 0.8), sigma=(1.0, 2.0), x0=(-3.0, -1.0),
                                  k0=(0.2, 1.0))
    else:
        # the batched sweep's barriers and oscillators on its 40-Bohr box
        cfg = F.FnoConfig(extent=40.0, prior_steps=2)
        ranges = F.ScenarioRanges()
    G, W, B = 64, 8, 8
    tol, verify_frac = 1e-2, 1.0 / 16
    chunk = G * W * 5
    nchunks = max(1, args.fno_pairs // chunk)
    model = F.FNO(cfg, seed=0, stream=stream)
    gen = F.PairGenerator(cfg, G, stream=stream)
    t_gen = t_train = 0.0
    # time a few training steps to turn the time budget into a step count
    t0 = time.perf_counter()
    data = F.make_dataset(cfg, chunk, W, G, seed=100, stream=stream, gen=gen, ranges=ranges)
    stream.synchronize()
    t_gen += time.perf_counter() - t0
    probe = F.FNO(cfg, seed=1, stream=stream)
    F.train(probe, data[:3], B, 5, 1e-4)
    t_probe = F.train(probe, data[:3], B, 20, 1e-4)["seconds"] / 20
    del probe
    total_steps = max(nchunks, int(args.fno_train_seconds / t_probe))
    per_chunk = total_steps // nchunks
    history, done = [], 0
    for c in range(nchunks):
        if c > 0:
            del data
            t0 = time.perf_counter()
            data = F.make_dataset(cfg, chunk, W, G, seed=100 + c, stream=stream, gen=gen, ranges=ranges)
            stream.synchronize()
            t_gen += time.perf_counter() - t0
        info = F.train(model, data[:3], B, per_chunk, args.fno_lr, warmup=200, log_every=max(1, per_chunk // 4),
                       seed=c, step_offset=done, total_steps=per_chunk * nchunks)
        done += info["steps"]
        t_train += info["seconds"]
        history += info["history"]
    del data
    torch.cuda.empty_cache()

    # held-out seeds: one random window per scenario
    rng = np.random.default_rng(777)
    e_net, e_f32, e_prior, n_err = [], [], [], []
    for g in range(args.fno_eval // G):
        held = F.make_dataset(cfg, G * W, W, G, seed=10_000 + g, stream=stream, gen=gen, ranges=ranges)
        rows = torch.tensor([int(rng.integers(W)) * G + i for i in range(G)], device=held[0].device)
        sel = tuple(torch.index_select(t, 0, rows) for t in held[:3])
        ev = F.evaluate(model, sel, batch=G, fast=True)
        e_net.append(ev["err_net"])
        e_prior.append(ev["err_prior"])
        n_err.append(ev["norm_err_net"])
        e_f32.append(F.evaluate(model, sel, batch=16)["err_net"])
        del held, sel
    e_net, e_f32, e_prior, n_err = (np.concatenate(e_net), np.concatenate(e_f32), np.concatenate(e_prior),
                                    np.concatenate(n_err))
    acc_net = (e_net <= tol) & (n_err <= tol)
    acc_prior = e_prior <= tol

    # cost of one jump per sample: plain (K exact steps) vs surrogate (coarse step + network)
    gen.setup(F.draw_scenarios(G, np.random.default_rng(5), ranges))
    T = cfg.jump_steps * cfg.dt
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn, reps):
        fn()
        stream.synchronize()
        ev0.record(stream)
        for _ in range(reps):
            fn()
        ev1.record(stream)
        stream.synchronize()
        return ev0.elapsed_time(ev1) / reps

    ms_plain = timed(lambda: gen.exact.run(cfg.jump_steps, cfg.dt, cfg.mass, graph=True), 5) / G
    ms_coarse = timed(lambda: gen.coarse.run(max(1, cfg.prior_steps), T / max(1, cfg.prior_steps), cfg.mass,
                                             graph=True), 10) / G if cfg.prior_steps else 0.0
    x = torch.zeros((G, 2, cfg.n3), dtype=torch.complex64, device=stream.device)
    psi = torch.zeros((G, cfg.n3), dtype=torch.complex64, device=stream.device)
    gen.snapshot(psi)
    prior = psi.clone()
    a2 = torch.empty(G, dtype=torch.float64, device=stream.device)
    lib = model.lib
    sp = ctypes.c_void_p(stream.cuda_stream)
    out = torch.empty_like(prior)
    out_norm = torch.zeros(G, dtype=torch.float64, device=stream.device)

    def infer():
        # |psi|^2 per sample (normalisation), then the jump on raw fields: the lift divides by
        # the RMS, the last layer adds s_b * network to the raw prior and accumulates |out|^2
        # for the norm test
        lib.wfs_fno_sample_norms(F._ptr(psi), None, cfg.n3, G, F._ptr(a2), None, sp)
        out_norm.zero_()
        model.jump_fast(psi, gen.V, prior, a2, G, out=out, out_norm=out_norm)

    def infer_f32():
        lib.wfs_fno_make_input(F._ptr(psi), F._ptr(gen.V), float(cfg.vscale), F._ptr(a2), F._ptr(x), G, cfg.n3, sp)
        for k in range(0, G, 16):
            model.forward(x[k:k + 16], prior[k:k + 16], 16, out=out[k:k + 16], keep_pre=False)

    ms_net = timed(infer, 5) / G
    ms_net_f32 = timed(infer_f32, 3) / G
    rej_net, rej_prior = 1.0 - acc_net.mean(), 1.0 - acc_prior.mean()
    ms_surr = ms_coarse + ms_net
    speed_net = ms_plain / (ms_surr + (rej_net + verify_frac) * ms_plain)
    speed_prior = ms_plain / (ms_coarse + (rej_prior + verify_frac) * ms_plain)
    nm = cfg.nmodes
    mix_flops = 2 * 4 * nm * cfg.width * cfg.width * cfg.layers  # fwd, per sample: 4 real MACs per complex MAC
    res = {"distribution": dist, "extent": cfg.extent, "prior_steps": cfg.prior_steps, "ranges": ranges.__dict__,
           "train_pairs": nchunks * chunk, "batch": B, "lr": args.fno_lr,
           "training": {"steps": done, "samples_seen": done * B, "seconds": t_train, "gen_seconds": t_gen,
                        "ms_per_step": 1e3 * t_train / max(1, done), "loss_history": history[-12:]},
           "held_out": {"seeds": int(e_net.size), "err_net_mean": float(e_net.mean()),
                        "err_net_median": float(np.median(e_net)),
                        "err_net_training_forward_mean": float(e_f32.mean()),
                        "err_prior_mean": float(e_prior.mean()), "err_prior_median": float(np.median(e_prior)),
                        "norm_err_net_max": float(n_err.max()), "accept_net": float(acc_net.mean()),
                        "accept_net_training_forward": float(((e_f32 <= tol) & (n_err <= tol)).mean()),
                        "accept_prior_only": float(acc_prior.mean())},
           "ms_per_jump_per_sample": {"plain": ms_plain, "coarse_prior": ms_coarse, "network": ms_net,
                                      "network_training_forward": ms_net_f32},
           "effective_speedup": {"surrogate": speed_net, "coarse_prior_only": speed_prior,
                                 "verify_fraction": verify_frac, "tolerance": tol},
           "network_only_site_jumps_per_s": cfg.n3 / (ms_net * 1e-3),
           "spectral_mixing_tflops": mix_flops / (ms_net * 1e-3) / 1e12}
    if not args.no_cpu_baseline:
        # FP64 NumPy oracle for two held-out jumps: accuracy of the exact engine and of the surrogate
        from oracle import wfs_oracle as orc

        held = F.make_dataset(cfg, G, 1, G, seed=20_000, stream=stream, gen=gen, ranges=ranges)
        pred = model.forward_fast(held[0][:2], held[1][:2], 2).cpu().numpy()
        xs, tg = held[0][:2].cpu().numpy(), held[2][:2].cpu().numpy()
        n3 = (cfg.N,) * 3
        dx = orc.delta_x((cfg.extent,) * 3, n3)
        t0 = time.perf_counter()
        errs = []
        for i in range(2):
            V = gen._potential(held[4][i]).astype(np.complex128)
            ex = orc.split_step(xs[i, 0].astype(np.complex128).reshape(n3), V, dx, cfg.dt, cfg.mass,
                                nsteps=cfg.jump_steps)
            nrm = np.linalg.norm(ex)
            errs.append({"engine_vs_fp64": float(np.linalg.norm(tg[i].reshape(n3) - ex) / nrm),
                         "surrogate_vs_fp64": float(np.linalg.norm(pred[i].reshape(n3) - ex) / nrm)})
        res["fp64_oracle_check"] = errs
        res["cpu_seconds_per_jump"] = (time.perf_counter() - t0) / 2
    del model, gen
    torch.cuda.empty_cache()
    return res


def run_surrogate(args):
    """FNO surrogate on the in-band distribution (the headline) and on the batched sweep's
    distribution (config 5's ranges), one JSON line."""
    import torch

    torch.cuda.set_device(args.device)
    stream = engine_stream(torch)
    dists = ["inband", "sweep"] if args.fno_dist == "both" else [args.fno_dist]
    res = {d: surrogate_distribution(args, d, stream) for d in dists}
    head = res[dists[0]]
    line = {"metric": "FNO surrogate effective speedup vs plain split step (K=50 jumps, 64^3 c64)",
            "value": head["effective_speedup"]["surrogate"], "unit": "x", "n_gpus": 1, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16 tensor-core products, f32 accumulation",
            "data": "synthetic",
            "config": {"workload": "FNO 64^3 width 32 modes 12 layers 4, K=50, jump = coarse prior + network",
                       "headline_distribution": dists[0]},
            "gpu_launches_per_jump": {"network": 9, "sample_norms": 2,
                                      "note": "lift, 4 x (mixing, layer), the last layer fused with both projections"},
            "distributions": res}
    if "cpu_seconds_per_jump" in head:
        line["cpu_baseline"] = {"value": 1.0 / head["cpu_seconds_per_jump"], "unit": "jumps/s", "cores": 1,
                                "kind": "port",
                                "sample": "2 held-out K=50 jumps of the FP64 NumPy split step (pocketfft, 1 thread)"}
    print(json.dumps(line))
    return 0


def run_render(args):
    """Headless volume view of the double slit after 200 steps: 1024 x 768 frames of psi and V
    (the reference's canvas size and step 0.1), without shadows and with the 50-step shadow march."""
    import torch
    from wavefunctionsimpython_gb300._lib import render_desc

    torch.cuda.set_device(args.device)
    stream = engine_stream(torch)
    e = build_engine(args.device, stream.cuda_stream)
    e.step_split(200, DT, 1.0)
    e.synchronize()
    out = {}
    for name, (w, h, shadows, reps) in {"frame_1024x768": (1024, 768, 0, 5),
                                         "frame_1024x768_shadows50": (1024, 768, 50, 1)}.items():
        d = render_desc(w, h, azimuth=30.0, shadow_steps=shadows)
        e.render(d)
        t0 = time.perf_counter()
        for _ in range(reps):
            img = e.render(d)
        out[name] = {"ms_per_frame": 1e3 * (time.perf_counter() - t0) / reps,
                     "mean_rgb": [float(v) for v in img[:, :, :3].reshape(-1, 3).mean(axis=0)]}
    line = {"metric": "headless volume render ms/frame (256^3 double slit, 1024x768, step 0.1 voxel)",
            "value": out["frame_1024x768"]["ms_per_frame"], "unit": "ms", "n_gpus": 1, "higher_is_better": False,
            "dtype": "f32", "data": "synthetic", "config": {"workload": "ray march of psi and V, host round trip included"},
            "frames": out}
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=["own", "reference"], default="own")
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--schedule", choices=["auto", "axis", "plane"], default="auto",
                    help="split-step schedule: fused yz-plane pass (auto) or one pass per axis")
    ap.add_argument("--workload", choices=["split", "taylor", "batch", "surrogate", "render"], default="split",
                    help="split: the headline 256^3 double slit; taylor: the 128^3 power-series workload; "
                         "batch: the 256-instance uneven sweep; surrogate: train and measure the FNO jump; "
                         "render: headless volume view frames")
    ap.add_argument("--fno-dist", choices=["inband", "sweep", "both"], default="both",
                    help="surrogate scenarios: oscillators inside the kept modes, the sweep's barriers and "
                         "oscillators on a 40-Bohr box, or both (one line, the in-band run as the headline)")
    ap.add_argument("--fno-train-seconds", type=float, default=240.0)
    ap.add_argument("--fno-pairs", type=int, default=20480)
    ap.add_argument("--fno-eval", type=int, default=2048)
    ap.add_argument("--fno-lr", type=float, default=1e-3)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "taylor":
        return run_taylor(args)
    if args.workload == "batch":
        return run_batch(args)
    if args.workload == "surrogate":
        return run_surrogate(args)
    if args.workload == "render":
        return run_render(args)
    return run_own(args)


if __name__ == "__main__":
    sys.exit(main())
