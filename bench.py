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
  roofline   dominant pass (by device time inside the timed region, per-launch
             CUDA events): algorithmic bytes per launch / mean launch time vs the
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
PROFILE_STRIDE = 10  # per-launch CUDA events on every 10th step of long timed regions


def profile_stride(steps):
    """Event sampling stride: every 10th step of long runs, every step of short ones."""
    return PROFILE_STRIDE if steps >= 20 * PROFILE_STRIDE else 1


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
    print(json.dumps(line))
    return 0


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
    e.profile_read(reset=True)
    e.profile_enable(True, stride=profile_stride(args.steps))
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
    prof = e.profile_read(reset=True)
    e.profile_enable(False)
    ms = max_over_ranks(pg, ms, device=f"cuda:{dev}" if world > 1 else None)
    value = world * N ** 3 * args.steps / (ms * 1e-3)

    # roofline of the dominant pass
    peak, peak_kind = load_peaks()
    site_bytes = {"x_kin": 16, "y": 16, "z": 16, "z_vph": 24, "observe": 8, "plane": 24}
    dom = max((k for k in prof if k in site_bytes), key=lambda k: prof[k][0])
    dom_ms, dom_n = prof[dom]
    alg_bytes = site_bytes[dom] * N ** 3
    achieved = alg_bytes / (dom_ms / dom_n * 1e-3) / 1e9
    traffic = None
    tp = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if os.path.exists(tp):
        with open(tp) as f:
            traffic = json.load(f).get("bytes_per_launch", {}).get(dom)
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
    e.step_taylor(args.warmup, 0.005, 1.0, order, 4)
    torch.cuda.synchronize()
    e.profile_read(reset=True)
    e.profile_enable(True, stride=profile_stride(args.steps))
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(args.device) as clk:
        torch.cuda.synchronize()
        start.record(stream)
        e.step_taylor(args.steps, 0.005, 1.0, order, 4)
        stop.record(stream)
        torch.cuda.synchronize()
    ms = start.elapsed_time(stop)
    prof = e.profile_read(reset=True)
    peak, peak_kind = load_peaks()
    t_ms, t_n = prof["taylor"]
    achieved = 40 * n ** 3 / (t_ms / t_n * 1e-3) / 1e9
    line = {"metric": "site-steps/s at 128^3 c64 (power series, order 10, 4th-order Laplacian)",
            "value": n ** 3 * args.steps / (ms * 1e-3), "unit": "site-steps/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c64", "data": "synthetic",
            "config": {"workload": "harmonic oscillator power series 128^3 c64, p=10, 4th-order stencil, dt 0.005",
                       "l2": "working set 4 x 16 MiB fits in L2; term-to-term reuse is part of the design"},
            "clocks": clk.summary(), "site_terms_per_s": n ** 3 * args.steps * order / (ms * 1e-3),
            "roofline": {"bound": "hbm", "kernel": "taylor", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_kind, "alg_bytes_per_launch": 40 * n ** 3,
                         "traffic": None},
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
    achieved = 24 * sites / (ms / steps * 1e-3) / 1e9
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
            "roofline": {"bound": "hbm", "kernel": "batch_kernel", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_kind, "alg_bytes_per_launch": 24 * sites,
                         "traffic": None},
            "transmitted_probability_mean": float(np.mean(probs))}
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
    ap.add_argument("--workload", choices=["split", "taylor", "batch"], default="split",
                    help="split: the headline 256^3 double slit; taylor: the 128^3 power-series workload; "
                         "batch: the 256-instance uneven sweep")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "taylor":
        return run_taylor(args)
    if args.workload == "batch":
        return run_batch(args)
    return run_own(args)


if __name__ == "__main__":
    sys.exit(main())
