#!/usr/bin/env python3
"""Benchmark of the GB300 synchrotron path.

Workload (one step): the synchrotron spectra of a Tristan-v2 dump-scale particle
set -- 3 species (e-, e+, p) x 3.3e7 particles = 9.9e7 particles, 512 log photon
bins 1e-4..1e9 mec^2, FP32 SoA four-velocities with |u| a power law of index -2.2
on [1, 1e4] times exp(-gamma/3e3) and isotropic directions, magnetic fields with
log-normal (0, 0.5) magnitude and isotropic directions, weights uniform on
[0.5, 1.5].  e- and e+ share the scalars B0 = g_syn = e_syn_at_g_syn = 1 and run
as one batched launch over two segments; protons use e_syn_at_g_syn / 1836.
Inputs are generated on the device from fixed seeds (synthetic; positions are
not an input of the spectrum and are not generated).

Reported: evals/s = particles x bins of spectrum produced per second (value:
device-resident inputs; e2e: host-resident pinned inputs through
rg_spectrum_run_host, H2D of the inputs and D2H of the spectra inside the timed
region every step, steps pipelined; the step-synchronous figure and a copy-only /
kernel-only breakdown beside it).  The plans sum by interval moments (the default
for reference-table particle plans): one particle stage per particle deposits FP64
moments per (table cell, bin interval), then a scan and a per-bin reduce; the
roofline is that of the deposit kernel (HBM: 28 algorithmic bytes per particle).
The fused per-eval kernel (every particle x bin pair in FP32) runs the same step
as a side case with its FP32-issue roofline.  Also: per-species error of the
headline spectra against the FP64 oracle, the CPU baseline, clocks.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""

from __future__ import annotations

import argparse
import glob
import json
import math
import os
import re
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "synchrotron particle×bin evals/s, fwd and fwd+adjoint vs plain GPU at 1e-5 rel"
UNIT = "evals/s"
NSPECIES = 3
N_PER_SPECIES = 33_000_000
NBINS = 512
BIN_LO, BIN_HI = 1e-4, 1e9
PROTON_MASS_RATIO = 1836.0
OPS_PER_EVAL = 6  # fused kernel: IADD, SHF, LOP, LDS.64, FFMA (F), FFMA (accumulate)
BYTES_PER_PARTICLE = 28  # u (12 B), B (12 B), w (4 B), FP32 SoA, read once per deposit


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the side cases (plain kernel, batched graph, adjoint, GEMM, Adam fit, histogram, "
                         "IC, the drop-in module calls)")
    ap.add_argument("--ref-seconds", type=float, default=90.0,
                    help="CPU seconds the reference arm spreads over its warm-up and timed steps")
    ap.add_argument("--cpu-seconds", type=float, default=12.0,
                    help="target CPU time of the cpu_baseline sample")
    ap.add_argument("--profile-case", nargs="?", const="spectrum",
                    choices=["spectrum", "spectrum200", "smooth", "smooth_moments", "gemm", "histogram", "ic",
                             "moments"],
                    help="small case for ncu captures, then exit: 'spectrum' = one 4.19e6-particle "
                         "species x 512 bins, 4 fused-kernel launches; 'gemm' = 4096 distributions x "
                         "1024 gamma bins x 1024 photon bins, 4 tcgen05 GEMM launches; 'histogram' = "
                         "energyDistribution of 3.3e7 particles into 200 log bins, 4 calls; 'ic' = "
                         "ICSpectrum 1024 x 1024 x 1024, 4 calls; 'moments' = one 2^24-particle species "
                         "x 512 bins by interval moments, 4 runs (deposit, scan, reduce); 'smooth' / "
                         "'smooth_moments' = the smooth table, 4 forward + 4 adjoint runs, fused kernels on "
                         "2^22 particles / cell moments on 2^24 particles")
    return ap.parse_args()


# ---------------------------------------------------------------------------------------
# synthetic inputs
# ---------------------------------------------------------------------------------------

def powerlaw_cutoff_torch(torch, n, gen, device, index=-2.2, lo=1.0, hi=1e4, gcut=3e3):
    """|u| ~ |u|^index on [lo, hi] times exp(-gamma/gcut), by rejection."""
    q = index + 1.0
    out = torch.empty(0, device=device)
    while out.numel() < n:
        m = int((n - out.numel()) * 1.1) + 1024
        r = torch.rand(m, device=device, generator=gen, dtype=torch.float64)
        u = ((hi**q - lo**q) * r + lo**q) ** (1.0 / q)
        acc = torch.rand(m, device=device, generator=gen, dtype=torch.float64) < torch.exp(
            -torch.sqrt(1.0 + u * u) / gcut)
        out = torch.cat([out, u[acc].float()])
    return out[:n]


def isotropic_torch(torch, mag, gen):
    n = mag.numel()
    mu = torch.rand(n, device=mag.device, generator=gen) * 2.0 - 1.0
    ph = torch.rand(n, device=mag.device, generator=gen) * (2.0 * math.pi)
    s = torch.sqrt(torch.clamp(1.0 - mu * mu, min=0.0))
    return [mag * s * torch.cos(ph), mag * s * torch.sin(ph), mag * mu]


def make_particles(torch, n_per, nspecies, device, seed):
    """SoA component tensors (u1..u3, b1..b3, w) holding all species back to back."""
    comps = [torch.empty(n_per * nspecies, device=device) for _ in range(7)]
    for s in range(nspecies):
        gen = torch.Generator(device=device).manual_seed(seed * 101 + s)
        u = isotropic_torch(torch, powerlaw_cutoff_torch(torch, n_per, gen, device), gen)
        b = isotropic_torch(torch, torch.exp(0.5 * torch.randn(n_per, device=device, generator=gen)), gen)
        w = torch.rand(n_per, device=device, generator=gen) + 0.5
        for k, v in enumerate(u + b + [w]):
            comps[k][s * n_per:(s + 1) * n_per] = v
    return comps


def make_particles_numpy(n, seed):
    import numpy as np  # noqa: PLC0415

    rng = np.random.default_rng(seed)
    q = -1.2
    out = np.empty(0)
    while out.size < n:
        m = int((n - out.size) * 1.1) + 1024
        u = ((1e4**q - 1.0) * rng.random(m) + 1.0) ** (1.0 / q)
        out = np.concatenate([out, u[rng.random(m) < np.exp(-np.sqrt(1 + u * u) / 3e3)]])
    umag = out[:n]

    def iso(mag):
        mu = rng.uniform(-1, 1, n)
        ph = rng.uniform(0, 2 * np.pi, n)
        s = np.sqrt(1 - mu**2)
        return [(mag * s * np.cos(ph)).astype(np.float32), (mag * s * np.sin(ph)).astype(np.float32),
                (mag * mu).astype(np.float32)]

    u = iso(umag)
    b = iso(rng.lognormal(0.0, 0.5, n))
    # the reference has no per-particle weight: the CPU sample runs with w = 1
    return {"ux": u[0], "uy": u[1], "uz": u[2], "bx": b[0], "by": b[1], "bz": b[2]}


def photon_bins():
    import numpy as np  # noqa: PLC0415

    from ragnar_gb300 import capi  # noqa: PLC0415

    bins = np.empty(NBINS, np.float32)
    capi.check(capi.lib().rg_logspace(BIN_LO, BIN_HI, NBINS, bins.ctypes.data))
    return bins


def photon_bins_cpu():
    """The same 512 photon bins for the CPU legs, from the oracle's Logspace (bit-identical
    to the library's): a CPU-only process must not load the product library."""
    import oracle  # noqa: PLC0415

    return oracle.logspace(BIN_LO, BIN_HI, NBINS)


# ---------------------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------------------

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50", "-i", str(self.gpu)],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.1)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), float(parts[3]), parts[5:9]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i, v in enumerate(r[3]) if v.lower().startswith("active")})
        loaded = [r[0] for r in rows if r[2] > 200.0] or [r[0] for r in rows]
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows), "power_w_max": max(r[2] for r in rows)}


# ---------------------------------------------------------------------------------------
# CPU baseline: the reference's own build when importable, else the oracle port
# ---------------------------------------------------------------------------------------

def cpu_spectrum_runner():
    """Returns (kind, fn(P, bins) -> spectrum, threads)."""
    import oracle  # noqa: PLC0415

    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    ref_so = glob.glob(os.path.join(ROOT, "oracle", "_ref", "ragnar*.so"))
    if ref_so:
        try:
            import importlib.util  # noqa: PLC0415

            spec = importlib.util.spec_from_file_location("ragnar", ref_so[0])
            rg = importlib.util.module_from_spec(spec)
            spec.loader.exec_module(rg)
            rg.Initialize()

            def run_ref(P, bins):
                prt = rg.Particles_3D("bench")
                prt.fromArrays({"U1": P["ux"], "U2": P["uy"], "U3": P["uz"],
                                "B1": P["bx"], "B2": P["by"], "B3": P["bz"]})
                b = rg.Bins(bins, rg.EnergyUnits.mec2)
                return rg.SynchrotronSpectrum_3D(prt, b, 1.0, 1.0, 1.0).as_array()

            return "reference", run_ref, threads
        except Exception:  # noqa: BLE001 - built for another machine
            pass
    oracle.build()
    table = oracle.tabulate_ffunc()

    def run_port(P, bins):
        return oracle.sync_spectrum_ref32(P, bins, 1.0, 1.0, 1.0, table)

    return "port", run_port, threads


def cpu_baseline(target_seconds: float):
    kind, fn, threads = cpu_spectrum_runner()
    bins = photon_bins_cpu()
    # calibrate on a small sample, then time one bounded sample of ~target_seconds
    calib = make_particles_numpy(20000, seed=7)
    t0 = time.perf_counter()
    fn(calib, bins)
    rate = 20000 * NBINS / max(time.perf_counter() - t0, 1e-6)
    n = int(min(max(rate * target_seconds / NBINS, 20000), 2e7))
    P = make_particles_numpy(n, seed=8)
    t0 = time.perf_counter()
    fn(P, bins)
    dt = time.perf_counter() - t0
    return {"value": n * NBINS / dt, "unit": UNIT, "cores": threads, "kind": kind,
            "sample": f"{n} particles of the e- species x {NBINS} bins (one spectrum, {dt:.1f} s)"}


def run_reference_arm(args, rank):
    if rank != 0:
        return
    kind, fn, threads = cpu_spectrum_runner()
    bins = photon_bins_cpu()
    calib = make_particles_numpy(20000, seed=7)
    t0 = time.perf_counter()
    fn(calib, bins)
    rate = 20000 * NBINS / max(time.perf_counter() - t0, 1e-6)
    per_step = max(args.ref_seconds / max(args.steps + args.warmup, 1), 0.2)
    n = int(min(max(rate * per_step / NBINS, 20000), 2e7))
    P = make_particles_numpy(n, seed=9)
    for _ in range(args.warmup):
        fn(P, bins)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        fn(P, bins)
    dt = (time.perf_counter() - t0) / max(args.steps, 1)
    value = n * NBINS / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded numpy sample of the same workload)",
        "config": workload_config(),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind,
                         "sample": f"each step: {n} particles of the e- species x {NBINS} bins"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def workload_config():
    return {
        "workload": "tristan-v2 dump scale: synchrotron spectra of 3 species x 3.3e7 particles, "
                    "512 log photon bins 1e-4..1e9 mec2",
        "particles": NSPECIES * N_PER_SPECIES, "photon_bins": NBINS, "species": ["e-", "e+", "p"],
        "u": "power law -2.2 on [1,1e4] x exp(-gamma/3e3), isotropic",
        "B": "log-normal(0,0.5) magnitude, isotropic", "weights": "U[0.5,1.5]",
        "scalars": {"B0": 1.0, "g_syn": 1.0, "e_syn_at_g_syn": {"e-": 1.0, "e+": 1.0, "p": 1 / 1836.0}},
        "l2": "inputs 2.77 GB per step > 129 MB L2 (no flush needed)",
        "parallelism": "one rank per GPU, each with its own particle set (weak scaling)",
    }


# ---------------------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------------------

def profile_value(key):
    """A figure from the committed ncu summaries (a line '- key: value')."""
    for path in sorted(glob.glob(os.path.join(ROOT, "profiles", "*.md"))):
        m = re.search(r"(?m)^- " + re.escape(key) + r":\s*([0-9.eE+-]+)", open(path).read())
        if m:
            return float(m.group(1))
    return None


def traffic_per_particle():
    """DRAM bytes per particle of the fused kernel from the committed ncu summary."""
    return profile_value("dram_bytes_per_particle")


def wavefronts_per_eval():
    """Shared-memory wavefronts per eval of the fused kernel from the committed ncu summary."""
    return profile_value("shared_wavefronts_per_eval")


def run_ours(args, rank, world, local_rank):
    import numpy as np  # noqa: PLC0415
    import torch  # noqa: PLC0415

    from ragnar_gb300 import capi, shard  # noqa: PLC0415

    dist = world > 1
    device = torch.device("cuda", local_rank)
    torch.cuda.set_device(device)
    capi.check(capi.lib().rg_init(local_rank))
    sms = torch.cuda.get_device_properties(device).multi_processor_count
    stream = torch.cuda.current_stream(device).cuda_stream

    n_per = N_PER_SPECIES
    comps = make_particles(torch, n_per, NSPECIES, device, seed=1000 + rank)
    bins = photon_bins()
    u, b, w = comps[0:3], comps[3:6], comps[6]
    prt_all = capi.particles(u, b=b, w=w, n=NSPECIES * n_per)
    off = 2 * n_per
    prt_p = capi.particles([c[off:] for c in u], b=[c[off:] for c in b], w=w[off:], n=n_per)
    plan_e = capi.SpectrumPlan(bins, 1.0, 1.0, 1.0)
    plan_p = capi.SpectrumPlan(bins, 1.0, 1.0, 1.0 / PROTON_MASS_RATIO)
    plan_e.reserve(2)
    offs_e = torch.tensor([0, n_per, 2 * n_per], dtype=torch.int64, device=device)
    out_e = torch.empty((2, NBINS), device=device)
    out_p = torch.empty(NBINS, device=device)

    def step():
        plan_e.run_batched(prt_all, offs_e, 2, out_e, stream)
        plan_p.run(prt_p, out_p, stream)

    evals_per_step = NSPECIES * n_per * NBINS
    launches_per_step = 6  # deposit + scan + reduce, for the e+- batch and for the protons

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    plan_e.check(stream)
    plan_p.check(stream)
    if dist:
        torch.distributed.barrier()
    plan_e.enable_timing(True)
    plan_p.enable_timing(True)
    sampler = ClockSampler(local_rank)
    sampler.start()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        step()
    e1.record()
    torch.cuda.synchronize()
    clocks = sampler.stop()
    t_step = e0.elapsed_time(e1) / 1e3 / max(args.steps, 1)
    ke_ms, ke_n = plan_e.kernel_time()
    kp_ms, kp_n = plan_p.kernel_time()
    plan_e.enable_timing(False)
    plan_p.enable_timing(False)
    plan_e.check(stream)
    plan_p.check(stream)
    spectra_ok = bool(torch.isfinite(out_e).all() and torch.isfinite(out_p).all() and out_e.sum() > 0)
    if dist:
        t_step = shard.max_over_ranks(t_step, device)
    device_spectra = torch.cat([out_e, out_p[None]]).cpu().numpy()
    parity = guarded(headline_parity, torch, capi, comps, n_per, bins, plan_e, plan_p, stream) \
        if rank == 0 else None

    # deposit-kernel roofline: HBM, 28 algorithmic bytes per particle (u, B, w read once)
    clk = clocks.get("sm_mhz") or 2070.0
    roofline = deposit_roofline(ke_ms + kp_ms, ke_n + kp_n, NSPECIES * n_per, sms, clk)

    result = {
        "metric": METRIC, "value": world * evals_per_step / t_step, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_step * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded, generated on the device)", "config": workload_config(),
        "roofline": roofline, "gpu_launches": launches_per_step * args.steps, "clocks": clocks,
    }

    if parity is not None:
        result["parity_vs_fp64"] = parity
    extra = {"spectra_finite": spectra_ok}
    if rank == 0 and not args.no_extras:
        extra["fused_per_eval_same_step"] = guarded(fused_same_step, torch, plan_e, plan_p, step, stream, sms,
                                                    evals_per_step, max(args.steps // 2, 3))
        extra["energy_distribution_dump"] = guarded(histogram_case, torch, capi, device, comps, NSPECIES * n_per)
        extra["dropin_module_3.3e7"] = guarded(dropin_module_case, torch, comps, n_per)
    # e2e: host-resident pinned inputs through the C ABI, copies inside the timed region
    if not args.no_e2e:
        host = [torch.empty(c.numel(), dtype=torch.float32, pin_memory=True) for c in comps]
        for h, c in zip(host, comps):
            h.copy_(c)
        breakdown = {"kernel_only": guarded(kernel_only_steps, torch, capi, comps, n_per,
                                            [plan_e, plan_e, plan_p], stream, max(args.steps, 1))}
        del comps, u, b, w
        torch.cuda.empty_cache()
        breakdown["copy_only"] = guarded(copy_only_steps, torch, host, n_per, device, max(args.steps, 1))
        depth = 3  # steps in flight when pipelined
        houts = [torch.empty((3, NBINS), dtype=torch.float32, pin_memory=True) for _ in range(depth)]
        douts = [torch.empty((3, NBINS), device=device) for _ in range(depth)]
        done = [torch.cuda.Event() for _ in range(depth)]
        species = []
        for s in range(NSPECIES):
            sl = slice(s * n_per, (s + 1) * n_per)
            species.append(capi.host_particles([h[sl] for h in host[0:3]], b=[h[sl] for h in host[3:6]],
                                               w=host[6][sl], n=n_per))
        plans = [plan_e, plan_e, plan_p]

        def enqueue(i):
            d, h = douts[i % depth], houts[i % depth]
            for s in range(NSPECIES):
                plans[s].run_host(species[s], d[s], stream)
            h.copy_(d, non_blocking=True)
            done[i % depth].record(torch.cuda.current_stream(device))

        def read(i):
            done[i % depth].synchronize()
            return bool(torch.isfinite(houts[i % depth]).all())

        def run_pipelined(k):
            # steps i+1 .. i+depth-1 are enqueued before step i's spectra are read back, so
            # the host link and the kernels do not wait on the host between steps
            ok = True
            for i in range(k):
                enqueue(i)
                if i >= depth - 1:
                    ok = read(i - depth + 1) and ok
            for i in range(max(0, k - depth + 1), k):
                ok = read(i) and ok
            return ok

        def run_synchronous(k):
            ok = True
            for i in range(k):
                enqueue(i)
                ok = read(i) and ok
            return ok

        def timed_e2e(fn):
            fn(max(args.warmup, 3))
            if dist:
                torch.distributed.barrier()
            t0 = time.perf_counter()
            ok = fn(max(args.steps, 1))
            t = (time.perf_counter() - t0) / max(args.steps, 1)
            if dist:
                t = shard.max_over_ranks(t, device)
            return t, ok

        # per-step wall times of the synchronous form (host stalls on a shared machine show
        # up as rare slow steps; the median is reported beside the mean-based values)
        def step_times(k):
            ts = []
            for i in range(k):
                t0 = time.perf_counter()
                enqueue(i)
                read(i)
                ts.append(time.perf_counter() - t0)
            return ts

        t_e2e, ok_p = timed_e2e(run_pipelined)
        t_sync, ok_s = timed_e2e(run_synchronous)
        e2e_steps = step_times(max(args.steps, 1))
        t_med = statistics.median(e2e_steps)
        breakdown["e2e_step_synchronous"] = step_stats(e2e_steps)
        # the host path's spectra against the device-resident ones of the same particles
        # (the chunks sum in another order, so they agree to FP32 rounding, not bit for bit)
        e2e_spectra = houts[(max(args.steps, 1) - 1) % depth].numpy().astype("float64")
        ref_spectra = device_spectra.astype("float64")
        nz = ref_spectra > 1e-12 * ref_spectra.max(axis=1, keepdims=True)
        breakdown["e2e_vs_device_max_rel_diff"] = float(
            (abs(e2e_spectra - ref_spectra)[nz] / ref_spectra[nz]).max())
        spectra_ok = spectra_ok and ok_p and ok_s
        extra["spectra_finite"] = spectra_ok
        result["e2e"] = {"value": world * evals_per_step / t_e2e, "unit": UNIT,
                         "h2d_bytes_per_step": 7 * 4 * NSPECIES * n_per,
                         "d2h_bytes_per_step": 4 * NSPECIES * NBINS,
                         "ms_per_step": t_e2e * 1e3,
                         "value_step_synchronous": world * evals_per_step / t_sync,
                         "ms_per_step_synchronous_median": t_med * 1e3,
                         "breakdown": breakdown,
                         "path": "rg_spectrum_run_host per species (pinned host SoA, chunked H2D through the "
                                 "device's staging pipeline, overlapped with the fused kernel) + D2H of the "
                                 "3 spectra every step; steps pipelined (up to 3 steps enqueued before the "
                                 "oldest one's spectra are read on the host); value_step_synchronous waits "
                                 "for each step's spectra before enqueuing the next"}
        plan_e.check(stream)
        plan_p.check(stream)
        del host

    # context beside the headline: the plain one-spectrum-per-launch kernel on one
    # species, and the 1e6-particle x 200-bin configuration (fused and plain)
    if rank == 0 and not args.no_extras:
        extra.update(guarded(side_measurements, torch, capi, device, stream))
        extra["batched_graph_256_segments"] = guarded(batched_graph_case, torch, capi, device)
        extra["fwd_adjoint_1e7x512"] = guarded(fwd_adjoint_case, torch, capi, device)
        peak_bf16, peak_src = measured_peak("bf16_tflops", 1900.0)
        extra["fromdist_gemm_4096x1024x1024"] = guarded(fromdist_gemm_case, torch, capi, device, peak_bf16)
        extra["fromdist_gemm_4096x1024x1024"]["peak_source"] = peak_src
        extra["adam_fit_1024x512x512"] = guarded(adam_fit_case, torch, capi, device)
        extra["ic_1024x1024x1024"] = guarded(ic_case, torch, capi, device, clocks.get("sm_mhz") or 2070.0)
        add_wavefront_rooflines(extra, sms, clocks.get("sm_mhz") or 2070.0)
        fa = extra["fwd_adjoint_1e7x512"]
        if "moments" in fa:
            # the metric's second figure: forward + adjoint of the differentiable spectrum
            result["fwd_plus_adjoint"] = {
                "value": fa["moments"]["fwd_plus_adjoint_evals_per_s"], "unit": UNIT,
                "workload": "1e7 particles x 512 bins 0.01..1e7, smooth table; dL/dw and dL/du",
                "ms": fa["moments"]["fwd_plus_adjoint_ms"], "roofline": fa["moments"]["roofline"],
                "fused_per_eval_value": fa["fused"].get("fwd_plus_adjoint_evals_per_s"),
                "plain_fwd_value": fa["plain_fwd_evals_per_s"]}
        if not args.no_cpu_baseline:
            result["cpu_baseline"] = cpu_baseline(args.cpu_seconds)
    result["extra"] = extra
    plan_e.close()
    plan_p.close()
    if rank == 0:
        print(json.dumps(result), flush=True)


def deposit_roofline(ms_total, launches, particles_per_step, sms, clk_mhz):
    """HBM roofline of the interval-moment deposit kernel over the timed steps: 28
    algorithmic bytes per particle (u, B, w read once) against the measured copy
    bandwidth; the secondary line is its instruction issue rate (thread instructions
    per particle from the committed ncu summary) against SMs x 128 lanes x clock."""
    ms = ms_total / max(launches, 1)
    steps = max(launches, 1) / 2.0  # two deposits per step: the e+- batch and the protons
    bytes_per_launch = BYTES_PER_PARTICLE * particles_per_step / 2.0
    achieved = BYTES_PER_PARTICLE * particles_per_step * steps / (ms_total / 1e3) / 1e9
    peak, src = measured_peak("hbm_gbs", 6800.0)
    dbp = profile_value("moments_dram_bytes_per_particle")
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "peak_source": src, "kernel": "moments_deposit_kernel", "kernel_ms_per_launch": ms,
            "bytes_per_launch": bytes_per_launch,
            "bytes_basis": f"{BYTES_PER_PARTICLE} B per particle (u, B, w, FP32) x particles per launch",
            "traffic": None if dbp is None else dbp * particles_per_step / 2.0}
    ipp = profile_value("moments_thread_inst_per_particle")
    if ipp:
        rate = ipp * particles_per_step * steps / (ms_total / 1e3)
        issue_peak = sms * 128 * clk_mhz * 1e6
        roof["secondary"] = {"bound": "instruction issue", "achieved": rate / 1e12, "peak": issue_peak / 1e12,
                             "unit": "T thread-instructions/s", "frac": rate / issue_peak,
                             "basis": f"{ipp} thread instructions per particle (ncu, committed summary) vs "
                                      f"{sms} SMs x 128 lanes x {clk_mhz:.0f} MHz"}
    return roof


def fused_same_step(torch, plan_e, plan_p, step, stream, sms, evals_per_step, k):
    """The headline step with the fused per-eval kernel (every particle x bin pair in
    FP32): evals/s and its FP32-issue roofline (6 FP32-pipe ops per eval against SMs x
    128 lanes x clock), the measure the per-eval design is bound by."""
    for p in (plan_e, plan_p):
        p.set_algorithm(1)
    try:
        for _ in range(2):
            step()
        torch.cuda.synchronize()
        plan_e.enable_timing(True)
        plan_p.enable_timing(True)
        sampler = ClockSampler(torch.cuda.current_device())
        sampler.start()
        t = timed(torch, step, k, warm=0)
        clocks = sampler.stop()
        ke_ms, ke_n = plan_e.kernel_time()
        kp_ms, kp_n = plan_p.kernel_time()
        plan_e.enable_timing(False)
        plan_p.enable_timing(False)
        plan_e.check(stream)
        plan_p.check(stream)
    finally:
        for p in (plan_e, plan_p):
            p.set_algorithm(0)
    kern_ms = (ke_ms + kp_ms) / max(ke_n + kp_n, 1)
    evals_per_launch = evals_per_step / 2.0
    clk = clocks.get("sm_mhz") or 2070.0
    achieved = OPS_PER_EVAL * evals_per_launch / (kern_ms / 1e3) / 1e12
    peak = sms * 128 * clk * 1e6 / 1e12
    out = {"evals_per_s": evals_per_step / t, "ms_per_step": t * 1e3, "kernel_ms_per_launch": kern_ms,
           "clocks": clocks,
           "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "Top/s",
                        "frac": achieved / peak, "kernel": "fused_spectrum_kernel<16>",
                        "basis": f"{OPS_PER_EVAL} FP32-pipe ops per eval vs {sms} SMs x 128 lanes x "
                                 f"{clk:.0f} MHz"}}
    wpe = wavefronts_per_eval()
    if wpe:
        lsu_peak = sms * clk * 1e6 / wpe
        out["roofline_shared_memory"] = {
            "bound": "shared-memory wavefronts", "achieved": evals_per_launch / (kern_ms / 1e3),
            "peak": lsu_peak, "unit": "evals/s", "frac": evals_per_launch / (kern_ms / 1e3) / lsu_peak,
            "basis": f"{sms} SMs x {clk:.0f} MHz / {wpe} wavefronts per eval (ncu, committed summary)"}
    return out


def step_stats(ts):
    """Mean, median and 95th percentile of per-step wall times, in ms."""
    s = sorted(ts)
    return {"steps": len(s), "mean_ms": 1e3 * sum(s) / len(s), "median_ms": 1e3 * statistics.median(s),
            "p95_ms": 1e3 * s[min(len(s) - 1, int(math.ceil(0.95 * len(s))) - 1)]}


def kernel_only_steps(torch, capi, comps, n_per, plans, stream, k):
    """The e2e step without its input copies: the three species' spectra from
    device-resident particles (one rg_spectrum_run each) and the D2H read of the three
    spectra, each step waited for (host wall clock per step)."""
    device = comps[0].device
    species = []
    for s in range(NSPECIES):
        sl = slice(s * n_per, (s + 1) * n_per)
        species.append(capi.particles([c[sl] for c in comps[0:3]], b=[c[sl] for c in comps[3:6]],
                                      w=comps[6][sl], n=n_per))
    d = torch.empty((NSPECIES, NBINS), device=device)
    h = torch.empty((NSPECIES, NBINS), dtype=torch.float32, pin_memory=True)

    def one():
        for s in range(NSPECIES):
            plans[s].run(species[s], d[s], stream)
        h.copy_(d, non_blocking=True)
        torch.cuda.current_stream(device).synchronize()

    for _ in range(3):
        one()
    ts = []
    for _ in range(k):
        t0 = time.perf_counter()
        one()
        ts.append(time.perf_counter() - t0)
    return step_stats(ts)


def copy_only_steps(torch, host, n_per, device, k, chunk=1 << 22):
    """The e2e step's input copies without its kernels: the same 7 components x 3 species
    in the same 2^22-particle chunks, pinned host -> two alternating device staging
    buffers on one copy stream (as the library's host staging issues them), each step
    waited for (host wall clock per step)."""
    stage = [torch.empty((len(host), chunk), device=device) for _ in range(2)]
    cs = torch.cuda.Stream(device)

    def one():
        i = 0
        with torch.cuda.stream(cs):
            for s in range(NSPECIES):
                for a in range(0, n_per, chunk):
                    m = min(chunk, n_per - a)
                    buf = stage[i % 2]
                    for c, hc in enumerate(host):
                        buf[c, :m].copy_(hc[s * n_per + a:s * n_per + a + m], non_blocking=True)
                    i += 1
        cs.synchronize()

    for _ in range(3):
        one()
    ts = []
    for _ in range(k):
        t0 = time.perf_counter()
        one()
        ts.append(time.perf_counter() - t0)
    out = step_stats(ts)
    out["bytes_per_step"] = 4 * len(host) * NSPECIES * n_per
    out["gbs_median"] = out["bytes_per_step"] / (out["median_ms"] * 1e-3) / 1e9
    return out


def headline_parity(torch, capi, comps, n_per, bins, plan_e, plan_p, stream, m=1_000_000):
    """Per-bin error of the headline spectra against the FP64 oracle, per species: the
    last m e- particles and the first m e+ particles as two segments of the e+- plan's
    batched launch, the first m protons through the proton plan (e_syn_at_g_syn / 1836),
    weights included; the oracle (FP64 restatement of synchrotron.cpp:107-145) runs on the
    same particles.  Error = max over bins above 1e-12 of the peak of |S - S64| / S64."""
    import numpy as np  # noqa: PLC0415

    import oracle  # noqa: PLC0415

    device = comps[0].device
    offs = torch.tensor([n_per - m, n_per, n_per + m], dtype=torch.int64, device=device)
    prt = capi.particles(comps[0:3], b=comps[3:6], w=comps[6], n=NSPECIES * n_per)
    got_e = torch.empty((2, NBINS), device=device)
    plan_e.run_batched(prt, offs, 2, got_e, stream)
    p0 = 2 * n_per
    sl = slice(p0, p0 + m)
    prt_p = capi.particles([c[sl] for c in comps[0:3]], b=[c[sl] for c in comps[3:6]], w=comps[6][sl], n=m)
    got_p = torch.empty(NBINS, device=device)
    plan_p.run(prt_p, got_p, stream)
    torch.cuda.synchronize()
    plan_e.check(stream)
    plan_p.check(stream)
    table = oracle.tabulate_ffunc()
    keys = ("ux", "uy", "uz", "bx", "by", "bz", "w")
    res = {"particles_per_species": m, "bins_compared": "bins above 1e-12 of the species' peak",
           "oracle": "FP64 restatement of the reference path (float table and bins as data)"}
    t0 = time.perf_counter()
    for name, a, eps, got in (("e-", n_per - m, 1.0, got_e[0]), ("e+", n_per, 1.0, got_e[1]),
                              ("p", p0, 1.0 / PROTON_MASS_RATIO, got_p)):
        P = {k: comps[i][a:a + m].cpu().numpy() for i, k in enumerate(keys)}
        ref = oracle.sync_spectrum_f64(P, bins, 1.0, 1.0, eps, table)
        g = got.cpu().numpy().astype(np.float64)
        mask = ref > 1e-12 * ref.max()
        res[name] = {"max_rel_err_vs_fp64": float(np.max(np.abs(g[mask] - ref[mask]) / ref[mask])),
                     "bins_compared": int(mask.sum())}
    res["oracle_seconds"] = time.perf_counter() - t0
    res["max_rel_err_vs_fp64"] = max(res[s]["max_rel_err_vs_fp64"] for s in ("e-", "e+", "p"))
    return res


def wavefront_roofline(achieved, evals_per_sm_clock, sms, clk_mhz, basis):
    """Fraction of the rate the shared-memory table reads allow (one wavefront per SM-clock)."""
    peak = sms * clk_mhz * 1e6 * evals_per_sm_clock
    return {"bound": "shared-memory wavefronts", "achieved": achieved, "peak": peak, "unit": "evals/s",
            "frac": achieved / peak, "basis": basis}


def add_wavefront_rooflines(extra, sms, clk_mhz):
    """Roofline fractions of the batched forward and of the forward + adjoint pair."""
    bg = extra.get("batched_graph_256_segments", {}).get("fused", {})
    if "graph_evals_per_s" in bg:
        bg["roofline"] = wavefront_roofline(
            bg["graph_evals_per_s"], 8.0, sms, clk_mhz,
            "200 bins 0.045 dex apart over 0.040-dex table segments: each 32-lane 8-byte lookup takes 4 "
            "wavefronts (16 lanes touch ~18 distinct entries), so 8 evals per SM-clock")
    fa = extra.get("fwd_adjoint_1e7x512", {}).get("fused", {})
    if "fwd_plus_adjoint_evals_per_s" in fa:
        basis = ("smooth table: every lane reads its own 16-byte Hermite segment, at least 4 wavefronts "
                 "per 32 evals in each kernel")
        fa["roofline"] = wavefront_roofline(fa["fwd_plus_adjoint_evals_per_s"], 4.0, sms, clk_mhz,
                                            basis + "; forward + adjoint = two passes, 4 evals per SM-clock")
        fa["roofline_fwd"] = wavefront_roofline(fa["fwd_evals_per_s"], 8.0, sms, clk_mhz,
                                                basis + ": 8 evals per SM-clock")
        fa["roofline_adjoint"] = wavefront_roofline(fa["adjoint_evals_per_s"], 8.0, sms, clk_mhz,
                                                    basis + ": 8 evals per SM-clock")


def guarded(fn, *a):
    """Runs one side case; a failure is reported in the JSON line instead of ending the run."""
    try:
        return fn(*a)
    except Exception as e:  # noqa: BLE001
        return {"error": f"{type(e).__name__}: {e}"}


def measured_peak(key, fallback):
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)[key]), "measured"
    except (OSError, KeyError, ValueError):
        return fallback, "fallback"


def timed(torch, fn, reps, warm=2):
    """Seconds per call of fn, CUDA events on the current stream after `warm` calls."""
    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        fn()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / 1e3 / reps


def logbins(capi, lo, hi, n):
    import numpy as np  # noqa: PLC0415

    b = np.empty(n, np.float32)
    capi.check(capi.lib().rg_logspace(lo, hi, n, b.ctypes.data))
    return b


def config1_particles(torch, n, gen, device, index=-2.0):
    """|u| ~ |u|^index on [1, 100] (per-particle index allowed), isotropic, B = z."""
    q = index + 1.0
    r = torch.rand(n, device=device, generator=gen, dtype=torch.float64)
    umag = ((100.0**q - 1.0) * r + 1.0) ** (1.0 / q)
    return isotropic_torch(torch, umag.float(), gen)


def side_measurements(torch, capi, device, stream):
    """The plain one-spectrum-per-launch kernel beside the fused one, and the
    1e6-particle x 200-bin configuration."""
    out = {}
    n = 8_000_000
    comps = make_particles(torch, n, 1, device, seed=77)
    prt = capi.particles(comps[0:3], b=comps[3:6], w=comps[6], n=n)
    plan = capi.SpectrumPlan(photon_bins(), 1.0, 1.0, 1.0)
    o = torch.empty(NBINS, device=device)
    out["dump_species_8e6_moments_evals_per_s"] = n * NBINS / timed(torch, lambda: plan.run(prt, o, stream), 10)
    plan.set_algorithm(capi.RG_ALGO_DIRECT)
    out["dump_species_8e6_fused_evals_per_s"] = n * NBINS / timed(torch, lambda: plan.run(prt, o, stream), 10)
    out["dump_species_8e6_plain_evals_per_s"] = n * NBINS / timed(torch, lambda: plan.run_plain(prt, o, stream), 2)
    plan.close()
    del comps
    n1 = 1_000_000
    gen = torch.Generator(device=device).manual_seed(5)
    u1 = config1_particles(torch, n1, gen, device)
    z = torch.zeros(n1, device=device)
    prt1 = capi.particles(u1, b=[z, z, torch.ones(n1, device=device)], n=n1)
    plan1 = capi.SpectrumPlan(logbins(capi, 0.01, 1e7, 200), 1.0, 1.0, 1.0)
    o1 = torch.empty(200, device=device)
    out["config1_moments_evals_per_s"] = n1 * 200 / timed(torch, lambda: plan1.run(prt1, o1, stream), 20)
    plan1.set_algorithm(capi.RG_ALGO_DIRECT)
    out["config1_fused_evals_per_s"] = n1 * 200 / timed(torch, lambda: plan1.run(prt1, o1, stream), 20)
    out["config1_plain_evals_per_s"] = n1 * 200 / timed(torch, lambda: plan1.run_plain(prt1, o1, stream), 5)
    plan1.close()
    return out


def batched_graph_case(torch, capi, device):
    """256 spectra of uneven size (counts log-uniform on [1e4, 1e7], power-law index
    uniform on [-3, -1.5] per segment, 200 bins 0.01..1e7): one persistent launch
    replayed from a CUDA graph, against the same launch eagerly and against one
    launch per segment."""
    nseg, nb = 256, 200
    gen = torch.Generator(device=device).manual_seed(303)
    counts = torch.floor(10.0 ** (4.0 + 3.0 * torch.rand(nseg, device=device, generator=gen,
                                                           dtype=torch.float64))).long()
    total = int(counts.sum())
    offs = torch.zeros(nseg + 1, dtype=torch.int64, device=device)
    offs[1:] = torch.cumsum(counts, 0)
    index = -3.0 + 1.5 * torch.rand(nseg, device=device, generator=gen, dtype=torch.float64)
    u = config1_particles(torch, total, gen, device,
                          index=torch.repeat_interleave(index, counts))
    bz = torch.ones(total, device=device)
    prt = capi.particles(u, b=[None, None, bz], n=total)
    res = {"segments": nseg, "particles": total, "photon_bins": nb}
    for algo, name in ((capi.RG_ALGO_MOMENTS, "moments"), (capi.RG_ALGO_DIRECT, "fused")):
        res[name] = batched_graph_algo(torch, capi, device, prt, offs, u, bz, nseg, nb, total, algo)
    return res


def batched_graph_algo(torch, capi, device, prt, offs, u, bz, nseg, nb, total, algo):
    plan = capi.SpectrumPlan(logbins(capi, 0.01, 1e7, nb), 1.0, 1.0, 1.0)
    plan.set_algorithm(algo)
    plan.reserve(nseg)
    out = torch.empty((nseg, nb), device=device)
    side = torch.cuda.Stream(device)
    side.wait_stream(torch.cuda.current_stream(device))
    with torch.cuda.stream(side):
        plan.run_batched(prt, offs, nseg, out, side.cuda_stream)
    torch.cuda.current_stream(device).wait_stream(side)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        plan.run_batched(prt, offs, nseg, out, torch.cuda.current_stream(device).cuda_stream)
    stream = torch.cuda.current_stream(device).cuda_stream
    t_graph = timed(torch, graph.replay, 10)
    ref = out.clone()
    t_eager = timed(torch, lambda: plan.run_batched(prt, offs, nseg, out, stream), 10)
    same = bool(torch.allclose(out, ref, rtol=2e-7, atol=0.0))
    host_offs = offs.cpu().tolist()
    segs = [capi.particles([c[a:b] for c in u], b=[None, None, bz[a:b]], n=b - a)
            for a, b in zip(host_offs[:-1], host_offs[1:])]

    def per_segment():
        for s in range(nseg):
            plan.run(segs[s], out[s], stream)

    t_loop = timed(torch, per_segment, 3, warm=1)
    plan.check(stream)
    plan.close()
    evals = total * nb
    return {"graph_evals_per_s": evals / t_graph, "graph_ms": t_graph * 1e3,
            "eager_batched_evals_per_s": evals / t_eager,
            "one_launch_per_segment_evals_per_s": evals / t_loop,
            "graph_matches_eager": same,
            "match": "bit-identical for the fused kernel; within FP32 rounding for interval moments"}


def fwd_adjoint_case(torch, capi, device):
    """1e7 particles (|u| ~ u^-2 on [1, 100], isotropic, B = z, w = 1) x 512 bins
    0.01..1e7 with the smooth (differentiable) table, which the plan aligns to these
    log-uniform bins: forward, adjoint (dL/dw and dL/du) and the pair, by cell moments
    (the default) and by the fused per-eval kernels, beside the plain reference-table
    kernel on the same particles."""
    n, nb = 10_000_000, 512
    gen = torch.Generator(device=device).manual_seed(404)
    u = config1_particles(torch, n, gen, device)
    z = torch.zeros(n, device=device)
    w = torch.ones(n, device=device)
    prt = capi.particles(u, b=[z, z, torch.ones(n, device=device)], w=w, n=n)
    bins = logbins(capi, 0.01, 1e7, nb)
    S = torch.empty(nb, device=device)
    gS = torch.rand(nb, device=device, generator=gen)
    gw = torch.empty(n, device=device)
    gu = [torch.empty(n, device=device) for _ in range(3)]
    stream = torch.cuda.current_stream(device).cuda_stream
    evals = n * nb
    res = {"particles": n, "photon_bins": nb, "table": "smooth, aligned to the bins"}
    for algo, name in ((capi.RG_ALGO_MOMENTS, "moments"), (capi.RG_ALGO_DIRECT, "fused")):
        plan = capi.SpectrumPlan(bins, 1.0, 1.0, 1.0, capi.RG_TABLE_SMOOTH)
        plan.set_algorithm(algo)
        t_fwd = timed(torch, lambda: plan.run(prt, S, stream), 10)
        t_adj = timed(torch, lambda: plan.adjoint(prt, gS, gw, gu, stream), 10)

        def step():
            plan.run(prt, S, stream)
            plan.adjoint(prt, gS, gw, gu, stream)

        t_step = timed(torch, step, 10)
        res[name] = {"fwd_evals_per_s": evals / t_fwd, "adjoint_evals_per_s": evals / t_adj,
                     "fwd_plus_adjoint_evals_per_s": evals / t_step, "fwd_plus_adjoint_ms": t_step * 1e3,
                     "fwd_ms": t_fwd * 1e3, "adjoint_ms": t_adj * 1e3}
        if plan.placement_supported():
            # the pair as torch_ext runs it: the forward records each particle's placement
            # (8 bytes per particle) and the adjoint reads it instead of placing the particle again
            place = torch.empty(2 * n, device=device, dtype=torch.int32)

            def step_placed():
                plan.run_placed(prt, S, place, stream)
                plan.adjoint_placed(prt, place, gS, gw, gu, stream)

            t_fwd_p = timed(torch, lambda: plan.run_placed(prt, S, place, stream), 10)
            t_adj_p = timed(torch, lambda: plan.adjoint_placed(prt, place, gS, gw, gu, stream), 10)
            t_step_p = timed(torch, step_placed, 10)
            res[name].update({
                "unplaced_fwd_plus_adjoint_ms": t_step * 1e3, "fwd_plus_adjoint_ms": t_step_p * 1e3,
                "fwd_plus_adjoint_evals_per_s": evals / t_step_p, "placed_fwd_ms": t_fwd_p * 1e3,
                "placed_adjoint_ms": t_adj_p * 1e3,
                "pair": "run_placed + adjoint_placed (the torch_ext path); fwd_ms / adjoint_ms: run + adjoint"})
            del place
        plan.check(stream)
        plan.close()
    # moments: HBM roofline of the pair (forward reads 28 B per particle, the adjoint
    # reads 28 B and writes 16 B: dL/dw and dL/du)
    peak, src = measured_peak("hbm_gbs", 6800.0)
    mo = res["moments"]
    gbs = 72.0 * n / (mo["fwd_plus_adjoint_ms"] * 1e-3) / 1e9
    mo["roofline"] = {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                      "peak_source": src,
                      "basis": "72 algorithmic bytes per particle per forward + adjoint pair (u, B, w read by "
                               "each; dL/dw and dL/du written)"}
    plain = capi.SpectrumPlan(bins, 1.0, 1.0, 1.0)
    t_plain = timed(torch, lambda: plain.run_plain(prt, S, stream), 3)
    plain.close()
    res["plain_fwd_evals_per_s"] = evals / t_plain
    return res


def fromdist_gemm_case(torch, capi, device, peak_bf16):
    """4096 distributions on 1024 log gamma bins [1, 1e6] (power laws, index uniform
    on [-3, -1.5], random cutoffs) -> 1024 photon bins 1e-2..1e13 through the
    split-precision tcgen05 GEMM; error against the FP64 product of the plan's
    own FP64 kernel matrix."""
    import numpy as np  # noqa: PLC0415

    nd, ng, ne = 4096, 1024, 1024
    gb = logbins(capi, 1.0, 1e6, ng)
    bins = logbins(capi, 1e-2, 1e13, ne)
    rng = np.random.default_rng(505)
    g = gb.astype(np.float64)[None, :]
    p = rng.uniform(-3.0, -1.5, (nd, 1))
    lo = 10.0 ** rng.uniform(0.0, 2.0, (nd, 1))
    hi = 10.0 ** rng.uniform(3.0, 6.0, (nd, 1))
    f_np = np.where((g >= lo) & (g < hi), g**p, 0.0).astype(np.float32)
    f = torch.from_numpy(f_np).to(device)
    out = torch.empty((nd, ne), device=device)
    stream = torch.cuda.current_stream(device).cuda_stream
    res = {"distributions": nd, "gamma_bins": ng, "photon_bins": ne}
    for terms in (6, 3):
        plan = capi.FromDistPlan(gb, True, bins, 1.0, 1.0, max_dist=nd, split_products=terms)
        tuned = plan.config()
        tuned_split = plan.split_k()
        shapes = {}
        for cfg, (bn, stages) in enumerate([(256, 4), (128, 6), (128, 4)]):
            plan.set_config(cfg, -1)
            shapes[f"128x{bn}_s{stages}_ms"] = timed(torch, lambda: plan.run(f, out, stream), 10) * 1e3
        plan.set_config([(256, 4), (128, 6), (128, 4)].index(tuned["fwd"]), -1)
        t = timed(torch, lambda: plan.run(f, out, stream), 20)
        plan.check(stream)
        K = plan.kernel_matrix()
        S = out.cpu().numpy().astype(np.float64)
        S64 = (f_np.astype(np.float64) @ K.T) * bins.astype(np.float64)[None, :]
        m = S64 > 1e-12 * S64.max(axis=1, keepdims=True)
        err = float(np.max(np.abs(S[m] - S64[m]) / S64[m]))
        flops = 2.0 * nd * ng * ne * terms
        res[f"bf16x{terms}"] = {
            "evals_per_s": nd * ng * ne / t, "ms": t * 1e3, "bf16_tflops": flops / t / 1e12,
            "frac_of_bf16_peak": flops / t / 1e12 / peak_bf16, "max_rel_err_vs_fp64": err,
            "autotuned_tile": {"fwd": list(tuned["fwd"]), "adj": list(tuned["adj"])},
            "autotuned_split_k": tuned_split, "tile_timings": shapes}
        plan.close()
    res["peak_bf16_tflops"] = peak_bf16
    return res


def adam_fit_case(torch, capi, device, steps=200):
    """1024 distributions of 512 log gamma bins [1, 1e5] fitted by Adam to target
    spectra of random broken power laws (indices uniform on [-3.5, -1.2], break
    log-uniform on [10, 1e4]) on 512 photon bins 1e-2..1e11; loss = log-space MSE.
    Gradients w.r.t. the distribution values flow through the GEMM forward and its
    transpose-GEMM adjoint; errors of the final forward and gradient are against
    FP64 products of the plan's FP64 kernel matrix."""
    import numpy as np  # noqa: PLC0415

    from ragnar_gb300 import torch_ext as rt  # noqa: PLC0415

    nd, ng, ne = 1024, 512, 512
    gb = logbins(capi, 1.0, 1e5, ng)
    bins = logbins(capi, 1e-2, 1e11, ne)
    plan = rt.fromdist_plan(gb, bins, max_dist=nd)
    gen = torch.Generator(device=device).manual_seed(606)
    lg = torch.log(torch.from_numpy(gb).to(device).double())[None, :]
    p1 = -3.5 + 2.3 * torch.rand((nd, 1), device=device, generator=gen, dtype=torch.float64)
    p2 = -3.5 + 2.3 * torch.rand((nd, 1), device=device, generator=gen, dtype=torch.float64)
    lb = math.log(10.0) * (1.0 + 3.0 * torch.rand((nd, 1), device=device, generator=gen, dtype=torch.float64))
    f_t = torch.exp(torch.where(lg < lb, p1 * lg, p1 * lb + p2 * (lg - lb))).float()
    with torch.no_grad():
        S_t = rt.synchrotron_from_dist_batched(plan, f_t)
    m_t = S_t > 1e-12 * S_t.amax(dim=1, keepdim=True)
    theta = (-2.0 * lg).float().repeat(nd, 1).contiguous().requires_grad_(True)
    opt = torch.optim.Adam([theta], lr=0.05)

    def loss_of(S):
        m = m_t & (S > 1e-12 * S.detach().amax(dim=1, keepdim=True))
        d = torch.log(torch.where(m, S, torch.ones_like(S))) - torch.log(torch.where(m, S_t, torch.ones_like(S)))
        return (d * d * m).sum() / m.sum().clamp(min=1)

    def step():
        opt.zero_grad(set_to_none=True)
        loss = loss_of(rt.synchrotron_from_dist_batched(plan, torch.exp(theta)))
        loss.backward()
        opt.step()
        return loss

    l0 = float(step().detach())
    torch.cuda.synchronize()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(steps - 1):
        loss = step()
    b.record()
    torch.cuda.synchronize()
    t_step = a.elapsed_time(b) / 1e3 / (steps - 1)
    l1 = float(loss.detach())

    # the same step captured once into a CUDA graph (forward GEMM, loss, transpose-GEMM
    # backward, Adam update) and replayed: no per-op launch or Python overhead
    theta_g = (-2.0 * lg).float().repeat(nd, 1).contiguous().requires_grad_(True)
    opt_g = torch.optim.Adam([theta_g], lr=0.05, capturable=True)

    def step_g():
        loss = loss_of(rt.synchrotron_from_dist_batched(plan, torch.exp(theta_g)))
        loss.backward()
        opt_g.step()
        return loss

    side = torch.cuda.Stream(device)
    side.wait_stream(torch.cuda.current_stream(device))
    with torch.cuda.stream(side):
        for _ in range(3):
            opt_g.zero_grad(set_to_none=True)
            step_g()
    torch.cuda.current_stream(device).wait_stream(side)
    graph = torch.cuda.CUDAGraph()
    opt_g.zero_grad(set_to_none=True)
    with torch.cuda.graph(graph):
        loss_static = step_g()
    for _ in range(3):
        graph.replay()
    torch.cuda.synchronize()
    a.record()
    for _ in range(steps - 1):
        graph.replay()
    b.record()
    torch.cuda.synchronize()
    t_graph = a.elapsed_time(b) / 1e3 / (steps - 1)
    l_graph = float(loss_static.detach())

    # final forward and gradient against FP64
    f = torch.exp(theta.detach()).contiguous().requires_grad_(True)
    S = rt.synchrotron_from_dist_batched(plan, f)
    loss = loss_of(S)
    gS, = torch.autograd.grad(loss, S, retain_graph=True)
    loss.backward()
    K = plan.kernel_matrix()
    e = bins.astype(np.float64)[None, :]
    f64 = f.detach().cpu().numpy().astype(np.float64)
    S64 = (f64 @ K.T) * e
    Sg = S.detach().cpu().numpy()
    mm = S64 > 1e-12 * S64.max(axis=1, keepdims=True)
    g64 = (gS.cpu().numpy().astype(np.float64) * e) @ K
    gg = f.grad.cpu().numpy()
    plan.check()
    plan.close()
    return {"distributions": nd, "gamma_bins": ng, "photon_bins": ne, "adam_steps": steps,
            "ms_per_adam_step": t_step * 1e3, "gemm_evals_per_s": 2.0 * nd * ng * ne / t_step,
            "ms_per_adam_step_cuda_graph": t_graph * 1e3, "loss_after_graphed_steps": l_graph,
            "loss_first": l0, "loss_last": l1,
            "fwd_max_rel_err_vs_fp64": float(np.max(np.abs(Sg[mm] - S64[mm]) / S64[mm])),
            "grad_max_err_vs_fp64_rel_to_row_max": float(np.max(np.abs(gg - g64) /
                                                                np.max(np.abs(g64), axis=1, keepdims=True)))}


def dropin_module_case(torch, comps, n, reps=3):
    """The reference-facing Python module on one dump-scale species, each call blocking as in
    the reference: Particles_3D.fromArrays from numpy (pageable host memory, allocation plus
    one host-to-device copy per component, in place of the reference's element-wise host
    loops), SynchrotronSpectrum_3D(...).as_array() and energyDistribution(Logbins(...))."""
    import ragnar_gb300 as rg  # noqa: PLC0415

    rg.SetVerbose(False)
    rg.Initialize()
    keys = ("U1", "U2", "U3", "B1", "B2", "B3")
    host = {k: comps[i][:n].cpu().numpy() for i, k in enumerate(keys)}
    bins = rg.Logbins(BIN_LO, BIN_HI, NBINS, rg.EnergyUnits.mec2)
    ebins = rg.Logbins(1e-2, 1e3, 200)

    def wall(fn):
        fn()
        ts = []
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
        return statistics.median(ts)

    held = {}

    def ingest():
        held.pop("p", None)
        p = rg.Particles_3D("e-")
        p.fromArrays(host)
        held["p"] = p

    t_in = wall(ingest)
    prt = held["p"]
    t_sp = wall(lambda: rg.SynchrotronSpectrum_3D(prt, bins, 1.0, 1.0, 1.0).as_array())
    t_h = wall(lambda: prt.energyDistribution(ebins))
    nbytes = 4 * len(keys) * n
    return {"particles": n, "timing": f"median of {reps} blocking calls (host wall clock)",
            "fromArrays_ms": t_in * 1e3, "fromArrays_gbs": nbytes / t_in / 1e9,
            "fromArrays_bytes": nbytes,
            "SynchrotronSpectrum_ms": t_sp * 1e3, "SynchrotronSpectrum_evals_per_s": n * NBINS / t_sp,
            "energyDistribution_ms": t_h * 1e3, "energyDistribution_particles_per_s": n / t_h}


def ic_case(torch, capi, device, clk_mhz=2070.0):
    """ICSpectrum of a 1024-bin particle power law (index -2 on [1e2, 1e7], exp cutoff at
    3e6) on a 1024-bin soft-photon field (1e-9..1e-3 mec2, dN/dE ~ E^-1) into 1024 IC bins
    1e-3..1e7: 1.07e9 (gamma, soft photon, IC bin) evals.  Bound: one MUFU lg2 per eval
    (16 per SM per clock)."""
    import numpy as np  # noqa: PLC0415

    n = 1024
    gb = logbins(capi, 1e2, 1e7, n)
    fp = (gb.astype(np.float64) ** -2.0 * np.exp(-gb / 3e6)).astype(np.float32)
    es = logbins(capi, 1e-9, 1e-3, n)
    fs = (1.0 / es.astype(np.float64)).astype(np.float32)
    eic = logbins(capi, 1e-3, 1e7, n)
    t = [torch.from_numpy(a).to(device) for a in (gb, fp, es, fs, eic)]
    out = torch.empty(n, device=device)
    stream = torch.cuda.current_stream(device).cuda_stream

    def run():
        capi.check(capi.lib().rg_ic_spectrum(t[0].data_ptr(), t[1].data_ptr(), n, 1, t[2].data_ptr(),
                                             t[3].data_ptr(), n, t[4].data_ptr(), n, out.data_ptr(), stream))

    dt = timed(torch, run, 10)
    sms = torch.cuda.get_device_properties(device).multi_processor_count
    evals = float(n) ** 3
    peak = sms * 16 * clk_mhz * 1e6
    return {"gamma_bins": n, "soft_photon_bins": n, "ic_bins": n, "ms": dt * 1e3, "evals_per_s": evals / dt,
            "mufu_peak_evals_per_s": peak, "frac_of_mufu_peak": evals / dt / peak,
            "finite": bool(torch.isfinite(out).all())}


def histogram_case(torch, capi, device, comps, n, reps=10):
    """Particles.energyDistribution of the dump-scale particles into 200 log gamma-beta
    bins 1e-2..1e3 (12 B/particle read: the HBM-bound kernel)."""
    import numpy as np  # noqa: PLC0415

    bins = logbins(capi, 1e-2, 1e3, 200)
    hist = torch.empty(200, device=device)
    stream = torch.cuda.current_stream(device).cuda_stream

    def run():
        capi.check(capi.lib().rg_energy_distribution(comps[0].data_ptr(), comps[1].data_ptr(),
                                                     comps[2].data_ptr(), n, bins.ctypes.data, 200, 1, 1,
                                                     hist.data_ptr(), None, stream))

    t = timed(torch, run, reps, warm=1)
    return {"particles": n, "bins": 200, "particles_per_s": n / t, "ms": t * 1e3,
            "hbm_gbs": 12.0 * n / t / 1e9}


def profile_case():
    """4 launches of the fused spectrum kernel on 2^22 particles x 512 bins
    (inputs 117 MB + a 256 MB buffer written between launches to flush L2)."""
    import torch  # noqa: PLC0415

    from ragnar_gb300 import capi  # noqa: PLC0415

    device = torch.device("cuda", 0)
    capi.check(capi.lib().rg_init(0))
    n = 1 << 22
    comps = make_particles(torch, n, 1, device, seed=3)
    plan = capi.SpectrumPlan(photon_bins(), 1.0, 1.0, 1.0)
    plan.set_algorithm(capi.RG_ALGO_DIRECT)
    out = torch.empty(NBINS, device=device)
    prt = capi.particles(comps[0:3], b=comps[3:6], w=comps[6], n=n)
    flush = torch.empty(64 << 20, device=device)
    for _ in range(4):
        flush.fill_(1.0)
        plan.run(prt, out, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    plan.check()
    plan.close()
    print("profile case done")


def profile_case_moments():
    """4 runs of the interval-moment path (deposit, scan, reduce) on 2^24 particles of
    the dump-scale e- species x 512 bins (inputs 470 MB, above the L2)."""
    import torch  # noqa: PLC0415

    from ragnar_gb300 import capi  # noqa: PLC0415

    device = torch.device("cuda", 0)
    capi.check(capi.lib().rg_init(0))
    n = 1 << 24
    comps = make_particles(torch, n, 1, device, seed=3)
    plan = capi.SpectrumPlan(photon_bins(), 1.0, 1.0, 1.0)
    assert plan.algorithm(1) == capi.RG_ALGO_MOMENTS
    out = torch.empty(NBINS, device=device)
    prt = capi.particles(comps[0:3], b=comps[3:6], w=comps[6], n=n)
    for _ in range(4):
        plan.run(prt, out, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    plan.check()
    plan.close()
    print("profile case (interval moments) done")


def profile_case_200():
    """4 launches of the fused kernel on 2^22 particles of the 1e6-particle configuration's
    kind (|u| ~ u^-2 on [1, 100], isotropic, B = z, w = 1) x 200 bins 0.01..1e7."""
    import torch  # noqa: PLC0415

    from ragnar_gb300 import capi  # noqa: PLC0415

    device = torch.device("cuda", 0)
    capi.check(capi.lib().rg_init(0))
    n = 1 << 22
    gen = torch.Generator(device=device).manual_seed(5)
    u = config1_particles(torch, n, gen, device)
    prt = capi.particles(u, b=[None, None, torch.ones(n, device=device)], n=n)
    plan = capi.SpectrumPlan(logbins(capi, 0.01, 1e7, 200), 1.0, 1.0, 1.0)
    plan.set_algorithm(capi.RG_ALGO_DIRECT)
    out = torch.empty(200, device=device)
    flush = torch.empty(64 << 20, device=device)
    for _ in range(4):
        flush.fill_(1.0)
        plan.run(prt, out, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    plan.check()
    plan.close()
    print("profile case (200 bins) done")


def profile_case_smooth(algo=1, n=1 << 22):
    """The differentiable path on n particles (|u| ~ u^-2 on [1, 100], isotropic, B = z,
    w = 1) x 512 bins 0.01..1e7 with the smooth table: 4 forward and 4 adjoint runs, by
    the fused kernels (algo 1) or the cell moments (algo 2, with the placement record the
    forward writes for the adjoint)."""
    import torch  # noqa: PLC0415

    from ragnar_gb300 import capi  # noqa: PLC0415

    device = torch.device("cuda", 0)
    capi.check(capi.lib().rg_init(0))
    gen = torch.Generator(device=device).manual_seed(5)
    u = config1_particles(torch, n, gen, device)
    w = torch.ones(n, device=device)
    prt = capi.particles(u, b=[None, None, torch.ones(n, device=device)], w=w, n=n)
    plan = capi.SpectrumPlan(logbins(capi, 0.01, 1e7, 512), 1.0, 1.0, 1.0, capi.RG_TABLE_SMOOTH)
    plan.set_algorithm(algo)
    out = torch.empty(512, device=device)
    gS = torch.rand(512, device=device, generator=gen)
    gw = torch.empty(n, device=device)
    gu = [torch.empty(n, device=device) for _ in range(3)]
    stream = torch.cuda.current_stream().cuda_stream
    place = torch.empty(2 * n, device=device, dtype=torch.int32) if plan.placement_supported() else None
    for _ in range(4):
        if place is not None:  # the torch_ext path: the forward records the placements the adjoint reads
            plan.run_placed(prt, out, place, stream)
            plan.adjoint_placed(prt, place, gS, gw, gu, stream)
        else:
            plan.run(prt, out, stream)
            plan.adjoint(prt, gS, gw, gu, stream)
    torch.cuda.synchronize()
    plan.check()
    plan.close()
    print("profile case (smooth table) done")


def profile_gemm_case():
    """4 launches of the split + tcgen05 GEMM forward on 4096 x 1024 x 1024 (6 products)."""
    import numpy as np  # noqa: PLC0415
    import torch  # noqa: PLC0415

    from ragnar_gb300 import capi  # noqa: PLC0415

    device = torch.device("cuda", 0)
    capi.check(capi.lib().rg_init(0))
    gb = logbins(capi, 1.0, 1e6, 1024)
    bins = logbins(capi, 1e-2, 1e13, 1024)
    rng = np.random.default_rng(505)
    f = torch.from_numpy((gb.astype(np.float64)[None, :] ** rng.uniform(-3.0, -1.5, (4096, 1)))
                         .astype(np.float32)).to(device)
    out = torch.empty((4096, 1024), device=device)
    plan = capi.FromDistPlan(gb, True, bins, 1.0, 1.0, max_dist=4096)
    for _ in range(4):
        plan.run(f, out, torch.cuda.current_stream().cuda_stream)
    plan.check()
    plan.close()
    print("profile gemm case done")


def profile_histogram_case():
    """4 energyDistribution calls on one dump-scale species (3.3e7 particles, 396 MB of u)."""
    import torch  # noqa: PLC0415

    from ragnar_gb300 import capi  # noqa: PLC0415

    device = torch.device("cuda", 0)
    capi.check(capi.lib().rg_init(0))
    comps = make_particles(torch, N_PER_SPECIES, 1, device, seed=3)
    for _ in range(4):
        histogram_case(torch, capi, device, comps, N_PER_SPECIES, reps=1)
    print("profile histogram case done")


def main():
    args = parse_args()
    if args.profile_case == "spectrum":
        profile_case()
        return
    if args.profile_case == "moments":
        profile_case_moments()
        return
    if args.profile_case == "spectrum200":
        profile_case_200()
        return
    if args.profile_case == "smooth":
        profile_case_smooth()
        return
    if args.profile_case == "smooth_moments":
        profile_case_smooth(2, 1 << 24)
        return
    if args.profile_case == "gemm":
        profile_gemm_case()
        return
    if args.profile_case == "histogram":
        profile_histogram_case()
        return
    if args.profile_case == "ic":
        import torch  # noqa: PLC0415

        from ragnar_gb300 import capi  # noqa: PLC0415

        capi.check(capi.lib().rg_init(0))
        print(json.dumps(ic_case(torch, capi, torch.device("cuda", 0))))
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference_arm(args, rank)
        return
    if world > 1:
        import torch  # noqa: PLC0415

        torch.cuda.set_device(local_rank)
        torch.distributed.init_process_group("nccl")
    try:
        run_ours(args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch  # noqa: PLC0415

            torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
