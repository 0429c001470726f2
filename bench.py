#!/usr/bin/env python3
"""Benchmark of the GB300 spectral random-field summators.

Metric: Gpoint*modes/s (points x Fourier modes summed per second) on one
GB300, for the chosen computation form, next to the plain FP64 kernel.

Workloads (synthetic, seeded numpy default_rng; the reference publishes no
benchmark data):
  c1  plain 2-D unstructured: 100,000 points in [0,100]^2, 1000 modes,
      Gaussian spectrum (k ~ N(0, 2/l^2), l = 10)
  c2  structured 3-D scalar: 256^3 grid, spacing 1, 2000 modes, exponential
      spectrum (multivariate Student-t nu=1, / l, l = 20)
  c3  unstructured 3-D: 16,777,216 points in [0,1000]^3, 4096 modes,
      exponential spectrum l = 5
  c4  incompressible 3-D: 192^3 grid, 2048 modes, Gaussian spectrum l = 8
  c5  batched ensemble: 512 realizations (seed r each; 2-D for r < 256, else
      3-D; points log-uniform 1e3..1e6 in [0,500]^d; modes log-uniform
      256..8192; Gaussian spectrum for even r, exponential for odd r,
      l uniform in [2, 50]) in one persistent launch replayed as a CUDA graph
  field  the reference's criterion field benchmarks (benches/main.rs:51-133):
      summate 2-D and 3-D, summate_incompr 2-D and 3-D, summate_fourier 2-D
      on 10,000 points x 1000 modes, inputs read from the reference's
      benches/input text format (--input-dir; synthesized stand-ins when
      absent); one step = the five calls
  all  [default] c1 .. c5 in turn; the JSON line is c5's (the largest
      workload, 1.7e11 point*modes per step) with every workload's full
      record under "configs" and a short "summary"

One step = one full summation of the workload.  `value` is timed with CUDA
events on the launch stream, inputs resident in HBM, L2 flushed (a 256 MiB
write) before every timed step; `e2e` is the same metric through the public
host API at tolerance 1e-6 (numpy in, numpy out, host<->device
copies inside the timed call).  Every workload's output is compared, value
by value, with an FP64 form on the GPU that is itself checked against the
oracle in the same run (error_vs_fp64_full), and a seeded subset with the
oracle directly (error_vs_oracle).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload all] [--form auto]
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "gstools-core_gb300"))
sys.path.insert(0, ROOT)

METRIC = ("Gpoint*modes/s on 1 GB300 at stated error vs FP64; chosen form vs plain FP64 "
          "kernel")
UNIT = "Gpoint*modes/s"


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------
def student_t(rng, dim, n, ell):
    return rng.standard_normal((dim, n)) / np.sqrt(rng.chisquare(1, n)) / ell


def workload(name: str):
    """Returns dict(dim, cov, z1, z2, pos=None | axes=None, incompr, desc)."""
    rng = np.random.default_rng(0)
    if name == "c1":
        pos = rng.uniform(0, 100, (2, 100000))
        cov = rng.normal(0, np.sqrt(2) / 10, (2, 1000))
        z1, z2 = rng.standard_normal(1000), rng.standard_normal(1000)
        return dict(dim=2, cov=cov, z1=z1, z2=z2, pos=pos, axes=None, incompr=False,
                    desc="plain 2-D unstructured, 1e5 points x 1000 modes, Gaussian l=10")
    if name == "c2":
        cov = student_t(rng, 3, 2000, 20.0)
        z1, z2 = rng.standard_normal(2000), rng.standard_normal(2000)
        ax = np.arange(256, dtype=np.float64)
        return dict(dim=3, cov=cov, z1=z1, z2=z2, pos=None, axes=(ax, ax, ax), incompr=False,
                    desc="structured 3-D scalar, 256^3 grid x 2000 modes, exponential l=20")
    if name == "c3":
        pos = rng.uniform(0, 1000, (3, 16777216))
        cov = student_t(rng, 3, 4096, 5.0)
        z1, z2 = rng.standard_normal(4096), rng.standard_normal(4096)
        return dict(dim=3, cov=cov, z1=z1, z2=z2, pos=pos, axes=None, incompr=False,
                    desc="unstructured 3-D, 16777216 points x 4096 modes, exponential l=5")
    if name == "c4":
        cov = rng.normal(0, np.sqrt(2) / 8, (3, 2048))
        z1, z2 = rng.standard_normal(2048), rng.standard_normal(2048)
        ax = np.arange(192, dtype=np.float64)
        return dict(dim=3, cov=cov, z1=z1, z2=z2, pos=None, axes=(ax, ax, ax), incompr=True,
                    desc="incompressible 3-D, 192^3 grid x 2048 modes, Gaussian l=8")
    raise SystemExit(f"unknown workload {name}")


def ensemble(count=512, stride=1):
    """The c5 ensemble: per realization r, rng = default_rng(r), draws in the
    order P, N, l, pos, cov, z1, z2.  stride > 1 keeps realizations 0,
    stride, 2 stride, ... (the same mix of sizes and dimensions at 1/stride
    of the work: a small case of the same kernel for profilers)."""
    items = []
    for r in range(0, count, stride):
        rng = np.random.default_rng(r)
        d = 2 if r < count // 2 else 3
        P = int(round(10 ** rng.uniform(3, 6)))
        N = int(round(2 ** rng.uniform(8, 13)))
        ell = rng.uniform(2, 50)
        pos = rng.uniform(0, 500, (d, P))
        if r % 2 == 0:
            cov = rng.normal(0, np.sqrt(2) / ell, (d, N))
        else:
            cov = student_t(rng, d, N, ell)
        z1, z2 = rng.standard_normal(N), rng.standard_normal(N)
        items.append({"kind": "scalar", "cov": cov, "z1": z1, "z2": z2, "pos": pos})
    return items


def flat_grid(axes):
    return np.ascontiguousarray(
        np.array(np.meshgrid(*axes, indexing="ij")).reshape(len(axes), -1))


def n_points(w):
    if w["pos"] is not None:
        return w["pos"].shape[1]
    return int(np.prod([len(a) for a in w["axes"]]))


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        # the raw samples go to GSC_CLOCKS_CSV when set (kept), else to a temporary file
        self.keep = bool(os.environ.get("GSC_CLOCKS_CSV"))
        self.path = os.environ.get("GSC_CLOCKS_CSV") or os.path.join(
            tempfile.gettempdir(), f"gsc_clocks_{os.getpid()}_{device_index}.csv")

    def __enter__(self):
        try:
            if os.path.dirname(self.path):
                os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        with open(self.path) as fh:
            lines = fh.readlines()
        if not self.keep:
            try:
                os.remove(self.path)
            except OSError:
                pass
        for line in lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                rows.append((float(f[1]), float(f[2]), float(f[3]) if f[3] not in ("[N/A]", "N/A") else 0.0, f[5:9]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [r[0] for r in rows]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for n, v in zip(names, r[3]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(r[1] for r in rows),
                "power_w_max": max(r[2] for r in rows), "samples": len(rows),
                "reasons": sorted(reasons)}


# ---------------------------------------------------------------------------
# reference arm / CPU baseline: the oracle on the host cores
# ---------------------------------------------------------------------------
def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_sample(w, target_s=2.0, max_points=None):
    """A bounded, seeded subset of the workload's points with all modes."""
    import oracle
    P = n_points(w)
    rng = np.random.default_rng(1234)
    cores = host_cores()
    # size the sample: calibrate on a small batch
    probe = min(P, 4 * cores)
    idx = np.sort(rng.choice(P, size=probe, replace=False))
    pos = sample_points(w, idx)
    fn = oracle.summator_incompr if w["incompr"] else oracle.summator
    t0 = time.perf_counter()
    fn(w["cov"], w["z1"], w["z2"], pos, num_threads=cores)
    dt = max(time.perf_counter() - t0, 1e-6)
    m = int(min(P, max(probe, probe * target_s / dt)))
    if max_points:
        m = min(m, max_points)
    idx = np.sort(rng.choice(P, size=m, replace=False))
    return sample_points(w, idx), fn, cores


def sample_points(w, idx):
    if w["pos"] is not None:
        return np.ascontiguousarray(w["pos"][:, idx])
    shape = [len(a) for a in w["axes"]]
    sub = np.unravel_index(idx, shape)
    return np.ascontiguousarray(np.array([w["axes"][d][sub[d]] for d in range(len(shape))]))


def time_cpu(w, steps, target_s):
    pos, fn, cores = cpu_sample(w, target_s)
    n = w["cov"].shape[1]
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        fn(w["cov"], w["z1"], w["z2"], pos, num_threads=cores)
        times.append(time.perf_counter() - t0)
    work = pos.shape[1] * n
    return work / np.mean(times) / 1e9, cores, pos.shape[1], np.mean(times)


# ---------------------------------------------------------------------------
# distributed plumbing (weak scaling: every rank runs the full workload)
# ---------------------------------------------------------------------------
def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        import torch
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local


def shard_range(n_points: int, rank: int, world: int):
    """Contiguous point range [lo, hi) of `rank`: points are independent, so
    a multi-GPU run needs no collective on the data path."""
    return n_points * rank // world, n_points * (rank + 1) // world


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, value: float) -> float:
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def default_form(w):
    """The chosen form per workload: the exact-leading-term tensor-core
    contraction on structured grids, the mixed-precision kernel on points."""
    return "sep_f16x5" if w["axes"] is not None else "mixed"


def other_forms(w, chosen):
    """Forms measured beside the chosen one (besides the plain FP64 arm)."""
    if w["axes"] is not None:
        cand = ["sep_f64", "sep_f16x3"]
    else:
        cand = ["mixed_f64phase"]
    return [f for f in cand if f != chosen]


def make_device_step(gsc, torch, w, form, dev, stream):
    """Returns (step(timing) -> None, out_tensor) running the workload on the device."""
    P = n_points(w)
    cov_d = torch.from_numpy(np.ascontiguousarray(w["cov"])).to(dev)
    z1_d = torch.from_numpy(w["z1"]).to(dev)
    z2_d = torch.from_numpy(w["z2"]).to(dev)
    nout = w["dim"] if w["incompr"] else 1
    out_d = torch.empty((nout, P) if w["incompr"] else (P,), dtype=torch.float64, device=dev)
    if w["axes"] is not None and form.startswith("sep"):
        axes_d = tuple(torch.from_numpy(a).to(dev) for a in w["axes"])
        call = gsc.summate_incompr_structured_device if w["incompr"] else gsc.summate_structured_device

        def step(timing=False):
            call(cov_d, z1_d, z2_d, axes_d, out_d, form=form, stream=stream.cuda_stream,
                 timing=timing)
    else:
        pos_h = w["pos"] if w["pos"] is not None else flat_grid(w["axes"])
        pos_d = torch.from_numpy(pos_h).to(dev)
        call = gsc.summate_incompr_device if w["incompr"] else gsc.summate_device

        def step(timing=False):
            call(cov_d, z1_d, z2_d, pos_d, out_d, form=form, stream=stream.cuda_stream,
                 timing=timing)
    return step, out_d


def timed_steps(torch, gsc, step, stream, steps, flush):
    """Per-step CUDA-event times (L2 flushed before each step) and kernel timings."""
    per_step, kern, launches = [], {}, 0
    for _ in range(steps):
        flush.fill_(1)                       # evict L2 (129 MB) between steps
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        step(timing=True)
        b.record(stream)
        b.synchronize()
        per_step.append(a.elapsed_time(b))
        tl = gsc.last_timings()
        launches += len(tl)
        for name, ms in tl:
            kern.setdefault(name, []).append(ms)
    return per_step, kern, launches


def split_timings(timings):
    """(kernel ms, copy ms) of one call's timing records."""
    k = sum(ms for name, ms in timings if not name.startswith("copy_"))
    c = sum(ms for name, ms in timings if name.startswith("copy_"))
    return k, c


def warm_up(torch, step, w, min_s=0.5, timing=False, flush=None):
    """At least w untimed steps, continued until min_s seconds have passed so
    that the clock sampler (50 ms period) sees the GPU under this load before
    the timed steps, which can be shorter than one sampling period.  The
    steps run as the timed ones do (L2 flush before each, per-kernel times
    recorded), so that one-time costs of those are paid here."""
    n, t0 = 0, time.perf_counter()
    while n < w or time.perf_counter() - t0 < min_s:
        if flush is not None:
            flush.fill_(1)
        if timing:
            step(timing=True)
        else:
            step()
        torch.cuda.synchronize()
        n += 1
    return n


def full_error(torch, got, ref):
    """max |got - ref| and RMS(got - ref) over every value, relative to the
    RMS of ref (device tensors, any shape)."""
    g = got.reshape(-1)
    r = ref.reshape(-1)
    rms = float(torch.sqrt(torch.mean(r * r)))
    d = (g - r).abs()
    return {"max_abs_over_rms": float(d.max()) / rms if rms > 0 else float(d.max()),
            "rms_over_rms": float(torch.sqrt(torch.mean(d * d))) / rms if rms > 0 else 0.0,
            "values_checked": int(g.numel())}


def run_ours(args, world, rank, local, wname, cpu_seconds, form_arg="auto"):
    import torch
    import gstools_core as gsc
    import oracle

    torch.cuda.set_device(local)
    w = workload(wname)
    P, N = n_points(w), w["cov"].shape[1]
    nout = w["dim"] if w["incompr"] else 1
    work = float(P) * N
    form = default_form(w) if form_arg == "auto" else form_arg
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    step, out_d = make_device_step(gsc, torch, w, form, dev, stream)

    # ---- warm-up and timed region, clocks sampled throughout -----------------
    with ClockSampler(local) as clk:
        warm = warm_up(torch, step, args.warmup, args.min_warmup_s, timing=True, flush=flush)
        gsc.device_status()
        barrier(world)
        torch.cuda.synchronize()
        t_wall = time.perf_counter()
        per_step, kern, launches = timed_steps(torch, gsc, step, stream, args.steps, flush)
        torch.cuda.synchronize()
        barrier(world)
        t_wall = time.perf_counter() - t_wall
    gsc.device_status()
    ms_step = max_over_ranks(world, float(np.mean(per_step)))
    value = work * world / (ms_step * 1e-3) / 1e9

    # ---- dominant kernel roofline ------------------------------------------
    dom = max(kern, key=lambda k: sum(kern[k]))
    launches_per_step = len(kern[dom]) / args.steps
    dom_ms = float(np.mean(kern[dom]))
    roof = roofline(args, w, dom, dom_ms, launches_per_step, wname=wname)

    # ---- parity of this very output against the oracle on a seeded subset --
    err, check = None, None
    if not args.no_check:
        rng = np.random.default_rng(7)
        # every point up to 2^17 (C1 in full), else a seeded 2^16-point subset; all modes
        idx = np.sort(rng.choice(P, size=P if P <= 1 << 17 else 1 << 16, replace=False))
        pos_s = sample_points(w, idx)
        fn = oracle.summator_incompr if w["incompr"] else oracle.summator
        ref = fn(w["cov"], w["z1"], w["z2"], pos_s, num_threads=host_cores())
        rms = float(np.sqrt(np.mean(ref ** 2)))

        def check(out_t):
            got = out_t.cpu().numpy()
            got = got[:, idx] if w["incompr"] else got[idx]
            return {"max_abs_over_rms": float(np.max(np.abs(got - ref)) / rms),
                    "rms_over_rms": float(np.sqrt(np.mean((got - ref) ** 2)) / rms),
                    "points_checked": int(len(idx)),
                    "reference": "oracle (field.rs restatement), FP64"}
        err = check(out_d)

    # ---- e2e through the public host API at tolerance 1e-6 (before
    # the long comparison arms, so that it runs in the same state of the GPU
    # as the timed steps).  The call GSTools makes -- summate(cov_samples, z1,
    # z2, pos) with pos the flattened meshgrid on structured grids -- plus
    # tolerance=1e-6; on a grid the library recognises the mesh on the host
    # and only the modes and the axes cross the bus.
    e2e, e2e_structured, dropin = None, None, None
    if not args.no_e2e:
        call = gsc.summate_incompr if w["incompr"] else gsc.summate
        if w["axes"] is not None:
            pos_h = flat_grid(w["axes"])
            h2d = (w["cov"].size + 2 * N + sum(len(a) for a in w["axes"])) * 8
        else:
            pos_h = w["pos"]
            h2d = (w["cov"].size + 2 * N + pos_h.size) * 8

        def host_e2e(fn, fargs, kwargs, reps, h2d_bytes, api):
            fn(*fargs, **kwargs)                  # staging buffers, result pool
            t0 = time.perf_counter()
            fn(*fargs, **kwargs)
            t_warm = time.perf_counter() - t0
            # short calls are repeated for about 50 ms (up to 200 calls)
            reps = max(reps, min(200, int(0.05 / max(t_warm, 1e-6))))
            ts = []
            barrier(world)
            for _ in range(reps):
                t0 = time.perf_counter()
                fn(*fargs, **kwargs)
                ts.append(time.perf_counter() - t0)
            # one more call with the library's event timing, for the split
            fn(*fargs, timing=True, **kwargs)
            tl = gsc.last_timings()
            k_ms, c_ms = split_timings(tl)
            t = max_over_ranks(world, float(np.mean(ts)))
            return {"value": work * world / t / 1e9, "unit": UNIT,
                    "h2d_bytes_per_step": int(h2d_bytes), "d2h_bytes_per_step": int(nout * P * 8),
                    "ms_per_step": t * 1e3, "calls": reps, "api": api,
                    "kernels": sorted({k for k, _ in tl if not k.startswith("copy_")}),
                    "kernel_ms_per_step": k_ms, "copy_ms_per_step": c_ms,
                    "timing": "host wall clock around each synchronous call, mean over the "
                              "calls (kernel_ms_per_step, copy_ms_per_step: one further call's "
                              "own kernels and host-device copies, CUDA events)"}
        reps = max(1, min(args.steps, 3))
        e2e = host_e2e(call, (w["cov"], w["z1"], w["z2"], pos_h), {"tolerance": 1e-6}, reps, h2d,
                       f"gstools_core.{call.__name__}(cov_samples, z1, z2, pos, tolerance=1e-6)"
                       + (" with pos the flattened meshgrid" if w["axes"] is not None else ""))
        if w["axes"] is not None:
            scall = gsc.summate_incompr_structured if w["incompr"] else gsc.summate_structured
            e2e_structured = host_e2e(
                scall, (w["cov"], w["z1"], w["z2"], w["axes"]), {"form": form}, reps, h2d,
                f"gstools_core.{scall.__name__} (the axes; no reference counterpart)")
            # default arguments: tolerance 1e-12, routed to the FP64 DMMA form
            dropin = host_e2e(call, (w["cov"], w["z1"], w["z2"], pos_h), {}, 2, h2d,
                              f"gstools_core.{call.__name__}(cov_samples, z1, z2, pos) with the "
                              "flattened meshgrid and default form / tolerance (1e-12)")
        del pos_h

    # ---- every value against an FP64 form on the GPU, itself checked
    # against the oracle here: the FP64 DMMA contraction on grids, the plain
    # FP64 kernel on points (its timed step is the plain arm) --------------------
    full, plain = None, None
    ref_form = "sep_f64" if w["axes"] is not None else "plain"
    if not args.no_check or not args.no_plain:
        rstep, rout = make_device_step(gsc, torch, w, ref_form, dev, stream)
        rstep()
        torch.cuda.synchronize()
        rt, rk, _ = timed_steps(torch, gsc, rstep, stream, 1, flush)
        gsc.device_status()
        rms_ = max_over_ranks(world, float(np.mean(rt)))
        if not args.no_check:
            full = full_error(torch, out_d, rout)
            pin = check(rout)
            full["reference"] = (f"{ref_form} on the GPU ("
                                 + ("FP64 DMMA contraction" if ref_form == "sep_f64"
                                    else "plain FP64 kernel")
                                 + f"), itself {pin['max_abs_over_rms']:.2e} of RMS from the "
                                   f"oracle on {pin['points_checked']} points in this run")
            full["reference_vs_oracle"] = pin["max_abs_over_rms"]
        if ref_form == "plain" and form != "plain":
            plain = {"value": work * world / (rms_ * 1e-3) / 1e9, "unit": UNIT, "ms_per_step": rms_,
                     "steps": 1, "path": "plain FP64 kernel",
                     "kernels_ms": {k: float(np.mean(v)) for k, v in rk.items()}}
            plain["speedup_of_chosen_form"] = value / plain["value"]
        del rout

    # ---- the other forms on the same workload (one timed step each) -------
    others = {}
    for oform in ([] if args.no_plain else other_forms(w, form)):
        ostep, oout = make_device_step(gsc, torch, w, oform, dev, stream)
        ostep()
        torch.cuda.synchronize()
        ot, ok_, _ = timed_steps(torch, gsc, ostep, stream, 2, flush)
        gsc.device_status()
        oms = max_over_ranks(world, float(np.mean(ot)))
        others[oform] = {"value": work * world / (oms * 1e-3) / 1e9, "unit": UNIT,
                         "ms_per_step": oms,
                         "kernels_ms": {k: float(np.mean(v)) for k, v in ok_.items()},
                         "error_vs_oracle": check(oout) if check else None}
        del oout

    # ---- the plain FP64 kernel on the flattened meshgrid of a grid ----------
    if plain is None and form != "plain" and not args.no_plain:
        pstep, pout = make_device_step(gsc, torch, w, "plain", dev, stream)
        pstep()
        torch.cuda.synchronize()
        pt, pk, _ = timed_steps(torch, gsc, pstep, stream, 1, flush)
        pms = max_over_ranks(world, float(np.mean(pt)))
        plain = {"value": work * world / (pms * 1e-3) / 1e9, "unit": UNIT, "ms_per_step": pms,
                 "steps": 1, "path": "plain FP64 kernel on the flattened meshgrid",
                 "kernels_ms": {k: float(np.mean(v)) for k, v in pk.items()}}
        plain["speedup_of_chosen_form"] = value / plain["value"]
        del pout

    # ---- CPU baseline (rank 0, N=1 only) -----------------------------------
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        v, cores, m, t = time_cpu(w, 1, cpu_seconds)
        cpu = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"{m} seeded points of the workload x all {N} modes, "
                         f"{t:.1f} s on {cores} threads (oracle/field_oracle.c, "
                         f"a restatement of src/field.rs; the Rust crate cannot be built here)"}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": ("f16 split operands, f32 accumulation (leading product exact), f64 output"
                  if form == "sep_f16x5" else
                  "f16/bf16 split operands, f32 accumulation, f64 output" if form.startswith("sep_")
                  else "u32 fixed-point phase, f32 (sincos, tile sums), f64 output"
                  if form == "mixed" else
                  "f64 phase, f32 (sincos, tile sums), f64 output"
                  if form.startswith("mixed") else "f64"),
        "data": "synthetic (seeded numpy default_rng)",
        "config": {"workload": wname, "desc": w["desc"], "points": P, "modes": N,
                   "point_modes": work, "form": form,
                   "l2": "flushed by a 256 MiB write before every timed step",
                   "warmup_steps_run": warm,
                   "clocks_window": "nvidia-smi every 50 ms over warm-up and timed steps",
                   "wall_s": t_wall},
        "error_vs_fp64_full": full,
        "error_vs_oracle": err,
        "plain_fp64": plain,
        "other_forms": others,
        "kernels_ms_per_step": {k: float(np.sum(v) / args.steps) for k, v in kern.items()},
        "gpu_launches": int(launches),
        "roofline": roof, "cpu_baseline": cpu, "e2e": e2e,
        "e2e_structured_api": e2e_structured, "dropin_e2e_default_tolerance": dropin,
        "clocks": clk.summary(),
    }
    del out_d, flush
    torch.cuda.empty_cache()
    return line


# ---------------------------------------------------------------------------
# c5: the batched ensemble
# ---------------------------------------------------------------------------
def ensemble_cpu_rate(items, target_s, steps=1):
    """Oracle throughput on a bounded sample of the ensemble: every 32nd
    realization, a seeded subset of its points, all its modes; the subset is
    sized so one pass takes about target_s on all host threads."""
    import oracle
    cores = host_cores()
    rng = np.random.default_rng(99)
    picked = items[::32]

    def sample(m):
        out = []
        for it in picked:
            P = it["pos"].shape[1]
            idx = np.sort(rng.choice(P, size=min(P, m), replace=False))
            out.append((it, np.ascontiguousarray(it["pos"][:, idx])))
        return out

    def run(smp):
        t0 = time.perf_counter()
        for it, pos in smp:
            oracle.summator(it["cov"], it["z1"], it["z2"], pos, num_threads=cores)
        return time.perf_counter() - t0

    probe = sample(4 * cores)
    dt = max(run(probe), 1e-6)
    m = int(max(4 * cores, 4 * cores * target_s / dt))
    smp = sample(m)
    times = [run(smp) for _ in range(steps)]
    work = sum(pos.shape[1] * it["cov"].shape[1] for it, pos in smp)
    t = float(np.mean(times))
    desc = (f"realizations 0, 32, ..., 480 ({len(smp)} of {len(items)}), up to {m} seeded "
            f"points each x all their modes ({work:.3g} point*modes), {t:.1f} s on {cores} "
            f"threads (oracle/field_oracle.c, a restatement of src/field.rs)")
    return work / t / 1e9, cores, desc, t


def run_ours_batch(args, world, rank, local, cpu_seconds, form_arg="auto"):
    import torch
    import gstools_core as gsc
    import oracle

    torch.cuda.set_device(local)
    items = ensemble(stride=args.ensemble_stride)
    work = float(sum(it["pos"].shape[1] * it["cov"].shape[1] for it in items))
    dims = {}
    for it in items:
        k = (it["pos"].shape[0], False)
        dims[k] = dims.get(k, 0.0) + it["pos"].shape[1] * it["cov"].shape[1] / work
    form = "mixed" if form_arg == "auto" else form_arg
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    dput = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    dev_items = [{"kind": "scalar", "cov": dput(it["cov"]), "z1": dput(it["z1"]),
                  "z2": dput(it["z2"]), "pos": dput(it["pos"]),
                  "out": torch.empty(it["pos"].shape[1], dtype=torch.float64, device=dev)}
                 for it in items]
    in_bytes = sum((it["cov"].size + 2 * it["cov"].shape[1] + it["pos"].size) * 8 for it in items)
    out_bytes = sum(it["pos"].shape[1] * 8 for it in items)

    t0 = time.perf_counter()
    plan = gsc.Batch(dev_items, form=form, timing=True)
    t_plan = time.perf_counter() - t0
    cfg = plan.config

    def step():
        plan.run_graph(stream.cuda_stream)

    with ClockSampler(local) as clk:
        warm = warm_up(torch, step, args.warmup, args.min_warmup_s, flush=flush)
        barrier(world)
        torch.cuda.synchronize()
        t_wall = time.perf_counter()
        per_step = []
        for _ in range(args.steps):
            flush.fill_(1)
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            step()
            b.record(stream)
            b.synchronize()
            per_step.append(a.elapsed_time(b))
        torch.cuda.synchronize()
        barrier(world)
        t_wall = time.perf_counter() - t_wall
    gsc.device_status()
    ms_step = max_over_ranks(world, float(np.mean(per_step)))
    value = work * world / (ms_step * 1e-3) / 1e9

    # per-kernel times of the same run sequence outside the graph
    flush.fill_(1)
    plan.run(stream.cuda_stream)
    torch.cuda.synchronize()
    kt = gsc.last_timings()
    kern = {}
    for name, ms in kt:
        kern[name] = kern.get(name, 0.0) + ms
    dom = max(kern, key=kern.get)
    roof = roofline(args, None, dom, kern[dom], 1, units=work, op_mix=dims, wname="c5")

    # parity on a spread of realizations against the oracle
    err = None
    pin_idx = {}
    if not args.no_check:
        rng = np.random.default_rng(7)
        worst, worst_rms = 0.0, 0.0
        for r in (0, 1, 100, 255, 256, 301, 511):
            it = items[r]
            P = it["pos"].shape[1]
            idx = np.sort(rng.choice(P, size=min(P, 512), replace=False))
            ref = oracle.summator(it["cov"], it["z1"], it["z2"],
                                  np.ascontiguousarray(it["pos"][:, idx]), num_threads=host_cores())
            pin_idx[r] = (idx, ref)
            got = dev_items[r]["out"].cpu().numpy()[idx]
            rms = float(np.sqrt(np.mean(ref ** 2)))
            worst = max(worst, float(np.max(np.abs(got - ref)) / rms))
            worst_rms = max(worst_rms, float(np.sqrt(np.mean((got - ref) ** 2)) / rms))
        err = {"max_abs_over_rms": worst, "rms_over_rms": worst_rms,
               "points_checked": "512 per realization of 0, 1, 100, 255, 256, 301, 511",
               "reference": "oracle (field.rs restatement), FP64"}

    # e2e through the host-array API (before the plain FP64 arm, so that it
    # runs in the same state of the GPU as the timed steps): the ensemble
    # call, and the drop-in -- one summate() per realization at tolerance 1e-6,
    # as GSTools calls the reference for every field of an ensemble
    e2e, dropin = None, None
    if not args.no_e2e:
        host = [{"kind": "scalar", "cov": it["cov"], "z1": it["z1"], "z2": it["z2"],
                 "pos": it["pos"]} for it in items]
        gsc.summate_batch(host, form=form)          # plan + tuning + staging buffers
        ts = []
        for _ in range(max(1, min(args.steps, 3))):
            barrier(world)
            t0 = time.perf_counter()
            gsc.summate_batch(host, form=form)
            ts.append(time.perf_counter() - t0)
        # one more call with the library's event timing, for the split
        gsc.summate_batch(host, form=form, timing=True)
        kms = [split_timings(gsc.last_timings())]
        t_e2e = max_over_ranks(world, float(np.mean(ts)))
        e2e = {"value": work * world / t_e2e / 1e9, "unit": UNIT,
               "h2d_bytes_per_step": int(in_bytes), "d2h_bytes_per_step": int(out_bytes),
               "ms_per_step": t_e2e * 1e3, "ms_each": [t * 1e3 for t in ts],
               "api": "gstools_core.summate_batch (the ensemble in one call; C ABI "
                      "gsc_summate_batch_f64, no reference counterpart)",
               "kernel_ms_per_step": float(np.mean([k for k, _ in kms])),
               "copy_ms_per_step": float(np.mean([c for _, c in kms])),
               "timing": "host wall clock around the synchronous call (kernel_ms_per_step, "
                         "copy_ms_per_step: one further call's own kernels and host-device "
                         "copies, CUDA events on its streams)"}
        # one untimed pass: every call shape's launch choices tuned and cached,
        # as they are for the ensemble call above
        for it in items:
            gsc.summate(it["cov"], it["z1"], it["z2"], it["pos"], tolerance=1e-6)
        ts = []
        for _ in range(2):
            barrier(world)
            t0 = time.perf_counter()
            for it in items:
                gsc.summate(it["cov"], it["z1"], it["z2"], it["pos"], tolerance=1e-6)
            ts.append(time.perf_counter() - t0)
        t_d = max_over_ranks(world, float(np.mean(ts)))
        dropin = {"value": work * world / t_d / 1e9, "unit": UNIT, "ms_per_step": t_d * 1e3,
                  "h2d_bytes_per_step": int(in_bytes), "d2h_bytes_per_step": int(out_bytes),
                  "api": "gstools_core.summate(cov_samples, z1, z2, pos, tolerance=1e-6), one "
                         "call per realization (512 calls per step)",
                  "timing": "host wall clock around the 512 synchronous calls"}

    # the plain FP64 form of the same ensemble (one graph step), whose
    # outputs are the full-field reference of every realization
    plain, full = None, None
    if (not args.no_plain or not args.no_check) and form != "plain":
        ref_items = [dict(d, out=torch.empty_like(d["out"])) for d in dev_items]
        pplan = gsc.Batch(ref_items, form="plain", timing=True)
        pplan.run_graph(stream.cuda_stream)
        torch.cuda.synchronize()
        flush.fill_(1)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        pplan.run_graph(stream.cuda_stream)
        b.record(stream)
        b.synchronize()
        pms = max_over_ranks(world, a.elapsed_time(b))
        plain = {"value": work * world / (pms * 1e-3) / 1e9, "unit": UNIT, "ms_per_step": pms,
                 "steps": 1, "path": "persistent FP64 batch kernel", "config": pplan.config}
        plain["speedup_of_chosen_form"] = value / plain["value"]
        if not args.no_check:
            worst, worst_rms, n_vals, pin = 0.0, 0.0, 0, 0.0
            for d, rd in zip(dev_items, ref_items):
                e = full_error(torch, d["out"], rd["out"])
                worst = max(worst, e["max_abs_over_rms"])
                worst_rms = max(worst_rms, e["rms_over_rms"])
                n_vals += e["values_checked"]
            for r, (idx, ref) in pin_idx.items():
                got = ref_items[r]["out"].cpu().numpy()[idx]
                pin = max(pin, float(np.max(np.abs(got - ref)) / np.sqrt(np.mean(ref ** 2))))
            full = {"max_abs_over_rms": worst, "rms_over_rms": worst_rms,
                    "values_checked": n_vals,
                    "per": "worst realization (each relative to its own field RMS)",
                    "reference": f"persistent plain FP64 batch kernel on the GPU, itself "
                                 f"{pin:.2e} of RMS from the oracle on the checked points "
                                 f"in this run",
                    "reference_vs_oracle": pin}
        pplan.close()
        del ref_items

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        v, cores, desc, _ = ensemble_cpu_rate(items, cpu_seconds)
        cpu = {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": desc}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": ("u32 fixed-point phase, f32 (sincos, tile sums), f64 output"
                  if form == "mixed" else "f64 phase, f32 (sincos, tile sums), f64 output"
                  if form.startswith("mixed") else "f64"),
        "data": "synthetic (seeded numpy default_rng, one seed per realization)",
        "config": {"workload": "c5" if args.ensemble_stride == 1 else
                   f"c5 every {args.ensemble_stride}th realization (profiling case)",
                   "desc": f"batched ensemble, {len(items)} realizations, "
                   f"{sum(it['pos'].shape[1] for it in items)} points, "
                   f"{sum(it['cov'].shape[1] for it in items)} modes in total",
                   "point_modes": work, "form": form, "plan": cfg, "plan_s": t_plan,
                   "step": "one CUDA-graph replay: tables, persistent kernel, split reduction",
                   "l2": "flushed by a 256 MiB write before every timed step",
                   "warmup_steps_run": warm,
                   "clocks_window": "nvidia-smi every 50 ms over warm-up and timed steps",
                   "wall_s": t_wall},
        "error_vs_fp64_full": full,
        "error_vs_oracle": err,
        "plain_fp64": plain,
        "kernels_ms_per_step": kern,
        # one replay: the range and table kernels (one timing record), the
        # persistent kernel, and the split reduction when items are split
        "gpu_launches": int((3 + (1 if cfg.get("max_splits", 1) > 1 else 0)) * args.steps),
        "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "dropin_e2e": dropin,
        "clocks": clk.summary(),
    }
    plan.close()
    del dev_items, flush
    torch.cuda.empty_cache()
    return line


# ---------------------------------------------------------------------------
# field: the reference's criterion field benchmarks, file inputs
# ---------------------------------------------------------------------------
def field_calls(args):
    """[(name, kind, dim, arrays...)] of benches/main.rs:76-132 from the input files."""
    from gstools_core import bench_inputs
    import tempfile
    d = args.input_dir
    if not d or not all(os.path.exists(os.path.join(d, f))
                        for f in bench_inputs.FILES_1D + bench_inputs.FILES_2D):
        d = tempfile.mkdtemp(prefix="gsc_field_inputs_")
        bench_inputs.synthesize_field_inputs(d)
        source = "synthesized stand-ins in the benches/input text format"
    else:
        source = f"files in {d}"
    a = bench_inputs.field_inputs(d)
    calls = [
        ("field summate 2d", "scalar", (a["cov_samples_2d"], a["z_1"], a["z_2"], a["pos_2d"])),
        ("field summate 3d", "scalar", (a["cov_samples_3d"], a["z_1"], a["z_2"], a["pos_3d"])),
        ("field summate incompr 2d", "incompr",
         (a["cov_samples_2d"], a["z_1"], a["z_2"], a["pos_2d"])),
        ("field summate incompr 3d", "incompr",
         (a["cov_samples_3d"], a["z_1"], a["z_2"], a["pos_3d"])),
        ("field summate Fourier 2d", "fourier",
         (a["spectrum_factor_2d"], a["modes_2d"], a["z_1_fourier"], a["z_2_fourier"],
          a["pos_2d"])),
    ]
    return calls, source


def field_work(calls):
    w = 0.0
    for _, kind, arrs in calls:
        pos = arrs[-1]
        n = arrs[1].shape[1] if kind == "fourier" else arrs[0].shape[1]
        w += float(pos.shape[1]) * n
    return w


def field_oracle(kind, arrs, cores):
    import oracle
    if kind == "fourier":
        return oracle.summator_fourier(*arrs, num_threads=cores)
    if kind == "incompr":
        return oracle.summator_incompr(*arrs, num_threads=cores)
    return oracle.summator(*arrs, num_threads=cores)


def run_ours_field(args, world, rank, local, form_arg="auto"):
    import torch
    import gstools_core as gsc

    torch.cuda.set_device(local)
    calls, source = field_calls(args)
    work = field_work(calls)
    form = "plain" if form_arg == "auto" else form_arg
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    dput = lambda x: torch.from_numpy(np.ascontiguousarray(x)).to(dev)
    dev_calls = []
    for name, kind, arrs in calls:
        darrs = [dput(x) for x in arrs]
        pos = arrs[-1]
        shape = (pos.shape[0], pos.shape[1]) if kind == "incompr" else (pos.shape[1],)
        out = torch.empty(shape, dtype=torch.float64, device=dev)
        fn = {"scalar": gsc.summate_device, "incompr": gsc.summate_incompr_device,
              "fourier": gsc.summate_fourier_device}[kind]
        dev_calls.append((name, kind, fn, darrs, out))

    def step(timing=False):
        for _, _, fn, darrs, out in dev_calls:
            fn(*darrs, out, form=form, stream=stream.cuda_stream, timing=timing)

    with ClockSampler(local) as clk:
        warm = warm_up(torch, step, args.warmup, args.min_warmup_s, timing=True, flush=flush)
        barrier(world)
        torch.cuda.synchronize()
        t_wall = time.perf_counter()
        per_step, kern, launches = [], {}, 0
        for _ in range(args.steps):
            flush.fill_(1)
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _, _, fn, darrs, out in dev_calls:
                fn(*darrs, out, form=form, stream=stream.cuda_stream, timing=True)
                for kname, ms in gsc.last_timings():
                    kern.setdefault(kname, []).append(ms)
                    launches += 1
            b.record(stream)
            b.synchronize()
            per_step.append(a.elapsed_time(b))
        barrier(world)
        t_wall = time.perf_counter() - t_wall
    gsc.device_status()
    ms_step = max_over_ranks(world, float(np.mean(per_step)))
    value = work * world / (ms_step * 1e-3) / 1e9
    tot = {k: float(np.sum(v)) / args.steps for k, v in kern.items()}
    dom = max(tot, key=tot.get)
    # units and dimension mix of the calls that ran the dominant kernel
    inc = "incompr" in dom
    mix, units = {}, 0.0
    for _, kind, arrs in calls:
        if (kind == "incompr") != inc:
            continue
        n = arrs[1].shape[1] if kind == "fourier" else arrs[0].shape[1]
        u = float(arrs[-1].shape[1]) * n
        key = (arrs[-1].shape[0], inc)
        mix[key] = mix.get(key, 0.0) + u
        units += u
    mix = {k: v / units for k, v in mix.items()}
    roof = roofline(args, None, dom, tot[dom], 1, units=units, op_mix=mix, wname="field")

    cores = host_cores()
    per_call, err = {}, {}
    for (name, kind, arrs), (_, _, fn, darrs, out) in zip(calls, dev_calls):
        ref = field_oracle(kind, arrs, cores)
        got = out.cpu().numpy()
        rms = float(np.sqrt(np.mean(ref ** 2)))
        err[name] = float(np.max(np.abs(got - ref)) / rms)
    # per call, device-resident, like criterion's per-function report
    for name, kind, fn, darrs, out in dev_calls:
        fn(*darrs, out, form=form, stream=stream.cuda_stream)
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(5):
            fn(*darrs, out, form=form, stream=stream.cuda_stream)
        b.record(stream)
        b.synchronize()
        per_call[name] = a.elapsed_time(b) / 5

    e2e = None
    if not args.no_e2e:
        host = {"scalar": gsc.summate, "incompr": gsc.summate_incompr,
                "fourier": gsc.summate_fourier}
        h2d = sum(sum(x.size for x in arrs) * 8 for _, _, arrs in calls)
        d2h = sum((arrs[-1].shape[0] if k == "incompr" else 1) * arrs[-1].shape[1] * 8
                  for _, k, arrs in calls)
        for _, kind, arrs in calls:
            host[kind](*arrs, form=form)
        ts = []
        for _ in range(max(1, args.steps)):
            t0 = time.perf_counter()
            for _, kind, arrs in calls:
                host[kind](*arrs, form=form)
            ts.append(time.perf_counter() - t0)
        t_e2e = max_over_ranks(world, float(np.mean(ts)))
        e2e = {"value": work * world / t_e2e / 1e9, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "ms_per_step": t_e2e * 1e3,
               "api": "gstools_core.summate / summate_incompr / summate_fourier",
               "timing": "host wall clock around the five synchronous calls"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        t0 = time.perf_counter()
        for _, kind, arrs in calls:
            field_oracle(kind, arrs, cores)
        t = time.perf_counter() - t0
        cpu = {"value": work / t / 1e9, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"the full five calls ({work:.3g} point*modes), {t:.2f} s on {cores} "
                         f"threads (oracle/field_oracle.c)"}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if form.startswith("plain") else
                 "f32 pairs (phase), f32 (sincos, tile sums), f64 output",
        "data": source,
        "config": {"workload": "field", "desc": "benches/main.rs field benchmarks: summate "
                   "2d/3d, summate_incompr 2d/3d, summate_fourier 2d, 1e4 points x 1000 modes",
                   "form": form, "point_modes": work,
                   "l2": "flushed by a 256 MiB write before every timed step",
                   "warmup_steps_run": warm, "wall_s": t_wall},
        "per_call_ms": per_call,
        "error_vs_oracle": {"max_abs_over_rms": err,
                            "reference": "oracle (field.rs restatement), FP64"},
        "kernels_ms_per_step": tot,
        "gpu_launches": int(launches),
        "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk.summary(),
    }
    return line


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh)
    except OSError:
        return {}


# FP64 pipe instructions per point*mode of the plain kernel's table path
# (phase 2d-1, reduction + polynomials + table combine 12, accumulate 1 or d)
PLAIN_FP64_OPS = {(1, False): 14, (2, False): 16, (3, False): 18, (2, True): 17, (3, True): 20}
# Instructions per point*mode of the mixed kernel (mixed_fx.cu) on the FMA
# pipe, by kind, counted from the source for calls whose every |BI| < 2^20
# (all workloads here): (high integer products, low integer products, FP32
# operations).  Per dimension one high product (BF Xh), one low product
# (BI' Xh) and one FP32 FMA (BI Xl 2^-29 in the chain); then 9 FP32 for the
# remainder float, its polynomials and the term; eight modes' terms are added
# (7 additions) before a 4-instruction Kahan step, 1.375 per point*mode; the
# incompressible field weights each pair per component (2 per pair) and adds
# the pairs before its Kahan step, 1.875 per point*mode and component.  The
# table index, shifts, the addition of the FP32 products' bits and the table
# load run on other pipes.  The kinds issue at different rates on the FMA
# pipe (measured live by gsc_selftest_pipe_rates: on GB300 about 30, 60 and
# 116 per clock per SM), so each is weighted by the FP32 rate over its own.
MIXED_OPS = {(1, False): (1, 1, 11.375), (2, False): (2, 2, 12.375), (3, False): (3, 3, 13.375),
             (2, True): (2, 2, 14.75), (3, True): (3, 3, 17.625)}


# DRAM bytes (read + write) per launch of the dominant kernel, from one ncu
# capture each (summaries in profiles/); None where no capture exists
PROFILED_TRAFFIC = {
    ("sep_tc_f16x5", "c2"): (12.49e6 + 88.12e6, "profiles/sep_tc_f16x5_c2.md"),
    ("sep_tc_f16x5", "c4"): (167.4e6, "profiles/sep_tc_f16x5_c4.md"),
    ("plain_f64_scalar", "c1"): (5.8e6, "profiles/plain_f64_scalar_c1.md"),
    ("mixed_scalar", "c1"): (1.906e6, "profiles/mixed_fx_c1.md"),
    ("mixed_scalar", "c3"): (411.7e6 + 115.0e6, "profiles/mixed_fx_c3.md"),
    ("batch_mixed", "c5"): (2275.9e6 + 668.5e6, "profiles/batch_fx_c5.md"),
}


def roofline(args, w, dom, dom_ms, launches_per_step, units=None, op_mix=None, wname=None):
    """Roofline entry for the dominant kernel.

    Tensor-core forms (bound "tensor"): FLOPs per launch = products x 2 x
    points x 2N (the real GEMM has K = 2N per output component; "products" is
    the number of split products the kernel issues: 5 for sep_f16x5, 3 for
    sep_f16x3 / sep_bf16x3), against the measured dense 16-bit peak.
    Plain FP64 form (bound "fp64"): the FP64 pipe instructions the kernel
    issues per point*mode (PLAIN_FP64_OPS), each counted as one fused
    multiply-add (2 FLOPs, the unit of the peak), against cuBLAS DGEMM
    measured on this GPU.  Mixed form (bound "fma_pipe"): its FMA-pipe
    instructions per point*mode by kind (MIXED_OPS), each weighted by the
    FP32 FMA rate over its kind's rate (both measured here), i.e. in FP32-FMA
    issue slots, times 2 FLOPs, against the FP32 FMA rate itself."""
    import torch
    if units is None:
        P, N = n_points(w), w["cov"].shape[1]
        units = P * N
    per_launch_units = units / max(launches_per_step, 1)
    traffic, tsrc = PROFILED_TRAFFIC.get((dom, wname), (None, None))
    entry = _roofline_entry(args, w, dom, dom_ms, per_launch_units, op_mix, torch)
    entry["traffic"] = traffic
    if tsrc:
        entry["traffic_source"] = f"ncu dram__bytes_read.sum + dram__bytes_write.sum, {tsrc}"
    return entry


def _roofline_entry(args, w, dom, dom_ms, per_launch_units, op_mix, torch):
    if dom.startswith("sep_tc"):
        d = w["dim"]
        nout = d if w["incompr"] else 1
        products = {"sep_tc_f16x5": 5, "sep_tc_f16x3": 3, "sep_tc_bf16x3": 3}[dom]
        flops = products * 2.0 * per_launch_units * 2 * nout
        achieved = flops / (dom_ms * 1e-3) / 1e12
        peaks = measured_peaks()
        peak = peaks.get("bf16_tflops")
        how = "MEASURED_PEAKS.json bf16_tflops (burst, cuBLAS bf16; f16 runs at the same rate)"
        if peak is None:
            peak, how = 1900.0, "fallback 1.9 PFLOP/s"
        return {"bound": "tensor", "kernel": dom, "achieved": achieved, "peak": peak,
                "unit": "TFLOP/s", "frac": achieved / peak, "traffic": None,
                "peak_source": how,
                "algorithmic_tflops_single_product": achieved / products,
                "note": f"{products} split products x 2 x points x 2N FLOPs per launch"}
    if op_mix is None:
        op_mix = {(w["dim"], bool(w["incompr"])): 1.0}
    # the algorithmic work per point*mode: 2d+3 FLOPs and one sincos (scalar),
    # 4d+2 FLOPs and one sincos (incompressible)
    alg = sum(f * ((4 * k[0] + 2) if k[1] else (2 * k[0] + 3)) for k, f in op_mix.items())
    rate = per_launch_units / (dom_ms * 1e-3)
    algo = {"flops_per_point_mode": alg, "tflops": alg * rate / 1e12, "sincos_per_s": rate}
    if dom == "mixed_f64phase":
        return {"bound": "fp32", "kernel": dom, "achieved": None, "peak": None, "unit": "TFLOP/s",
                "frac": None, "traffic": None, "algorithmic": algo,
                "note": "no instruction count kept for the FP64-phase variant"}
    if "mixed" in dom:
        hi_r, imad_r, ffma_r = pipe_rates()
        w_hi, w_imad = ffma_r / hi_r, ffma_r / imad_r
        kinds = [sum(f * MIXED_OPS[k][i] for k, f in op_mix.items()) for i in range(3)]
        slots = kinds[0] * w_hi + kinds[1] * w_imad + kinds[2]
        achieved = 2.0 * slots * rate / 1e12
        peak = 2.0 * ffma_r / 1e12
        return {"bound": "fma_pipe", "kernel": dom, "achieved": achieved, "peak": peak,
                "unit": "TFLOP/s", "frac": achieved / peak, "traffic": None,
                "peak_source": "measured here: FP32 FMA issue rate of independent chains "
                               "(gsc_selftest_pipe_rates), x 2 FLOPs",
                "fma_slots_per_point_mode": slots,
                "ops_per_point_mode": {"imad_hi": kinds[0], "imad": kinds[1], "fp32": kinds[2]},
                "weights": {"imad_hi": w_hi, "imad": w_imad, "fp32": 1.0},
                "fp32_sgemm_tflops": fp32_peak(torch)[0],
                "algorithmic": algo,
                "note": "FMA-pipe issue slots per point*mode (kinds counted from the kernel "
                        "source, weighted by their measured issue rates) x 2 FLOPs"}
    ops = sum(f * PLAIN_FP64_OPS[k] for k, f in op_mix.items())
    achieved = 2.0 * ops * per_launch_units / (dom_ms * 1e-3) / 1e12
    peak, how = fp64_peak(torch)
    return {"bound": "fp64", "kernel": dom, "achieved": achieved,
            "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak if peak else None,
            "traffic": None, "peak_source": how,
            "pipe_ops_per_point_mode": ops, "algorithmic": algo,
            "note": f"{ops:.1f} FP64 pipe instructions per point*mode "
                    f"(from the kernel source), each counted as one FMA = 2 FLOPs"}


_PEAKS = {}


def _gemm_peak(torch, dtype, name):
    """Best of 5 cuBLAS GEMMs 8192^3 (TF32 off), TFLOP/s."""
    if name not in _PEAKS:
        n = 8192
        prev = torch.backends.cuda.matmul.allow_tf32
        torch.backends.cuda.matmul.allow_tf32 = False
        a = torch.randn(n, n, dtype=dtype, device="cuda")
        b = torch.randn(n, n, dtype=dtype, device="cuda")
        torch.matmul(a, b)
        torch.cuda.synchronize()
        best = 1e9
        for _ in range(5):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b)
            e1.record()
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1))
        torch.backends.cuda.matmul.allow_tf32 = prev
        _PEAKS[name] = 2 * n ** 3 / (best * 1e-3) / 1e12
        del a, b
    return _PEAKS[name]


def fp64_peak(torch):
    """FP64 peak as delivered by cuBLAS DGEMM on this GPU (measured here);
    MEASURED_PEAKS.json carries no FP64 figure."""
    return _gemm_peak(torch, torch.float64, "fp64"), "measured: cuBLAS DGEMM 8192^3, best of 5"


def fp32_peak(torch):
    """FP32 (CUDA-core) peak as delivered by cuBLAS SGEMM with TF32 off."""
    return (_gemm_peak(torch, torch.float32, "fp32"),
            "measured: cuBLAS SGEMM 8192^3 (TF32 off), best of 5")


def pipe_rates():
    """(high integer multiply-adds, low integer multiply-adds, FP32 FMAs) per
    second on this GPU, measured once by the library's issue-rate probe."""
    if "pipe" not in _PEAKS:
        import ctypes
        from gstools_core import _native
        r = (ctypes.c_double * 3)()
        _native.check(_native.lib.gsc_selftest_pipe_rates(-1, r))
        _PEAKS["pipe"] = (r[0], r[1], r[2])
    return _PEAKS["pipe"]


# ---------------------------------------------------------------------------
def reference_line(args, world, wname, cpu_seconds):
    """The reference's CPU algorithm (oracle restatement) on the host cores,
    one JSON record for workload `wname`."""
    common = {"impl": "reference", "metric": METRIC, "unit": UNIT, "n_gpus": world,
              "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
              "scaling": "weak", "vs_baseline": None, "dtype": "f64"}
    if wname == "field":
        calls, source = field_calls(args)
        work = field_work(calls)
        cores = host_cores()
        ts = []
        for _ in range(max(1, args.steps)):
            t0 = time.perf_counter()
            for _, kind, arrs in calls:
                field_oracle(kind, arrs, cores)
            ts.append(time.perf_counter() - t0)
        t = float(np.mean(ts))
        v = work / t / 1e9
        return dict(common, value=v, ms_per_step=t * 1e3, data=source,
                    config={"workload": "field", "desc": "benches/main.rs field benchmarks",
                            "form": "reference CPU (rayon-equivalent restatement)"},
                    cpu_baseline={"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                                  "sample": "the full five calls per step"},
                    e2e={"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0})
    if wname == "c5":
        items = ensemble()
        v, cores, desc, t = ensemble_cpu_rate(items, cpu_seconds, max(1, args.steps))
        return dict(common, value=v, ms_per_step=t * 1e3,
                    data="synthetic (seeded numpy default_rng, one seed per realization)",
                    config={"workload": "c5", "desc": "batched ensemble, 512 realizations",
                            "form": "reference CPU (rayon-equivalent restatement)"},
                    cpu_baseline={"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                                  "sample": desc},
                    e2e={"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0})
    w = workload(wname)
    N = w["cov"].shape[1]
    v, cores, m, t = time_cpu(w, max(1, args.steps), cpu_seconds)
    return dict(common, value=v, ms_per_step=t * 1e3, data="synthetic (seeded numpy default_rng)",
                config={"workload": wname, "desc": w["desc"], "points": n_points(w), "modes": N,
                        "form": "reference CPU (rayon-equivalent restatement)"},
                cpu_baseline={"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                              "sample": f"{m} seeded points x all {N} modes per step"},
                e2e={"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                note="the Rust crate cannot be compiled here (no cargo/rustc); the arm times "
                     "oracle/field_oracle.c, a bit-exact restatement of src/field.rs, on all "
                     "host threads")


def run_reference(args, world, rank):
    if rank != 0:
        return
    if args.workload != "all":
        print(json.dumps(reference_line(args, world, args.workload, args.cpu_seconds)))
        return
    line = reference_line(args, world, HEADLINE, args.cpu_seconds)
    configs = {n: reference_line(args, world, n, args.cpu_seconds_other)
               for n in ALL_WORKLOADS if n != HEADLINE}
    configs[HEADLINE] = dict(line)
    line["configs"] = configs
    line["config"] = dict(line["config"],
                          workload=f"{HEADLINE} (headline; every workload under configs)")
    print(json.dumps(line))


ALL_WORKLOADS = ("c1", "c2", "c3", "c4", "c5")
HEADLINE = "c5"          # the largest workload: 1.7e11 point*modes per step


def run_workload(args, world, rank, local, wname, cpu_seconds, form_arg):
    if wname == "c5":
        return run_ours_batch(args, world, rank, local, cpu_seconds, form_arg)
    if wname == "field":
        return run_ours_field(args, world, rank, local, form_arg)
    return run_ours(args, world, rank, local, wname, cpu_seconds, form_arg)


def run_all(args, world, rank, local):
    """Every workload in turn; the headline's JSON record carries them all."""
    lines = {}
    for n in ALL_WORKLOADS:
        lines[n] = run_workload(args, world, rank, local, n,
                                args.cpu_seconds if n == HEADLINE else args.cpu_seconds_other,
                                "auto")
    head = dict(lines[HEADLINE])
    head["configs"] = lines
    head["config"] = dict(head["config"],
                          workload=f"{HEADLINE} (headline; every workload under configs)")
    fr = [l["error_vs_fp64_full"]["max_abs_over_rms"] for l in lines.values()
          if l.get("error_vs_fp64_full")]
    head["summary"] = {
        n: {"value": l["value"], "form": l["config"]["form"], "ms_per_step": l["ms_per_step"],
            "e2e": (l.get("e2e") or {}).get("value"),
            "max_err_full": (l.get("error_vs_fp64_full") or {}).get("max_abs_over_rms"),
            "speedup_vs_plain_fp64": (l.get("plain_fp64") or {}).get("speedup_of_chosen_form"),
            "roofline_frac": (l.get("roofline") or {}).get("frac"),
            "cpu": (l.get("cpu_baseline") or {}).get("value")}
        for n, l in lines.items()}
    head["summary"]["max_err_full_all"] = max(fr) if fr else None
    return head


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="all",
                    choices=["all", "c1", "c2", "c3", "c4", "c5", "field"])
    ap.add_argument("--input-dir", default=None,
                    help="benches/input directory of the reference (workload field)")
    ap.add_argument("--form", default="auto", help="form of a single workload (not 'all')")
    ap.add_argument("--cpu-seconds", type=float, default=10.0,
                    help="CPU baseline sample of the headline (or the single) workload")
    ap.add_argument("--cpu-seconds-other", type=float, default=3.0,
                    help="CPU baseline sample of the other workloads of 'all'")
    ap.add_argument("--ensemble-stride", type=int, default=1,
                    help="c5: every k-th realization only (a small case for profilers; "
                         "not a bench line)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-check", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--min-warmup-s", type=float, default=0.5,
                    help="keep warming up until this many seconds passed (clock sampling)")
    args = ap.parse_args()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        if args.workload == "all":
            line = run_all(args, world, rank, local)
        else:
            line = run_workload(args, world, rank, local, args.workload, args.cpu_seconds,
                                args.form)
        if rank == 0:
            print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
