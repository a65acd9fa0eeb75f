#!/usr/bin/env python
"""Benchmark of the LES time step on GB300.

Metric: Mcell-steps/s = n1m*n2m*n3m*steps / seconds / 1e6, one step being the
three RK3 substeps with SGS, momentum RHS + ADI, Poisson, projection,
temperature and the per-step checks.  Workload (default, `--config
channel590`): the turbulent channel at Re_tau ~ 590 with passive heat
transfer, 2pi x 2 x pi, 384x256x384 cells (37.7M), seeded synthetic initial
field (laminar profile + 10% uniform perturbation) -- the largest of the
benchmark's configurations that runs on one GPU.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Our arm (one JSON line on rank 0):
  value    : device-resident throughput of the mixed-precision form (FP32
             stencils, SGS and x/z ADI sweeps; FP64 wall-normal sweeps,
             projection, flow-rate and divergence; Poisson solves in FP32
             under an FP64 defect correction where timed faster); every step is
             bracketed by CUDA events on the case's own stream and L2 is
             flushed (256 MiB write) between timed steps, outside the timed
             region.  `--form fp64` times the plain FP64 form instead.
  fp64, mixed_vs_fp64, error : with the default form, the FP64 form is timed
             the same way on the same config, and `error` states the mixed
             form's deviation from it after `steps` steps from the same
             initial field (relative L2 of u, v, w, p, t; divergence; bulk
             velocity; drag and heat flux).
  e2e      : the same metric through the C ABI with host buffers: each step
             uploads u,v,w,p,t from pinned host memory (lesgpu_set_fields),
             steps (lesgpu_step, which reads the step report back) and
             downloads u,v,w,p,t (lesgpu_get_fields); host wall clock.
  roofline : the dominant kernel class (largest device time in the
             instrumented steps), its algorithmic bytes per launch divided by
             its average launch time (events on the launching stream), against
             the measured HBM copy bandwidth.  Algorithmic bytes: each distinct
             operand read once and each result written once, at the width it
             is stored in (FP32 mirrors, histories and SGS temporaries of the
             mixed form at 4 B, FP64 state at 8 B); `step_roofline` is the
             whole step against the per-phase model of the hot path (289 FP64
             words per cell-step for the channel, with the same precision map
             for the mixed form); `traffic` is the dominant class's measured
             DRAM bytes per launch from the committed ncu summary
             (profiles/roofline_traffic.md) when it holds the workload.
  serving  : a bounded sample of the serving stream through lesgpu_server
             (mixed form, cases admitted and advanced concurrently): p50/p99
             time-to-solution and aggregate Mcell-steps/s, beside the same
             cases run one at a time in the FP64 form.
  cpu_baseline : the CPU oracle (C/OpenMP restatement of the solver, the
             reference's Fortran cannot be built on this host) on a bounded
             sample of the same workload with OMP threads set to every host
             core (stated in `cores`), and `single_thread`: the same oracle
             with one thread on a bounded sample (one step of the 64^3
             channel).
Reference arm (--impl reference): the same CPU restatement timed on the same
config with every host core; rank 0 alone runs under torchrun.

Multi-GPU: replicas only (one independent case per GPU, no collective on the
data path); value = all ranks' cell-steps / max over ranks of the time.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mcell-steps/s (mixed vs FP64 GPU) at stated error; p50/p99 served-case latency"
UNIT = "Mcell-steps/s"

KCLASS = {1: "rhs", 2: "adi", 3: "sgs_filter", 4: "poisson", 5: "rhs_t"}


def poisson_words(case, rep):
    """FP64 words per cell of one Poisson solve: poiss_ftft 6 (divgsum in,
    phi out, the half spectrum's round trips between the z and x passes);
    poiss_z_ft / poiss_x_ft 4 + 14 per V-cycle (mean over the step's
    substeps); poiss_mgrd 2 + 44 per BiCGSTAB iteration (two V-cycles, two
    operator applications, the vector updates)."""
    from leswht_gb300 import abi
    its = [x for x in rep["poisson_iters"] if x > 0] or [0]
    nbar = sum(its) / len(its)
    pk = case.settings.get("poisson", abi.POISSON_FTFT)
    if pk in (abi.POISSON_Z_FT, abi.POISSON_X_FT):
        return 4.0 + 14.0 * nbar, nbar
    if pk == abi.POISSON_MGRD:
        return 2.0 + 44.0 * nbar, nbar
    return 6.0, 0.0


def poisson_bytes(case, form, rep):
    """Bytes per cell of one Poisson solve: poisson_words at 8 B, except that
    the mixed form's multigrid cycles (poiss_z_ft / poiss_x_ft), which relax
    and transfer the correction in FP32, count 4 B per cycle word."""
    from leswht_gb300 import abi
    w, nbar = poisson_words(case, rep)
    if form == "mixed" and case.settings.get("poisson") in (abi.POISSON_Z_FT, abi.POISSON_X_FT):
        return 4.0 * 8 + 14.0 * nbar * 4
    return w * 8


def class_bytes(case, form, rep):
    """Algorithmic bytes per cell and per step of each instrumented kernel
    class: every distinct operand read once and every result written once,
    at the width it is stored in.  The FP64 form stores everything in 8 B;
    the mixed form reads FP32 mirrors of the fields and eddy viscosities,
    keeps its RK3 histories and SGS temporaries in FP32 (4 B), and keeps the
    right-hand sides, the fields and the wall-normal sweep's operands in FP64.
      rhs    : read u,v,w,p [nu, nu1(3)], rk3o(3); write rhs(3) (FP64),
               rk3o(3), rk3oo(3)                         3 launches a step
      adi    : per component: z reads and writes rhs (FP64) and reads its
               viscosity; y reads rhs, its viscosity (FP64) and writes the
               intermediate (FP64); x reads the intermediate and its
               viscosity and adds to the field (FP64 read + write); the
               x and z sweeps run in FP32 in the mixed form
      sgs_filter : 24 (Vreman) + 19 (EDM) test-filtered temporaries, each
               read and written once                      once a step
      poisson : poisson_bytes                            3 solves a step
      rhs_t  : read t,u,v,w [al1(3)], rk3to; write rhs (FP64), rk3to, rk3too"""
    s = case.settings
    f = 4 if form == "mixed" else 8
    les = s.get("iles", 0) == 1
    ht = s.get("ihtrans", 0) == 1
    dyn = s.get("idvmon", 0) == 1
    nc = 3 if case.grid.n3m != 1 else 2
    nvx = f if les else 0          # viscosity of an x or z sweep
    nvy = 8 if les else 0          # of the FP64 wall-normal sweep
    out = {}
    out["rhs"] = 3 * ((4 + (4 if les else 0) + 3) * f + 3 * 8 + 6 * f)
    per_comp = (16 + nvx) + (16 + nvy) + (24 + nvx)
    out["adi"] = 3 * (nc + (1 if ht else 0)) * per_comp
    nf = (24 if les and dyn else 0) + (19 if les and dyn and ht else 0)
    out["sgs_filter"] = nf * 2 * f
    out["poisson"] = 3 * poisson_bytes(case, form, rep)
    out["rhs_t"] = 3 * ((4 + (3 if les else 0) + 1) * f + 8 + 2 * f) if ht else 0
    return out


def step_bytes(case, form, rep):
    """Bytes per cell-step of the whole step by the per-phase minimum-traffic
    model of the hot path: in FP64 words, per substep RHS + SGS cross terms
    17 (+3 rk3oo with IB), ADI 8 per momentum component, divergence 4,
    Poisson (poisson_words), projection 11, flow-rate scalars 5 (ICH = 1;
    else the CFL pass, 1), rhs_t 12, temperature ADI 8, tvolcalc 3 (ICH = 1);
    per step the SGS model 19 (9 momentum + 10 thermal); plus per IB forcing
    point and component 87 words a substep.  For the channel this is 289
    words (2312 B) per cell-step.  The mixed form's FP32-stored operands
    (field mirrors read by the FP32 stencils and x/z sweeps, RK3 histories,
    SGS velocities) count 4 B; everything else 8 B."""
    from leswht_gb300 import abi
    s = case.settings
    f = 4 if form == "mixed" else 8
    ib = s.get("ibmon", 0) == 1
    ht = s.get("ihtrans", 0) == 1
    ich = s.get("ich", 0) == 1
    nc = 3 if case.grid.n3m != 1 else 2
    rhs = 11 * f + 3 * 8 + 3 * f + (3 * f if ib else 0)
    adi = nc * (48 + 2 * f)
    sub = rhs + adi + 4 * 8 + poisson_bytes(case, form, rep) + 11 * 8 + (5 if ich else 1) * 8
    if ht:
        sub += 9 * f + 8 + 2 * f + (48 + 2 * f) + (3 * 8 if ich else 0)
    step = 3 * sub + (3 * f + 48) + ((4 * f + 48) if ht else 0)
    if ib and case.ibm is not None:
        nint = sum(int(case.ibm["nintp"][l]) for l in range(4 if ht else 3))
        nin = sum(int(case.ibm["nbody"][l]) - int(case.ibm["nintp"][l]) for l in range(4 if ht else 3))
        step += 3 * (87 * nint + 3 * nin) * 8 / case.cells
    return step


def load_traffic(config, form):
    """Measured DRAM bytes (read + write) per cell and per step of each kernel
    class, from the ncu summary profiles/roofline_traffic.md (rows
    `| config | form | class | bytes per cell-step | ...`), or {}."""
    out = {}
    path = os.path.join(ROOT, "profiles", "roofline_traffic.md")
    try:
        with open(path) as fh:
            for line in fh:
                cols = [x.strip() for x in line.strip().strip("|").split("|")]
                if len(cols) >= 4 and cols[0] == config and cols[1] == form:
                    try:
                        out[cols[2]] = float(cols[3])
                    except ValueError:
                        pass
    except OSError:
        pass
    return out


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def make_case(name, form):
    from leswht_gb300 import abi, cases
    prec = abi.PREC_FP64 if form == "fp64" else abi.PREC_MIXED
    if name == "channel64":
        return cases.channel(64, 64, 64, precision=prec)
    if name == "channel590":
        return cases.PRESETS["channel590"](precision=prec)
    if name == "channel_small":
        return cases.channel(32, 32, 16, precision=prec)
    if name == "channel590_slab":
        return cases.channel(384, 64, 384, lx=2 * math.pi, lz=math.pi, re=10950.0, precision=prec)
    if name == "cylinder100":
        return cases.PRESETS["cylinder100"](precision=prec)
    if name == "cylinder3900":
        return cases.PRESETS["cylinder3900"](precision=prec)
    if name == "cylinder100_mgrd":
        return cases.with_poisson(cases.PRESETS["cylinder100"](precision=prec), abi.POISSON_MGRD)
    if name == "channel64_mgrd":
        return cases.with_poisson(cases.channel(64, 64, 64, precision=prec), abi.POISSON_MGRD)
    raise SystemExit(f"unknown config {name}")


WORKLOAD = {
    "channel64": "turbulent channel Re_tau~180 with passive heat transfer, 4pi x 2 x 4pi/3, 64x64x64 cells, "
                 "tanh wall-normal stretching (gamma 2.75), CFR forcing, dynamic Vreman + dynamic EDM, poiss_ftft",
    "channel590": "turbulent channel Re_tau~590 with passive heat transfer, 2pi x 2 x pi, 384x256x384 cells, poiss_ftft",
    "channel_small": "turbulent channel 32x32x16 (test size)",
    "channel590_slab": "the Re_tau~590 channel's 384x384 x-z plane with 64 wall-normal cells (9.4M cells): "
                       "per-kernel ncu captures at the x/z line lengths of channel590 with ~3 GB resident",
    "cylinder100": "heated circular cylinder Re=100 Pr=0.71, 30D x 20D x pi D, 128x96x16 cells clustered at the "
                   "body (first spacing 0.02D), uniform inflow, convective outlet, slip lateral walls, periodic z, "
                   "dynamic SGS, direct-forcing IB, poiss_z_ft (z FFT + x-y multigrid)",
    "cylinder3900": "heated circular cylinder Re=3900 Pr=0.71, 30D x 20D x pi D, 256x192x64 cells clustered at the "
                    "body, IB direct forcing, poiss_z_ft",
    "cylinder100_mgrd": "the cylinder100 case solved with poiss_mgrd (BiCGSTAB + MG3D V-cycle, NLEV 3)",
    "channel64_mgrd": "the channel64 case solved with poiss_mgrd (BiCGSTAB + MG3D V-cycle, NLEV 5)",
}


class Clocks:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            with open(self.path) as f:
                for line in f:
                    parts = [x.strip() for x in line.split(",")]
                    if len(parts) >= 9:
                        rows.append(parts)
            os.unlink(self.path)
        except Exception:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            for n, v in zip(names, r[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def host_threads():
    """Host cores this process may use (the OpenMP thread count of the CPU legs)."""
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def oracle_steps(name, threads, seconds=None, warmup=1, steps=None):
    """The oracle on `threads` OpenMP threads: `warmup` untimed steps, then
    `steps` timed steps (or as many as fit in `seconds`, at least one)."""
    import oracle
    from leswht_gb300 import solver
    case = make_case(name, "fp64")
    lib = oracle.load()
    lib.ref_set_threads(int(threads))
    if lib.ref_get_threads() != int(threads):
        raise RuntimeError("could not set the oracle's thread count")
    s = solver.Solver(lib, "ref_", case)
    for _ in range(warmup):
        s.step()                               # page-in, first touch
    n, t0 = 0, time.perf_counter()
    while True:
        s.step()
        n += 1
        el = time.perf_counter() - t0
        if steps is not None:
            if n >= steps:
                break
        elif el >= seconds or n >= 200:
            break
    s.close()
    return case, n, el


def cpu_baseline(name, seconds=12.0):
    """The oracle on the host cores: a bounded sample of the same workload on
    every core, and one step of the 64^3 channel on one core."""
    threads = host_threads()
    case, n, el = oracle_steps(name, threads, seconds=seconds)
    out = {"value": case.cells * n / el / 1e6, "unit": UNIT, "cores": threads, "kind": "port",
           "sample": f"{n} steps of {case.name} after 1 warm-up step ({el:.1f} s), C/OpenMP oracle, "
                     f"OMP threads = {threads}",
           "steps": n, "seconds": el}
    c1, n1, e1 = oracle_steps("channel64", 1, steps=1)
    out["single_thread"] = {"value": c1.cells * n1 / e1 / 1e6, "unit": UNIT, "cores": 1,
                            "sample": f"{n1} step of {c1.name} after 1 warm-up step ({e1:.1f} s), OMP threads = 1"}
    c2, n2, e2 = oracle_steps("channel64", threads, steps=2)
    out["single_thread"]["same_sample_all_cores"] = c2.cells * n2 / e2 / 1e6
    return out


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    threads = host_threads()
    os.environ["OMP_NUM_THREADS"] = str(threads)
    case, n, el = oracle_steps(args.config, threads, warmup=args.warmup, steps=args.steps)
    v = case.cells * args.steps / el / 1e6
    sample = (f"{args.steps} timed steps of {case.name} after {args.warmup} warm-up, C/OpenMP restatement of "
              f"the reference solver on {threads} OMP threads (the Fortran reference cannot be compiled: no "
              "Fortran compiler on the host)")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded PCG64 perturbation of the laminar profile)",
            "config": {"workload": WORKLOAD[args.config], "cells": case.cells, "form": "fp64 CPU"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def time_form(args, form, lib, dev, world, rank, flush, full):
    """Time one arithmetic form of the step on this GPU.  Returns the
    device-resident figures and, when `full`, the live per-kernel-class
    timings, the roofline of the dominant class and the end-to-end figure."""
    import numpy as np
    import torch
    import leswht_gb300
    from leswht_gb300 import abi

    case = make_case(args.config, form)
    s = leswht_gb300.gpu_solver(case)
    h = s.h
    stream_ptr = C.c_void_p()
    lib.lesgpu_stream(h, C.byref(stream_ptr))
    stream = torch.cuda.ExternalStream(stream_ptr.value, device=torch.device("cuda", dev))

    def check(rc, what):
        if rc != 0:
            raise RuntimeError(f"{what}: {lib.lesgpu_strerror(rc).decode()}")

    for _ in range(args.warmup):                     # warm-up (captures the step graph)
        check(lib.lesgpu_step_async(h, 1), "step")
    torch.cuda.synchronize()
    kps = C.c_int64()
    check(lib.lesgpu_launch_count(h, C.byref(kps)), "launch_count")

    # ---- device-resident timed region
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    with Clocks(dev) as clk:
        with torch.cuda.stream(stream):
            for q in range(args.steps):
                flush.zero_()
                ev[q][0].record(stream)
                check(lib.lesgpu_step_async(h, 1), "step")
                ev[q][1].record(stream)
        torch.cuda.synchronize()
    step_ms = [x.elapsed_time(y) for x, y in ev]
    tot_s = sum(step_ms) / 1e3
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([tot_s], device=f"cuda:{dev}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        tot_s = float(t.item())
    rep = s.report()
    import leswht_gb300
    tuned = [({"dir": "xyz"[d], "components": nc, "fp32": bool(f32), "tiled": True} if w == 128 else
              {"dir": "xyz"[d], "components": nc, "fp32": bool(f32), "lanes_per_line": w & 63,
               "register_capped": bool(w & 64)}) if d < 3 else
             {"fft": "xyz"[nc], "lines_per_block": w} if d == 3 else {"mg_cluster_blocks": w} if d == 4 else
             {"ftft_fp32_with_fp64_correction": bool(w)}
             for d, nc, f32, w in leswht_gb300.tuning(lib, h)]
    out = {"case": case, "value": world * case.cells * args.steps / tot_s / 1e6, "autotune": tuned,
           "ms_per_step": tot_s / args.steps * 1e3, "kernels_per_step": int(kps.value),
           "clocks": clk.summary(), "report": rep,
           "step_ms": {"min": min(step_ms), "median": statistics.median(step_ms), "max": max(step_ms)}}
    if not full or rank != 0:
        s.close()
        return out

    # ---- live per-kernel-class timing (instrumented eager steps)
    kstats = {}
    nins = max(2, min(args.steps, 5))
    for cls in (1, 2, 3, 4, 5):
        check(lib.lesgpu_instrument(h, cls), "instrument")
        with torch.cuda.stream(stream):
            for q in range(nins):
                flush.zero_()
                check(lib.lesgpu_step_async(h, 1), "step")
        ms, n = C.c_double(), C.c_int64()
        check(lib.lesgpu_instrument_read(h, C.byref(ms), C.byref(n)), "instrument_read")
        if n.value > 0:
            kstats[KCLASS[cls]] = {"ms_total": ms.value, "launches": n.value,
                                   "avg_us": ms.value / n.value * 1e3, "cls": cls,
                                   "launches_per_step": n.value / nins}
    check(lib.lesgpu_instrument(h, 0), "instrument")
    peak, src = peaks()
    cb = class_bytes(case, form, rep)
    traffic = load_traffic(args.config, form)
    for k, d in kstats.items():
        per_step = cb.get(k, 0) * case.cells            # algorithmic bytes of the class in one step
        d["algorithmic_bytes_per_launch"] = per_step / d["launches_per_step"]
        d["achieved_gbs"] = d["algorithmic_bytes_per_launch"] / (d["avg_us"] * 1e-6) / 1e9
        d["frac"] = d["achieved_gbs"] / peak
        if k in traffic:
            d["dram_bytes_per_launch"] = traffic[k] * case.cells / d["launches_per_step"]
    dom_name, dom = max(kstats.items(), key=lambda kv: kv[1]["ms_total"])
    out["roofline"] = {"bound": "hbm", "achieved": dom["achieved_gbs"], "peak": peak, "unit": "GB/s",
                       "frac": dom["frac"], "traffic": dom.get("dram_bytes_per_launch"), "kernel": dom_name,
                       "peak_source": src, "algorithmic_bytes_per_launch": dom["algorithmic_bytes_per_launch"],
                       "avg_launch_us": dom["avg_us"], "kernels": kstats,
                       "traffic_source": "profiles/roofline_traffic.md" if dom_name in traffic else None}
    sb = step_bytes(case, form, rep)
    step_gbs = sb * case.cells / (out["ms_per_step"] * 1e-3) / 1e9
    out["step_roofline"] = {"bytes_per_cell_step": sb, "fp64_words_per_cell_step": sb / 8.0,
                            "achieved": step_gbs, "peak": peak, "unit": "GB/s", "frac": step_gbs / peak,
                            "model": "per-phase minimum traffic of the hot path, stored widths of the form"}

    # ---- end to end through the C ABI with host buffers
    shape = case.grid.shape
    host = {k: torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy() for k in ("u", "v", "w", "p", "t")}
    f0 = s.fields()
    for k in host:
        host[k][...] = f0[k]
    r0 = s.report()
    tm, dt, ih, m = r0["time"], r0["dt"], r0["ihist"], r0["m"]
    ptr = lambda a: a.ctypes.data_as(abi.PD)
    rep_s = abi.StepReport()
    n_e2e = max(3, min(args.steps, 20))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(n_e2e):
        check(lib.lesgpu_set_fields(h, *(ptr(host[k]) for k in ("u", "v", "w", "p", "t")), tm, dt, ih, m), "set_fields")
        check(lib.lesgpu_step(h, C.byref(rep_s)), "step")
        check(lib.lesgpu_get_fields(h, *(ptr(host[k]) for k in ("u", "v", "w", "p", "t"))), "get_fields")
        tm, dt, ih, m = rep_s.time, rep_s.dt, rep_s.ihist, rep_s.m
    el = time.perf_counter() - t0
    nbytes = 5 * int(np.prod(shape)) * 8
    out["e2e"] = {"value": case.cells * n_e2e / el / 1e6, "unit": UNIT, "h2d_bytes_per_step": nbytes,
                  "d2h_bytes_per_step": nbytes + C.sizeof(abi.StepReport), "steps": n_e2e,
                  "path": "lesgpu_set_fields + lesgpu_step + lesgpu_get_fields, pinned host buffers"}
    s.close()
    return out


def form_error(args, nsteps):
    """The mixed form's error against the FP64 form: both run `nsteps` steps
    from the same initial field; relative L2 of each field, the divergence
    after the last projection, and the drag / heat-flux / bulk diagnostics."""
    import numpy as np
    import leswht_gb300
    a = leswht_gb300.gpu_solver(make_case(args.config, "fp64"))
    b = leswht_gb300.gpu_solver(make_case(args.config, "mixed"))
    for _ in range(nsteps):
        ra, rb = a.step(), b.step()
    fa, fb = a.fields(), b.fields()

    def rel(x, y):
        d = float(np.linalg.norm(y))
        return float(np.linalg.norm(x - y)) / (d if d > 0 else 1.0)

    def reldiff(x, y):
        return abs(x - y) / max(abs(y), 1e-300)

    err = {"steps": nsteps, "rel_l2": {k: rel(fb[k], fa[k]) for k in ("u", "v", "w", "p", "t")},
           "max_div_mixed": rb["dvmax"], "max_div_fp64": ra["dvmax"],
           "ubulk_rel": reldiff(rb["ubulk"], ra["ubulk"])}
    if make_case(args.config, "fp64").settings.get("ibmon", 0) == 1:
        err["drag_rel"] = reldiff(rb["cd"][0], ra["cd"][0])
    err["heat_flux_x_abs"] = abs(rb["heat_flux"][0] - ra["heat_flux"][0])
    a.close(); b.close()
    return err


def long_horizon(config, nsteps, avg_from):
    """The mixed form against the FP64 form over a configuration's own
    horizon: both run `nsteps` steps from the same initial field with
    field_avg on, its sums restarted after step `avg_from`; the statistics
    of the window after it are compared (leswht_gb300.stats): max divergence
    over the run, relative L2 of u and T at the end, mean and rms profiles
    (channel) or fields (cylinder), drag, Strouhal and Nusselt numbers."""
    import numpy as np
    import leswht_gb300
    from leswht_gb300 import stats
    runs = {}
    for form in ("fp64", "mixed"):
        case = make_case(config, form)
        case.settings.update(iavg=1, avg_tst=0.0)
        sol = leswht_gb300.gpu_solver(case)
        hist, dvmax, unconv = [], 0.0, 0
        t0 = time.perf_counter()
        for n in range(1, nsteps + 1):
            r = sol.step()
            dvmax = max(dvmax, r["dvmax"])
            unconv += r["poisson_unconverged"]
            if n == avg_from:
                sol.averages(reset=True)
            elif n > avg_from:
                hist.append(r)
        avg, nsamp = sol.averages()
        runs[form] = {"case": case, "hist": hist, "avg": avg, "nsamp": nsamp, "fields": sol.fields(),
                      "dvmax": dvmax, "unconv": unconv, "seconds": time.perf_counter() - t0}
        sol.close()
    a, b = runs["fp64"], runs["mixed"]
    case = a["case"]
    s = case.settings

    def rd(x, y):
        return abs(x - y) / max(abs(y), 1e-300)

    out = {"steps": nsteps, "window_steps": len(a["hist"]),
           "window_time": sum(r["dt"] for r in a["hist"]),
           "max_div": {"fp64": a["dvmax"], "mixed": b["dvmax"]},
           "poisson_unconverged": {"fp64": a["unconv"], "mixed": b["unconv"]},
           "rel_l2_end": {k: stats.rel_l2(b["fields"][k], a["fields"][k]) for k in ("u", "t")},
           "seconds": {"fp64": a["seconds"], "mixed": b["seconds"]}}
    st = {}
    for form, r in runs.items():
        times = [q["time"] for q in r["hist"]]
        dts = [q["dt"] for q in r["hist"]]
        win = float(sum(dts))
        m = stats.mean_and_rms(r["avg"], win)
        d = {"m": m, "drag": stats.time_mean(times, dts, [q["cd"][0] for q in r["hist"]])}
        if s.get("ibmon", 0) == 1:
            d["strouhal"] = stats.strouhal(times, [q["cd"][1] for q in r["hist"]])
            if s.get("ihtrans", 0) == 1:
                hb = stats.time_mean(times, dts, [q["heat_body"] for q in r["hist"]])
                d["nusselt"] = stats.cylinder_nusselt(hb, s["re"], s["pr"], 2.0 * s["body"]["r"],
                                                      case.grid.zl, 0.0 - s["tflu_i"])
        else:
            d["wall_shear"] = stats.time_mean(times, dts, [-q["pmi"][0] for q in r["hist"]])
            if s.get("ihtrans", 0) == 1:
                d["nusselt"] = stats.channel_nusselt(m["t"], m["u"], case.grid)
        st[form] = d
    fa, fb = st["fp64"], st["mixed"]
    keys = [k for k in ("u_rms", "v_rms", "w_rms", "t_rms") if k in fa["m"]]
    if s.get("ibmon", 0) == 1:
        out["rms_rel_l2"] = {k: stats.rel_l2(fb["m"][k], fa["m"][k]) for k in keys}
        out["mean_rel_l2"] = {k: stats.rel_l2(fb["m"][k], fa["m"][k]) for k in ("u", "t") if k in fa["m"]}
        out["drag"] = {"fp64": fa["drag"], "mixed": fb["drag"], "rel": rd(fb["drag"], fa["drag"])}
        out["strouhal"] = {"fp64": fa["strouhal"], "mixed": fb["strouhal"],
                           "rel": rd(fb["strouhal"], fa["strouhal"]) if fa["strouhal"] and fb["strouhal"] else None}
    else:
        out["rms_profile_rel_l2"] = {k: stats.rel_l2(stats.plane_profile(fb["m"][k]), stats.plane_profile(fa["m"][k]))
                                     for k in keys}
        out["mean_profile_rel_l2"] = {k: stats.rel_l2(stats.plane_profile(fb["m"][k]),
                                                      stats.plane_profile(fa["m"][k]))
                                      for k in ("u", "t") if k in fa["m"]}
        out["wall_shear"] = {"fp64": fa["wall_shear"], "mixed": fb["wall_shear"],
                             "rel": rd(fb["wall_shear"], fa["wall_shear"])}
    if "nusselt" in fa:
        out["nusselt"] = {"fp64": fa["nusselt"], "mixed": fb["nusselt"], "rel": rd(fb["nusselt"], fa["nusselt"])}
    return out


def serving_sample(args, lib):
    """A bounded sample of the serving stream (seeded Poisson arrivals at
    2 cases/s; grid, body, Re and Pr drawn as in the benchmark stream), run
    through the server in the mixed form, then the same cases one at a time
    in the FP64 form.  p50/p99 are times from arrival to completion."""
    from leswht_gb300 import abi, serving
    stream = serving.c4_stream(n_cases=args.serving_cases, rate=2.0, nsteps=args.serving_steps)
    keys = ("p50_s", "p99_s", "mcell_steps_per_s", "elapsed_s")
    out = {"sample": f"{args.serving_cases} cases x {args.serving_steps} steps of the seeded serving stream "
                     "(Poisson arrivals 2/s; grids 64x48x8 .. 256x192x32; circle/square/sphere; Re 40-1000; "
                     "Pr 0.71/7); the benchmark stream has 256 cases x 500 steps"}
    if args.serving_legs in ("both", "realtime"):
        # real-time replay: latency (p50/p99 from arrival) at the stream's rate
        srv = serving.Server(lib, hbm_budget_bytes=64 << 30, max_active=16, steps_in_flight=4)
        mixed = serving.serve(srv, stream, precision=abi.PREC_MIXED)
        srv.close()
        seq = serving.one_at_a_time(lib, stream, precision=abi.PREC_FP64)
        out["realtime"] = {"served_mixed": {k: mixed[k] for k in keys + ("completed",)},
                           "one_at_a_time_fp64": {k: seq[k] for k in keys},
                           "throughput_ratio": mixed["mcell_steps_per_s"] / seq["mcell_steps_per_s"]}
    if args.serving_legs == "realtime":
        return out
    # saturated: every case arrives at once, so aggregate throughput is the
    # GPU's, not the arrival rate's
    srv = serving.Server(lib, hbm_budget_bytes=64 << 30, max_active=16, steps_in_flight=4)
    mixed = serving.serve(srv, stream, precision=abi.PREC_MIXED, time_scale=1e9)
    srv.close()
    seq = serving.one_at_a_time(lib, stream, precision=abi.PREC_FP64, time_scale=1e9)
    out["saturated"] = {"served_mixed": {k: mixed[k] for k in keys + ("completed",)},
                        "one_at_a_time_fp64": {k: seq[k] for k in keys},
                        "throughput_ratio": mixed["mcell_steps_per_s"] / seq["mcell_steps_per_s"]}
    return out


def profile_one_step(args):
    """For an ncu capture with --profile-from-start off: build the case,
    start it (autotuning included) and run `warmup` steps, then one step
    between cudaProfilerStart and cudaProfilerStop; prints one line."""
    import torch
    import leswht_gb300
    torch.cuda.set_device(0)
    lib = leswht_gb300.load_library()
    case = make_case(args.config, args.form)
    s = leswht_gb300.gpu_solver(case)
    for _ in range(args.warmup):
        if lib.lesgpu_step_async(s.h, 1) != 0:
            raise RuntimeError("step failed")
    torch.cuda.synchronize()
    kps = C.c_int64()
    lib.lesgpu_launch_count(s.h, C.byref(kps))
    torch.cuda.profiler.start()
    if lib.lesgpu_step_async(s.h, 1) != 0:
        raise RuntimeError("step failed")
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    print(json.dumps({"profiled": case.name, "form": args.form, "cells": case.cells,
                      "kernels_per_step": int(kps.value)}))
    s.close()
    return 0


def run_ours(args):
    import torch
    import leswht_gb300

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world != args.gpus and world > 1:
        print(f"warning: WORLD_SIZE={world} but --gpus {args.gpus}", file=sys.stderr)
    dev = local if torch.cuda.device_count() > local else 0
    torch.cuda.set_device(dev)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", dev))
    lib = leswht_gb300.load_library()
    if lib.lesgpu_set_device(dev) != 0:
        raise RuntimeError("lesgpu_set_device failed")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{dev}")

    main = time_form(args, args.form, lib, dev, world, rank, flush, full=True)
    other_form = "fp64" if args.form == "mixed" else None
    other = time_form(args, other_form, lib, dev, world, rank, flush, full=False) if other_form else None

    if rank == 0:
        case, rep = main["case"], main["report"]
        cpu = None
        if world == 1 and not args.no_cpu:
            cpu = cpu_baseline(args.config, seconds=args.cpu_seconds)
        line = {"metric": METRIC, "value": main["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": main["ms_per_step"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.form == "fp64" else "f32/f64",
                "data": "synthetic (seeded PCG64 perturbation of the laminar profile)",
                "config": {"workload": WORKLOAD[args.config], "cells": case.cells, "form": args.form,
                           "l2": "flushed between timed steps (256 MiB write, outside the timed region)",
                           "parallelism": "replicas" if world > 1 else "single GPU"},
                "roofline": main.get("roofline"), "step_roofline": main.get("step_roofline"),
                "cpu_baseline": cpu, "e2e": main.get("e2e"),
                "gpu_launches": main["kernels_per_step"] * args.steps, "kernels_per_step": main["kernels_per_step"],
                "clocks": main["clocks"],
                "check": {"dvmax": rep["dvmax"], "ubulk": rep["ubulk"], "csgsts": rep["csgsts"],
                          "time": rep["time"], "dt": rep["dt"]},
                "step_ms": main["step_ms"], "autotune": main["autotune"]}
        if args.serving_cases > 0 and world == 1:
            try:
                line["serving"] = serving_sample(args, lib)
            except Exception as e:          # the measured line above stands; say what failed
                line["serving"] = {"error": f"{type(e).__name__}: {e}"}
        if other is not None:
            line["fp64"] = {"value": other["value"], "ms_per_step": other["ms_per_step"],
                            "kernels_per_step": other["kernels_per_step"], "clocks": other["clocks"],
                            "autotune": other["autotune"]}
            line["mixed_vs_fp64"] = main["value"] / other["value"]
            line["gpu_launches"] += other["kernels_per_step"] * args.steps
            line["error"] = form_error(args, args.steps)
        if world == 1:
            acc = {}
            if args.accuracy_steps > 0:
                acc["channel64"] = long_horizon("channel64", args.accuracy_steps, args.accuracy_steps // 2)
            if args.accuracy_c1_steps > 0:
                acc["cylinder100"] = long_horizon("cylinder100", args.accuracy_c1_steps, args.accuracy_c1_steps // 2)
            if args.accuracy_c3_steps > 0:
                acc["cylinder3900"] = long_horizon("cylinder3900", args.accuracy_c3_steps, args.accuracy_c3_steps // 2)
            if acc:
                line["accuracy"] = acc
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", default="channel590", choices=sorted(WORKLOAD))
    ap.add_argument("--form", default="mixed", choices=["fp64", "mixed"],
                    help="mixed (default): the mixed form is timed, then the FP64 form on the same "
                         "config, and the mixed form's error against FP64 is stated")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--serving-cases", type=int, default=16,
                    help="cases in the serving sample (0: skip it)")
    ap.add_argument("--serving-steps", type=int, default=40)
    ap.add_argument("--serving-legs", default="both", choices=["both", "realtime", "saturated"],
                    help="which arrival patterns the serving sample replays (both by default)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--accuracy-steps", type=int, default=2000,
                    help="steps of the 64^3 channel's mixed-vs-FP64 statistics comparison (0: skip); "
                         "statistics over the second half")
    ap.add_argument("--accuracy-c1-steps", type=int, default=0,
                    help="steps of the same comparison on the Re=100 cylinder, 128x96x16, long enough for "
                         "vortex shedding to set in (0: skip)")
    ap.add_argument("--accuracy-c3-steps", type=int, default=0,
                    help="steps of the same comparison on the Re=3900 cylinder, 256x192x64 (0: skip)")
    ap.add_argument("--serving-only", action="store_true",
                    help="run only the serving sample (--serving-cases x --serving-steps) and print it as one "
                         "JSON line, e.g. --serving-cases 64 --serving-steps 500 --serving-legs saturated")
    ap.add_argument("--accuracy-only", action="store_true",
                    help="run only the statistics comparisons and print them as one JSON line")
    ap.add_argument("--profile-one-step", action="store_true",
                    help="run warm-up steps, then one step inside cudaProfilerStart/Stop (for ncu "
                         "--profile-from-start off); no timing, no JSON result line")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.profile_one_step:
        return profile_one_step(args)
    if args.serving_only:
        import torch
        import leswht_gb300
        torch.cuda.set_device(0)
        print(json.dumps({"serving": serving_sample(args, leswht_gb300.load_library())}))
        return 0
    if args.accuracy_only:
        import torch
        torch.cuda.set_device(0)
        acc = {}
        if args.accuracy_steps > 0:
            acc["channel64"] = long_horizon("channel64", args.accuracy_steps, args.accuracy_steps // 2)
        if args.accuracy_c1_steps > 0:
            acc["cylinder100"] = long_horizon("cylinder100", args.accuracy_c1_steps, args.accuracy_c1_steps // 2)
        if args.accuracy_c3_steps > 0:
            acc["cylinder3900"] = long_horizon("cylinder3900", args.accuracy_c3_steps, args.accuracy_c3_steps // 2)
        print(json.dumps({"accuracy": acc}))
        return 0
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
