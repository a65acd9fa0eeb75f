"""Serving stream of immersed-body LES cases over the lesgpu_server C ABI.

`Server` wraps lesgpu_server_*: cases are submitted as they arrive, admitted
on the device by HBM footprint, advanced together (each resident case on its
own stream and step graph) and read back when done.  `c4_stream` draws the
benchmark stream: seeded Poisson arrivals; grid from {64x48x8, 96x64x16,
128x96x16, 192x128x32, 256x192x32}; body from {circle, square, sphere} with
its centre jittered uniformly by +-0.5 D; Re log-uniform in [40, 1000]; Pr
from {0.71, 7}.  `serve` replays a stream in real time (optionally
time-compressed) and reports p50 / p99 time-to-solution and the aggregate
Mcell-steps/s; `one_at_a_time` runs the same cases sequentially.
"""
from __future__ import annotations

import ctypes as C
import math
import time
from dataclasses import dataclass
from typing import Dict, List, Optional

import numpy as np

from . import abi, cases

GRIDS = [(64, 48, 8), (96, 64, 16), (128, 96, 16), (192, 128, 32), (256, 192, 32)]
BODIES = [abi.BODY_CYLINDER, abi.BODY_SQUARE, abi.BODY_SPHERE]
PRS = [0.71, 7.0]

WAITING, RUNNING, DONE, FAILED, CANCELLED = 0, 1, 2, 3, 4


def declare(lib) -> None:
    P = C.c_void_p
    I = C.c_int64
    lib.lesgpu_server_create.argtypes = [I, I, I, I, C.POINTER(P)]
    lib.lesgpu_server_submit.argtypes = [P, C.POINTER(abi.Config), C.POINTER(abi.Grid), C.POINTER(abi.Ibm),
                                         abi.PD, abi.PD, abi.PD, abi.PD, abi.PD, C.c_double, C.c_double, I, I, I,
                                         C.POINTER(I)]
    lib.lesgpu_server_poll.argtypes = [P, I, C.POINTER(I), C.POINTER(I)]
    lib.lesgpu_server_result.argtypes = [P, I, abi.PD, abi.PD, abi.PD, abi.PD, abi.PD, C.POINTER(abi.StepReport),
                                         C.POINTER(C.c_double)]
    lib.lesgpu_server_release.argtypes = [P, I]
    lib.lesgpu_server_stats.argtypes = [P, C.POINTER(I), C.POINTER(I), C.POINTER(I), C.POINTER(C.c_double)]
    lib.lesgpu_server_destroy.argtypes = [P]
    for n in ("create", "submit", "poll", "result", "release", "stats", "destroy"):
        getattr(lib, "lesgpu_server_" + n).restype = C.c_int


class ServerError(RuntimeError):
    pass


class Server:
    def __init__(self, lib, device: int = 0, hbm_budget_bytes: int = 64 << 30, max_active: int = 32,
                 steps_in_flight: int = 4):
        declare(lib)
        self.lib = lib
        self.h = C.c_void_p()
        self._check(lib.lesgpu_server_create(device, hbm_budget_bytes, max_active, steps_in_flight, C.byref(self.h)),
                    "create")
        self.meta: Dict[int, dict] = {}

    def _check(self, rc, what):
        if rc != 0:
            raise ServerError(f"lesgpu_server_{what}: {abi.ERR_NAMES.get(rc, rc)}")

    def submit(self, case, nsteps: int) -> int:
        cfg = abi.pack_config(case.settings)
        grid = abi.pack_grid(case.grid)
        g = case.grid
        ibm = abi.pack_ibm(case.ibm, g.n1m, g.n2m, g.n3m) if case.ibm is not None else None
        f = {k: np.ascontiguousarray(case.fields[k], dtype=np.float64) for k in ("u", "v", "w", "p", "t")}
        t = C.c_int64()
        ptr = lambda a: a.ctypes.data_as(abi.PD)
        self._check(self.lib.lesgpu_server_submit(self.h, C.byref(cfg), C.byref(grid.struct),
                                                  C.byref(ibm.struct) if ibm is not None else None,
                                                  *(ptr(f[k]) for k in ("u", "v", "w", "p", "t")),
                                                  float(case.time), float(case.dt), int(case.ihist), int(case.m),
                                                  int(nsteps), C.byref(t)), "submit")
        self.meta[t.value] = {"shape": g.shape, "cells": case.cells, "nsteps": nsteps}
        return t.value

    def poll(self, ticket: int):
        st, n = C.c_int64(), C.c_int64()
        self._check(self.lib.lesgpu_server_poll(self.h, ticket, C.byref(st), C.byref(n)), "poll")
        return st.value, n.value

    def result(self, ticket: int):
        sh = self.meta[ticket]["shape"]
        out = {k: np.empty(sh) for k in ("u", "v", "w", "p", "t")}
        rep = abi.StepReport()
        secs = C.c_double()
        self._check(self.lib.lesgpu_server_result(self.h, ticket, *(out[k].ctypes.data_as(abi.PD)
                                                                     for k in ("u", "v", "w", "p", "t")),
                                                  C.byref(rep), C.byref(secs)), "result")
        return out, rep.as_dict(), secs.value

    def release(self, ticket: int):
        self._check(self.lib.lesgpu_server_release(self.h, ticket), "release")
        self.meta.pop(ticket, None)

    def stats(self):
        p, a, b, cs = C.c_int64(), C.c_int64(), C.c_int64(), C.c_double()
        self._check(self.lib.lesgpu_server_stats(self.h, C.byref(p), C.byref(a), C.byref(b), C.byref(cs)), "stats")
        return {"pending": p.value, "active": a.value, "bytes_used": b.value, "cell_steps": cs.value}

    def close(self):
        if self.h:
            self.lib.lesgpu_server_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class Arrival:
    t: float
    spec: dict


def c4_stream(n_cases: int = 256, rate: float = 2.0, seed: int = 20261203, nsteps: int = 500,
              grids=GRIDS) -> List[Arrival]:
    """The seeded serving stream (Poisson arrivals at `rate` cases/s)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out, t = [], 0.0
    for q in range(n_cases):
        t += rng.exponential(1.0 / rate)
        g = grids[int(rng.integers(len(grids)))]
        body = BODIES[int(rng.integers(len(BODIES)))]
        cx, cy = rng.uniform(-0.5, 0.5, size=2)
        re = math.exp(rng.uniform(math.log(40.0), math.log(1000.0)))
        pr = PRS[int(rng.integers(len(PRS)))]
        out.append(Arrival(t, dict(grid=g, body=body, center=(float(cx), float(cy), 0.5 * math.pi),
                                   re=float(re), pr=pr, nsteps=nsteps, seed=seed + q)))
    return out


def build_case(spec: dict, precision: int):
    n1m, n2m, n3m = spec["grid"]
    return cases.cylinder(n1m, n2m, n3m, re=spec["re"], pr=spec["pr"], body_kind=spec["body"],
                          center=spec["center"], seed=spec["seed"], precision=precision,
                          name=f"served_{n1m}x{n2m}x{n3m}")


def serve(server: Server, stream: List[Arrival], precision: int = abi.PREC_MIXED,
          time_scale: float = 1.0, keep_results: bool = False, poll_s: float = 0.002) -> dict:
    """Replay `stream` against `server` (arrival times divided by
    `time_scale`); returns per-case times-to-solution and the aggregate."""
    built = [(a.t / time_scale, build_case(a.spec, precision), a.spec["nsteps"]) for a in stream]
    t0 = time.perf_counter()
    tickets, submitted, nxt = {}, {}, 0
    done: Dict[int, dict] = {}
    while len(done) < len(built):
        now = time.perf_counter() - t0
        while nxt < len(built) and built[nxt][0] <= now:
            tk = server.submit(built[nxt][1], built[nxt][2])
            tickets[tk] = nxt
            submitted[tk] = time.perf_counter()
            nxt += 1
        for tk in list(tickets):
            st, _ = server.poll(tk)
            if st in (DONE, FAILED, CANCELLED):
                q = tickets.pop(tk)
                rec = {"index": q, "state": st, "wall_s": time.perf_counter() - submitted[tk],
                       "cells": built[q][1].cells, "nsteps": built[q][2]}
                if st == DONE:
                    f, rep, secs = server.result(tk)
                    rec["tts_s"] = secs
                    rec["dvmax"] = rep["dvmax"]
                    if keep_results:
                        rec["fields"] = f
                server.release(tk)
                done[q] = rec
        time.sleep(poll_s)
    el = time.perf_counter() - t0
    recs = [done[q] for q in range(len(built))]
    ok = [r for r in recs if r["state"] == DONE]
    tts = np.array([r["tts_s"] for r in ok]) if ok else np.zeros(1)
    work = sum(r["cells"] * r["nsteps"] for r in ok)
    return {"cases": len(recs), "completed": len(ok), "elapsed_s": el,
            "p50_s": float(np.percentile(tts, 50)), "p99_s": float(np.percentile(tts, 99)),
            "mcell_steps_per_s": work / el / 1e6, "records": recs}


def one_at_a_time(lib, stream: List[Arrival], precision: int = abi.PREC_FP64, time_scale: float = 1.0) -> dict:
    """The same cases run one after another, each alone on the GPU, with the
    arrival times (divided by `time_scale`) honoured: a case waits for its
    arrival and for the case before it; time-to-solution counts from arrival."""
    from .solver import Solver
    built = [(a.t / time_scale, build_case(a.spec, precision), a.spec["nsteps"]) for a in stream]
    t0 = time.perf_counter()
    recs = []
    for at, case, nsteps in built:
        now = time.perf_counter() - t0
        start = max(now, at)
        if start > now:
            time.sleep(start - now)
        s = Solver(lib, "lesgpu_", case)
        lib.lesgpu_step_async(s.h, nsteps)
        rep = s.report()          # synchronises
        s.close()
        fin = time.perf_counter() - t0
        recs.append({"tts_s": fin - at, "cells": case.cells, "nsteps": nsteps, "dvmax": rep["dvmax"]})
    el = time.perf_counter() - t0
    tts = np.array([r["tts_s"] for r in recs])
    work = sum(r["cells"] * r["nsteps"] for r in recs)
    return {"cases": len(recs), "elapsed_s": el, "p50_s": float(np.percentile(tts, 50)),
            "p99_s": float(np.percentile(tts, 99)), "mcell_steps_per_s": work / el / 1e6, "records": recs}
