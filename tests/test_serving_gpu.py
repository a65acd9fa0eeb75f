"""Serving loop (lesgpu_server_*): cases submitted together are admitted by
device footprint and advance together -- by default each in its own graph;
with LESGPU_SERVER_BUCKET_MAX=0 the cases of one grid shape as one size
bucket (one graph per bucket step, the multigrid mode solves of the bucket's
cases in one batched launch).  Either way each result is the same as the
case run alone (bitwise: every kernel of a case is deterministic, and the
batched launch gives every case's modes the arithmetic of its own solve).
SPECS holds buckets of three and two cases."""
import time

import numpy as np
import pytest

import leswht_gb300
from leswht_gb300 import abi, cases, serving

pytestmark = pytest.mark.gpu

SPECS = [dict(grid=(64, 48, 8), body=abi.BODY_CYLINDER, center=(0.2, -0.1, 0.5 * np.pi), re=100.0, pr=0.71, seed=1),
         dict(grid=(64, 48, 8), body=abi.BODY_SQUARE, center=(-0.3, 0.25, 0.5 * np.pi), re=300.0, pr=7.0, seed=2),
         dict(grid=(96, 64, 16), body=abi.BODY_SPHERE, center=(0.1, 0.4, 0.5 * np.pi), re=60.0, pr=0.71, seed=3),
         dict(grid=(96, 64, 16), body=abi.BODY_CYLINDER, center=(-0.2, 0.1, 0.5 * np.pi), re=150.0, pr=7.0, seed=4),
         dict(grid=(64, 48, 8), body=abi.BODY_SPHERE, center=(0.0, 0.0, 0.5 * np.pi), re=40.0, pr=0.71, seed=5)]
NSTEPS = 6


def alone(spec, precision):
    s = leswht_gb300.gpu_solver(serving.build_case(spec, precision))
    s.lib.lesgpu_step_async(s.h, NSTEPS)
    s.report()
    return s.fields()


def wait_all(srv, tickets, timeout=120.0):
    t0 = time.time()
    while True:
        st = [srv.poll(t)[0] for t in tickets]
        if all(x in (serving.DONE, serving.FAILED) for x in st):
            return st
        assert time.time() - t0 < timeout
        time.sleep(0.01)


@pytest.mark.parametrize("bucket_max", ["1", "0"])
@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED])
def test_results_same_alone_and_in_the_mix(monkeypatch, precision, bucket_max):
    monkeypatch.setenv("LESGPU_SERVER_BUCKET_MAX", bucket_max)     # read when the server starts
    lib = leswht_gb300.load_library()
    srv = serving.Server(lib, hbm_budget_bytes=32 << 30, max_active=8, steps_in_flight=2)
    tickets = [srv.submit(serving.build_case(sp, precision), NSTEPS) for sp in SPECS]
    st = wait_all(srv, tickets)
    assert st == [serving.DONE] * len(SPECS)
    for sp, tk in zip(SPECS, tickets):
        f, rep, secs = srv.result(tk)
        ref = alone(sp, precision)
        assert rep["ntime"] == NSTEPS and secs > 0.0
        for k in ("u", "v", "w", "p", "t"):
            assert np.array_equal(f[k], ref[k]), k
        srv.release(tk)
    srv.close()


def test_admission_by_footprint_serialises_when_memory_is_short():
    lib = leswht_gb300.load_library()
    # a budget of one small case: the second waits until the first is freed
    srv = serving.Server(lib, hbm_budget_bytes=1, max_active=8, steps_in_flight=2)
    tickets = [srv.submit(serving.build_case(sp, abi.PREC_MIXED), NSTEPS) for sp in SPECS[:2]]
    seen_active = 0
    t0 = time.time()
    while True:
        s = srv.stats()
        seen_active = max(seen_active, s["active"])
        st = [srv.poll(t)[0] for t in tickets]
        if all(x == serving.DONE for x in st):
            break
        assert time.time() - t0 < 120.0
        time.sleep(0.002)
    assert seen_active <= 1
    for tk in tickets:
        srv.release(tk)
    assert srv.stats()["bytes_used"] == 0
    srv.close()


def test_cancel_waiting_request():
    lib = leswht_gb300.load_library()
    srv = serving.Server(lib, hbm_budget_bytes=1, max_active=1, steps_in_flight=2)
    a = srv.submit(serving.build_case(SPECS[0], abi.PREC_MIXED), 40)
    b = srv.submit(serving.build_case(SPECS[1], abi.PREC_MIXED), 40)
    srv.release(b)                       # still waiting: removed
    with pytest.raises(serving.ServerError):
        srv.poll(b)
    assert wait_all(srv, [a]) == [serving.DONE]
    srv.release(a)
    srv.close()


def test_stream_replay_reports_latency():
    lib = leswht_gb300.load_library()
    stream = serving.c4_stream(n_cases=4, rate=50.0, nsteps=4, grids=[(64, 48, 8), (96, 64, 16)])
    srv = serving.Server(lib, hbm_budget_bytes=32 << 30, max_active=8, steps_in_flight=2)
    out = serving.serve(srv, stream)
    srv.close()
    assert out["completed"] == 4 and out["p99_s"] >= out["p50_s"] > 0.0
    assert all(r["dvmax"] < 1e-4 for r in out["records"])
