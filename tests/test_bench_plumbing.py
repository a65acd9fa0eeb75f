"""The benchmark's roofline plumbing on the CPU: the DRAM traffic it reports
beside the roofline fraction comes from the committed ncu summary of the
channel slab, one row per kernel class the bench instruments, and the
per-class algorithmic byte model covers the same classes."""
import importlib.util
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def _bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_traffic_rows_cover_every_instrumented_class():
    b = _bench()
    traffic = b.load_traffic("channel590", "mixed")
    assert set(traffic) == set(b.KCLASS.values())
    assert all(v > 0 for v in traffic.values())


def test_traffic_absent_for_unmeasured_workloads():
    b = _bench()
    assert b.load_traffic("channel64", "mixed") == {}
    assert b.load_traffic("channel590", "fp64") == {}
