"""The C-ABI library loads and exports every entry point include/lesgpu.h
declares (no compute call: this runs without a GPU)."""
import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    text = (ROOT / "include" / "lesgpu.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(lesgpu_[a-z_0-9]+)\s*\(", text)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("lesgpu_create", "lesgpu_step", "lesgpu_set_fields", "lesgpu_get_fields", "lesgpu_destroy"):
        assert s in syms


def test_library_exports_all_declared_symbols(gpu_lib):
    missing = [s for s in declared_symbols() if not hasattr(gpu_lib, s)]
    assert not missing, missing


def test_strerror_and_version(gpu_lib):
    assert gpu_lib.lesgpu_abi_version() == 2
    assert gpu_lib.lesgpu_strerror(-8) == b"option not built in this library"


def test_create_rejects_bad_grid(gpu_lib):
    from leswht_gb300 import abi, cases
    c = cases.channel(16, 16, 8)
    cfg = abi.pack_config(c.settings)
    grid = abi.pack_grid(c.grid)
    grid.struct.n1 = grid.struct.n1m + 5          # inconsistent sizes: rejected before any CUDA call
    h = C.c_void_p()
    assert gpu_lib.lesgpu_create(C.byref(cfg), C.byref(grid.struct), C.byref(h)) == abi.ERR_ARG
    assert gpu_lib.lesgpu_create(None, None, None) == abi.ERR_ARG
