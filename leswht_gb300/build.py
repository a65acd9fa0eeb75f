"""Build recipe of liblesgpu.so (sm_103a) -- nvcc, no cmake.

Each .cu file under csrc/ is compiled to an object in parallel and the
objects are linked into leswht_gb300/_build/liblesgpu.so with the CUDA
runtime linked statically, so the library needs only the driver at run time.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
BUILD = HERE / "_build"
SO = BUILD / "liblesgpu.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def sources():
    return sorted(CSRC.glob("*.cu"))


def _stale() -> bool:
    if not SO.exists():
        return True
    t = SO.stat().st_mtime
    deps = list(sources()) + list(CSRC.glob("*.cuh")) + [HERE.parent / "include" / "lesgpu.h"]
    return any(p.stat().st_mtime > t for p in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and not _stale():
        return SO
    BUILD.mkdir(exist_ok=True)
    nv = nvcc()

    def compile_one(src: Path) -> Path:
        obj = BUILD / (src.stem + ".o")
        cmd = [nv] + ARCH + FLAGS + ["-c", str(src), "-o", str(obj)]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, sources()))
    tmp = SO.with_suffix(".so.tmp%d" % os.getpid())
    cmd = [nv] + ARCH + ["-shared", "-o", str(tmp)] + [str(o) for o in objs] + ["-cudart", "static"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stderr)
    os.replace(tmp, SO)
    return SO


if __name__ == "__main__":
    import sys
    build(force=True, verbose="-v" in sys.argv)
    print(SO)
