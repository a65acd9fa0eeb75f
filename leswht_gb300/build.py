"""Build recipe of liblesgpu.so (sm_103a) -- nvcc, no cmake.

Each .cu file under csrc/ is compiled to an object in parallel and the
objects are linked into leswht_gb300/_build/liblesgpu.so with the CUDA
runtime linked statically, so the library needs only the driver at run time.
The compiled case driver (exec/lesgpu_exec.cpp, the counterpart of the
reference's solver_exec) is linked against it as _build/lesgpu_exec with an
$ORIGIN run path.
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
EXEC_SRC = HERE / "exec" / "lesgpu_exec.cpp"
EXEC = BUILD / "lesgpu_exec"
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


def build_exec(force: bool = False) -> Path:
    """g++ the case driver against liblesgpu.so."""
    if not force and EXEC.exists() and EXEC.stat().st_mtime > max(EXEC_SRC.stat().st_mtime, SO.stat().st_mtime):
        return EXEC
    cxx = shutil.which("g++") or "g++"
    tmp = EXEC.with_suffix(".tmp%d" % os.getpid())
    cmd = [cxx, "-std=c++17", "-O2", "-I", str(HERE.parent / "include"), str(EXEC_SRC), "-o", str(tmp),
           "-L", str(BUILD), "-llesgpu", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("g++ failed on lesgpu_exec.cpp:\n" + r.stderr)
    os.replace(tmp, EXEC)
    return EXEC


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and not _stale():
        build_exec()
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
    build_exec(force=True)
    return SO


if __name__ == "__main__":
    import sys
    build(force=True, verbose="-v" in sys.argv)
    print(SO)
