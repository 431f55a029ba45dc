"""Build the native library ``libmqgb.so`` in-tree (sm_103a CUDA kernels + C++ host code).

The host C++ is compiled with ``-ffp-contract=off`` so set-up arithmetic (grid solve,
E field, injection constants) is bit-identical on x86-64 and aarch64 hosts; the FP64
kernels (channel and tandem) and the device Laplace solver are compiled with ``--fmad=false``
for the same reason.  Translation units are
compiled in parallel; the whole build takes well under a minute.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIB = PKG / "libmqgb.so"
CHECK_BUILD = PKG / "_build_check"
CHECK_LIB = PKG / "libmqgb_check.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CXXFLAGS = ["-O3", "-std=c++17", "-fPIC", "-pthread", "-ffp-contract=off", "-Wall", "-Wno-unused-function"]

# (source, extra nvcc flags)
CUDA_UNITS = [
    ("mq_f64.cu", ["--fmad=false"]),
    ("mq_mixed.cu", []),
    ("mq_tandem.cu", ["--fmad=false"]),
    ("mq_tandem_mixed.cu", []),
    ("mq_solve.cu", ["--fmad=false"]),
    ("mq_noalloc.cu", []),
    ("mq_probe.cu", []),
]
CXX_UNITS = ["mq_grid.cpp", "mq_engine.cpp", "mq_cube.cpp", "mq_fit.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmqgb.so")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(obj: Path, src: Path) -> bool:
    if not obj.exists():
        return True
    deps = [src] + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    t = obj.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps if d.exists())


def build(verbose: bool = False, force: bool = False, check: bool = False) -> Path:
    """Compile the library; ``check=True`` makes the bounds-checked debug build
    ``libmqgb_check.so`` (-DMQ_CHECK, its own object directory) instead."""
    nvcc = _nvcc()
    bdir, lib = (CHECK_BUILD, CHECK_LIB) if check else (BUILD, LIB)
    defs = ["-DMQ_CHECK"] if check else []
    bdir.mkdir(exist_ok=True)
    jobs = []
    objs = []
    for name, extra in CUDA_UNITS:
        src = CSRC / name
        if not src.exists():
            continue
        obj = bdir / (name + ".o")
        objs.append(obj)
        if force or _stale(obj, src):
            jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                         "-Xptxas", "-warn-spills", *defs, *extra, f"-I{INCLUDE}", f"-I{CSRC}", "-c", str(src), "-o", str(obj)])
    for name in CXX_UNITS:
        src = CSRC / name
        if not src.exists():
            continue
        obj = bdir / (name + ".o")
        objs.append(obj)
        if force or _stale(obj, src):
            jobs.append(["g++", *CXXFLAGS, *defs, f"-I{INCLUDE}", f"-I{CSRC}", "-I/usr/local/cuda/include", "-c", str(src),
                         "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for cmd, fut in [(c, ex.submit(_run, c)) for c in jobs]:
            if verbose:
                print(" ".join(cmd), file=sys.stderr)
            fut.result()
    if jobs or not lib.exists():
        tmp = lib.with_suffix(".so.tmp")
        _run([nvcc, *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *map(str, objs), "-lpthread", "-ldl", "-lrt"])
        os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv, check="--check" in sys.argv))
