"""Build libgrus.so (the sm_103a CUDA library behind include/grus.h).

Plain nvcc invocations, one translation unit per process, compiled in
parallel; no cmake, no torch extension machinery.  The library links the CUDA
runtime statically so it never clashes with another runtime copy loaded in
the same process (e.g. PyTorch's).  Outputs go to grus_framework_gb300/_lib/.
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
OUT = PKG / "_lib"
OBJ = PKG / "_build"
LIB = OUT / "libgrus.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
    "-I", str(ROOT / "include"), "-I", str(CSRC),
]

SOURCES = [
    "graph.cu",
    "graph_gen.cu",
    "bfs.cu",
    "sssp.cu",
    "cc.cu",
    "pagerank.cu",
    "msbfs.cu",
    "msssp.cu",
    "batch.cu",
    "serve.cu",
    "tune.cu",
    "tools.cu",
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("command failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr)


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, extra_flags: list[str] | None = None) -> Path:
    """Compile every CUDA source for sm_103a and link libgrus.so."""
    OUT.mkdir(exist_ok=True)
    OBJ.mkdir(exist_ok=True)
    cc = nvcc()
    headers = list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h"))
    jobs = []
    objs = []
    for src in SOURCES:
        s = CSRC / src
        o = OBJ / (s.stem + ".o")
        objs.append(o)
        if _stale(o, [s] + headers):
            cmd = [cc, *ARCH, *NVCC_FLAGS, *(extra_flags or []), "-c", str(s), "-o", str(o)]
            jobs.append(cmd)
    if jobs:
        workers = min(len(jobs), os.cpu_count() or 4)
        with cf.ThreadPoolExecutor(workers) as ex:
            for cmd in jobs:
                if verbose:
                    print(" ".join(cmd), file=sys.stderr)
            list(ex.map(_run, jobs))
    if _stale(LIB, objs):
        _run([cc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-cudart", "static", "-ldl"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
