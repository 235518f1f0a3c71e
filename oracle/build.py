"""Build recipe for the CPU oracle (test infrastructure only).

  liboracle  : g++ -O3 -fopenmp on grus_oracle.cpp -> oracle/_build/libgrus_oracle.so
  ref pin    : when the Grus sources are present (build container only),
               oracle/ref_pin.cu is compiled with nvcc against the reference's
               own include/ directory into oracle/_ref/ref_pin.  It runs the
               reference's host code (graph_loader::ReadGraphGR and csr_tocsc)
               on the CPU; tests/golden/make_golden.py uses it to pin the
               oracle's .gr reader and transpose.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"
LIB = BUILD / "libgrus_oracle.so"
# The Grus source tree, read in place (never copied): GRUS_REFERENCE, else the
# build container's checkout.  Absent on the GPU machine, where the pin is skipped.
REF_SRC = Path(os.environ.get("GRUS_REFERENCE", "/root/reference"))


def _run(cmd):
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("command failed:\n" + " ".join(map(str, cmd)) + "\n" + res.stdout + res.stderr)


def build_oracle() -> Path:
    BUILD.mkdir(exist_ok=True)
    src = HERE / "grus_oracle.cpp"
    hdr = HERE / "grus_oracle.h"
    if not LIB.exists() or LIB.stat().st_mtime < max(src.stat().st_mtime, hdr.stat().st_mtime):
        cxx = os.environ.get("CXX", "g++")
        _run([cxx, "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", str(src), "-o", str(LIB)])
    return LIB


def build_ref_pin() -> Path | None:
    """Compile the reference-pinning driver if the reference tree is present."""
    inc = REF_SRC / "include"
    if not (inc / "graph_loader.cuh").exists():
        return None
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    REF_OUT.mkdir(exist_ok=True)
    out = REF_OUT / "ref_pin"
    drv = HERE / "ref_pin.cu"
    if out.exists() and out.stat().st_mtime > drv.stat().st_mtime:
        return out
    gflags_dir = ROOT / "grus_framework_gb300" / "mgg"
    _run([nvcc, "-std=c++17", "-O1", "-include", str(HERE / "ref_pin_shim.h"),
          "-I", str(inc), "-I", str(gflags_dir), str(drv), "-o", str(out)])
    return out


def build() -> Path:
    lib = build_oracle()
    try:
        build_ref_pin()
    except Exception as exc:  # the pin is optional; the oracle is not
        print(f"[oracle] reference pin not built: {exc}")
    return lib


if __name__ == "__main__":
    print(build())
