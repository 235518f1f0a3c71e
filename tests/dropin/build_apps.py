"""Builds tests/dropin/apps.cu (the mgg drop-in test program) against the
drop-in headers and libgrus.so; used by the drop-in tests."""
import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
MGG = ROOT / "grus_framework_gb300" / "mgg"
LIBDIR = ROOT / "grus_framework_gb300" / "_lib"
OUT = ROOT / "tests" / "dropin" / "_build"

NVCC_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O2",
              "-I", str(MGG), "-I", str(ROOT / "include")]


def nvcc():
    for c in ("/usr/local/cuda/bin/nvcc", "nvcc"):
        if Path(c).exists() or c == "nvcc":
            return c


def link_args():
    return ["-L", str(LIBDIR), "-lgrus", "-Xlinker", f"-rpath={LIBDIR}"]


def build_program(sources, out_name):
    OUT.mkdir(exist_ok=True)
    exe = OUT / out_name
    deps = [Path(s) for s in sources] + list(MGG.glob("*.cuh")) + [MGG / "worklist.cu"]
    if exe.exists() and all(d.stat().st_mtime < exe.stat().st_mtime for d in deps):
        return exe
    cmd = [nvcc(), *NVCC_FLAGS, *map(str, sources), str(MGG / "worklist.cu"), *link_args(), "-o", str(exe)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr)
    return exe


def build_apps():
    return build_program([ROOT / "tests" / "dropin" / "apps.cu"], "apps")
