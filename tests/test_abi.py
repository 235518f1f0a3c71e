"""CPU: the C-ABI library loads and exports every entry point include/*.h
declares, and the status strings are stable.  No compute calls (no GPU)."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        for m in re.finditer(r"GRUS_API\s+[\w\s\*]+?\b(grus_\w+)\s*\(", h.read_text()):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from grus_framework_gb300 import build as b
    path = b.build()
    return ctypes.CDLL(str(path))


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "grus_bfs" in names and "grus_graph_load_gr" in names
    assert len(names) >= 15


@pytest.mark.parametrize("name", declared_symbols())
def test_symbol_exported(lib, name):
    assert hasattr(lib, name), f"{name} declared in include/ but not exported"


def test_no_unexpected_exports(lib):
    import subprocess
    out = subprocess.run(["nm", "-D", "--defined-only", str(ROOT / "grus_framework_gb300" / "_lib" / "libgrus.so")],
                         capture_output=True, text=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln and ln.split()[-1].startswith("grus_")}
    assert exported == set(declared_symbols())


def test_status_strings(lib):
    lib.grus_strerror.restype = ctypes.c_char_p
    assert lib.grus_strerror(0) == b"ok"
    assert lib.grus_strerror(-22) == b"invalid argument"
    assert lib.grus_strerror(-110) == b"device wait timed out"
    lib.grus_version.restype = ctypes.c_char_p
    assert b"sm_103a" in lib.grus_version()


def test_package_import_fails_loudly_without_library(tmp_path, monkeypatch):
    """No CPU fallback: a missing libgrus.so is an import error."""
    import importlib.util
    import shutil
    pkg = tmp_path / "grus_framework_gb300"
    shutil.copytree(ROOT / "grus_framework_gb300", pkg, ignore=shutil.ignore_patterns("_lib", "_build", "__pycache__"))
    spec = importlib.util.spec_from_file_location("grus_copy", pkg / "__init__.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    with pytest.raises(ImportError):
        mod.version()
    with pytest.raises(ImportError):
        mod.Graph.rmat(8)


STRUCTS = {"Stats": "grus_stats", "GraphInfo": "grus_graph_info", "LevelTrace": "grus_level_trace",
           "Query": "grus_query", "BatchConfig": "grus_batch_config", "ServerConfig": "grus_server_config",
           "Completion": "grus_completion", "ServerStats": "grus_server_stats",
           "Telemetry": "grus_telemetry", "Tuning": "grus_tuning"}


def test_ctypes_structs_match_header(tmp_path):
    """Every ctypes mirror in the package has the C struct's size and each of
    its fields the C field's offset and size, as gcc lays out include/grus.h."""
    import subprocess
    import grus_framework_gb300 as pkg
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "grus.h"', "int main(void) {"]
    expect = []
    for py, c in STRUCTS.items():
        cls = getattr(pkg, py)
        lines.append(f'  printf("%zu\\n", sizeof({c}));')
        expect.append(ctypes.sizeof(cls))
        for name, _ in cls._fields_:
            f = getattr(cls, name)
            lines.append(f'  printf("%zu %zu\\n", offsetof({c}, {name}), sizeof((({c} *)0)->{name}));')
            expect.append(f"{f.offset} {f.size}")
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    got = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")[:-1]
    assert got == [str(e) for e in expect]

