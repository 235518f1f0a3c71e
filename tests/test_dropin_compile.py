"""CPU: the reference's samples compile and link UNCHANGED against the mgg
drop-in headers (grus_framework_gb300/mgg) and libgrus.so -- the drop-in
contract of the template/operator API (include/*.cuh, samples/*).  The samples are
read from the Grus source tree where it is present (build container); the
test is skipped elsewhere.  The repository's own drop-in test program is
compiled too."""
import concurrent.futures as cf
import os
from pathlib import Path

import pytest

import sys
sys.path.insert(0, str(Path(__file__).resolve().parent / "dropin"))
import build_apps  # noqa: E402

from oracle.build import REF_SRC as REF  # noqa: E402  (GRUS_REFERENCE: the Grus source tree)
SAMPLES = ["bfs", "sssp", "cc", "pagerank", "bfs_2s"]


@pytest.fixture(scope="module")
def lib_built():
    from grus_framework_gb300 import build as b
    return b.build()


@pytest.mark.skipif(not (REF / "samples").exists(), reason="Grus source tree not present")
def test_reference_samples_compile_unchanged(lib_built):
    def one(app):
        srcs = sorted((REF / "samples" / app).glob("*.cu"))
        return build_apps.build_program(srcs, f"ref_{app}")
    with cf.ThreadPoolExecutor(len(SAMPLES)) as ex:
        exes = list(ex.map(one, SAMPLES))
    for e in exes:
        assert e.exists() and os.access(e, os.X_OK)


def test_dropin_test_program_compiles(lib_built):
    exe = build_apps.build_apps()
    assert exe.exists()
