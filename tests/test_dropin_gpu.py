"""GPU: the mgg drop-in template API (graph_loader, Frontier<BDF|BITMAP|WL|
BDF_AUTO>, kernel<>, kernel_pull<>, user updater/generator/pull_selector
functors, CSR2CSC, SaveResults) driven by tests/dropin/apps.cu, checked
against the oracle: BFS depths, SSSP distances and CC labels bit-exact in
push and pull modes and every push frontier kind; the reference's delta-push
PageRank within a stated tolerance of its sequential restatement."""
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

sys.path.insert(0, str(Path(__file__).resolve().parent / "dropin"))
import build_apps  # noqa: E402

from conftest import GOLDEN

pytestmark = pytest.mark.gpu
INF = 4294967294


@pytest.fixture(scope="module")
def apps(grus):
    return build_apps.build_apps()


def run(apps, tmp_path, gr, algo, src=0, extra=()):
    out = tmp_path / f"{algo}_{src}_{'_'.join(extra).replace('-', '')}.txt"
    res = subprocess.run([str(apps), f"--algo={algo}", f"--input={gr}", f"--src={src}",
                          f"--output={out}", *extra], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    vals = [ln.split()[1] for ln in out.read_text().splitlines()]
    return vals


@pytest.fixture(scope="module")
def rmat_gr(tmp_path_factory, oracle_mod):
    d = tmp_path_factory.mktemp("gr")
    g = oracle_mod.rmat(14, 16, 21, oracle_mod.GEN_SYMMETRIC | oracle_mod.GEN_RELABEL | oracle_mod.GEN_WEIGHTED)
    p = d / "rmat14.gr"
    oracle_mod.write_gr(p, g)
    gd = oracle_mod.rmat(12, 8, 5, oracle_mod.GEN_RELABEL | oracle_mod.GEN_WEIGHTED)
    pd = d / "rmat12_dir.gr"
    oracle_mod.write_gr(pd, gd)
    return {"sym": (p, g), "dir": (pd, gd)}


@pytest.mark.parametrize("frontier", ["bdf", "wl", "auto", "bitmap"])
@pytest.mark.parametrize("kind", ["sym", "dir"])
def test_dropin_bfs_push(apps, tmp_path, rmat_gr, oracle_mod, frontier, kind):
    p, g = rmat_gr[kind]
    src = oracle_mod.max_degree_vertex(g)
    got = np.array(run(apps, tmp_path, p, "bfs", src, (f"--frontier={frontier}",)), np.uint64)
    assert np.array_equal(got, oracle_mod.bfs(g, src).astype(np.uint64))


@pytest.mark.parametrize("kind", ["sym", "dir"])
def test_dropin_bfs_pull(apps, tmp_path, rmat_gr, oracle_mod, kind):
    p, g = rmat_gr[kind]
    src = oracle_mod.max_degree_vertex(g)
    got = np.array(run(apps, tmp_path, p, "bfs", src, ("--pull",)), np.uint64)
    assert np.array_equal(got, oracle_mod.bfs(g, src).astype(np.uint64))


@pytest.mark.parametrize("mode", [(), ("--pull",), ("--frontier=wl",)])
def test_dropin_sssp(apps, tmp_path, rmat_gr, oracle_mod, mode):
    for kind in ("sym", "dir"):
        p, g = rmat_gr[kind]
        src = oracle_mod.max_degree_vertex(g)
        got = np.array(run(apps, tmp_path, p, "sssp", src, mode), np.uint64)
        assert np.array_equal(got, oracle_mod.sssp(g, src).astype(np.uint64))


@pytest.mark.parametrize("mode", [(), ("--pull",), ("--frontier=auto",)])
def test_dropin_cc(apps, tmp_path, rmat_gr, oracle_mod, mode):
    p, g = rmat_gr["sym"]
    got = np.array(run(apps, tmp_path, p, "cc", 0, mode), np.uint64)
    assert np.array_equal(got, oracle_mod.cc(g).astype(np.uint64))


def test_dropin_golden_fixtures(apps, tmp_path):
    import json
    ans = json.loads((GOLDEN / "known_answers.json").read_text())
    for name, a in ans.items():
        for s, exp in a["bfs"].items():
            got = [int(x) for x in run(apps, tmp_path, GOLDEN / f"{name}.gr", "bfs", int(s))]
            assert got == exp, name
        for s, exp in a["sssp"].items():
            got = [int(x) for x in run(apps, tmp_path, GOLDEN / f"{name}.gr", "sssp", int(s))]
            assert got == exp, name


def test_dropin_delta_pagerank(apps, tmp_path, rmat_gr, oracle_mod):
    """Delta-push PR with float atomics: order-dependent, so compared with the
    sequential restatement within 1% relative (max) and 1e-3 mean."""
    p, g = rmat_gr["sym"]
    got = np.array(run(apps, tmp_path, p, "pr", 0), np.float64)
    ref, _ = oracle_mod.delta_pagerank(g)
    rel = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-12)
    assert rel.mean() < 1e-3 and rel.max() < 1e-2, (rel.mean(), rel.max())


# The two-stage active-subgraph BFS (the reference's bfs_2s: Frontier_2S<BDF>,
# Subgraph<NORMAL>, kernel_2s): every level gathers the frontier's rows into a
# compact subgraph on the device and expands over it.  Depths bit-exact
# against the oracle, with the CSR in HBM and in managed memory under half the
# CSR bytes as device budget.
MEM_MODES = [(), ("--mem=managed", "--budget=0.5")]


@pytest.mark.parametrize("mem", MEM_MODES)
@pytest.mark.parametrize("kind", ["sym", "dir"])
def test_dropin_bfs_2s(apps, tmp_path, rmat_gr, oracle_mod, kind, mem):
    p, g = rmat_gr[kind]
    deg = np.diff(g.offs.astype(np.int64))
    for src in (oracle_mod.max_degree_vertex(g), int(np.flatnonzero(deg > 0)[7])):
        got = np.array(run(apps, tmp_path, p, "bfs2s", src, mem), np.uint64)
        assert np.array_equal(got, oracle_mod.bfs(g, src).astype(np.uint64)), src


@pytest.mark.parametrize("mem", MEM_MODES)
def test_dropin_bfs_2s_golden_fixtures(apps, tmp_path, mem):
    import json
    ans = json.loads((GOLDEN / "known_answers.json").read_text())
    for name, a in ans.items():
        for s, exp in a["bfs"].items():
            got = [int(x) for x in run(apps, tmp_path, GOLDEN / f"{name}.gr", "bfs2s", int(s), mem)]
            assert got == exp, name
