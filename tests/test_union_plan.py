"""CPU: the host planning of the batch's whole-GPU SSSP lane
(grus_framework_gb300/csrc/union_plan.h, no CUDA), compiled with g++ into a
small driver: packs of at most 32 queries of one graph, round r made of every
graph's r-th pack, rounds cut greedily into launches of at most 64 graphs
whose distance rows fit the cap."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
CAP_DEFAULT = 1 << 23
DRIVER = r"""
#include <cstdio>
#include "union_plan.h"
int main() {
  size_t G = 0, Q = 0;
  unsigned long long cap = 0, maxg = 0, piece = 0;
  if (scanf("%zu %zu %llu %llu %llu", &G, &Q, &cap, &maxg, &piece) != 5) return 2;
  std::vector<uint64_t> gn(G), gm(G);
  for (size_t g = 0; g < G; ++g) {
    unsigned long long n, m;
    if (scanf("%llu %llu", &n, &m) != 2) return 2;
    gn[g] = n;
    gm[g] = m;
  }
  std::vector<int> sssp(Q);
  std::vector<uint32_t> qgraph;
  for (size_t i = 0; i < Q; ++i) {
    int qi;
    unsigned g;
    if (scanf("%d %u", &qi, &g) != 2) return 2;
    sssp[i] = qi;
    if ((size_t)qi >= qgraph.size()) qgraph.resize(qi + 1);
    qgraph[qi] = g;
  }
  const grus::UnionPlan p = grus::plan_union(sssp, qgraph, gn, gm, cap, maxg, piece);
  printf("%d %llu %llu %u\n", p.unions, (unsigned long long)p.max_v,
         (unsigned long long)p.max_m, p.max_ks);
  for (const auto &l : p.launches) {
    printf("L");
    for (const auto &pk : l) {
      printf(" %u:", pk.graph);
      for (size_t i = 0; i < pk.q.size(); ++i) printf(i ? ",%d" : "%d", pk.q[i]);
    }
    printf("\n");
  }
  return 0;
}
"""


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    d = tmp_path_factory.mktemp("plan")
    (d / "plan.cpp").write_text(DRIVER)
    exe = d / "plan"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", str(ROOT / "grus_framework_gb300" / "csrc"),
                    str(d / "plan.cpp"), "-o", str(exe)], check=True)
    return exe


def width(k):
    return 8 if k <= 8 else (16 if k <= 16 else 32)


def plan(driver, gn, gm, queries, cap=CAP_DEFAULT, maxg=64, piece=128):
    """queries: list of (query index, graph), grouped by graph."""
    lines = [f"{len(gn)} {len(queries)} {cap} {maxg} {piece}"]
    lines += [f"{n} {m}" for n, m in zip(gn, gm)]
    lines += [f"{qi} {g}" for qi, g in queries]
    out = subprocess.run([str(driver)], input="\n".join(lines) + "\n", capture_output=True,
                         text=True, check=True).stdout.splitlines()
    unions, max_v, max_m, max_ks = map(int, out[0].split())
    launches = []
    for ln in out[1:]:
        packs = []
        for tok in ln.split()[1:]:
            g, qs = tok.split(":")
            packs.append((int(g), [int(x) for x in qs.split(",")]))
        launches.append(packs)
    return (unions, max_v, max_m, max_ks), launches


def check_invariants(gn, gm, queries, head, launches, cap=CAP_DEFAULT, maxg=64, piece=128):
    qgraph = dict(queries)
    per_graph = {}
    for qi, g in queries:
        per_graph.setdefault(g, []).append(qi)
    seen = []
    rounds = []
    got = {}
    for packs in launches:
        graphs = [g for g, _ in packs]
        assert len(set(graphs)) == len(graphs) and 1 <= len(packs) <= maxg
        rs = set()
        for g, qs in packs:
            assert 1 <= len(qs) <= 32 and all(qgraph[q] == g for q in qs)
            r = len(got.get(g, [])) // 32
            assert qs == per_graph[g][32 * r: 32 * r + 32]  # the graph's r-th pack
            got.setdefault(g, []).extend(qs)
            rs.add(r)
            seen += qs
        assert len(rs) == 1
        rounds.append(rs.pop())
        if len(packs) > 1:
            v = sum(gn[g] for g in graphs)
            m = sum(gm[g] for g in graphs)
            assert v * width(max(len(qs) for _, qs in packs)) <= cap
            assert v < 0xFFFFFFF0 and v + m // piece + 1024 < 0xFFFFFFF0
    assert sorted(seen) == sorted(qi for qi, _ in queries)
    assert rounds == sorted(rounds)
    # greedy: a launch ends only where the next pack of its round cannot join
    for a, b in zip(launches, launches[1:]):
        ra, rb = rounds[launches.index(a)], rounds[launches.index(b)]
        if ra != rb:
            continue
        g, qs = b[0]
        graphs = [x for x, _ in a] + [g]
        k = max([len(q) for _, q in a] + [len(qs)])
        v = sum(gn[x] for x in graphs)
        m = sum(gm[x] for x in graphs)
        assert (len(a) >= maxg or v * width(k) > cap or v >= 0xFFFFFFF0
                or v + m // piece + 1024 >= 0xFFFFFFF0)
    unions = [p for p in launches if len(p) > 1]
    assert head[0] == len(unions)
    if unions:
        assert head[1] == max(sum(gn[g] for g, _ in p) for p in unions)
        assert head[2] == max(sum(gm[g] for g, _ in p) for p in unions)
        assert head[3] == max(width(max(len(q) for _, q in p)) for p in unions)


def test_plan_of_the_gpu_test_batch(driver):
    """The scenario of the GPU batch test: 40 + 1 + 8 + 3 + 17 SSSP queries
    on five small graphs -> one multi-graph launch of the first packs, then
    the 40-query graph's second pack alone."""
    gn = [1024, 2048, 4096, 8192, 4096, 512, 2000]
    gm = [16384, 65536, 262144, 131072, 131072, 4096, 7820]
    per = {0: 40, 1: 1, 2: 8, 5: 3, 6: 17}
    queries, qi = [], 0
    for g in sorted(per):
        for _ in range(per[g]):
            queries.append((qi, g))
            qi += 1
    head, launches = plan(driver, gn, gm, queries)
    check_invariants(gn, gm, queries, head, launches)
    assert [[(g, len(q)) for g, q in p] for p in launches] == [
        [(0, 32), (1, 1), (2, 8), (5, 3), (6, 17)], [(0, 8)]]
    assert head == (1, sum(gn[g] for g in per), sum(gm[g] for g in per), 32)


def test_plan_of_the_256_query_batch(driver):
    """256 SSSP queries over the 32 RMAT graphs of the batched benchmark
    (scales 14-20, 8 queries each, all on the whole-GPU lane): 15 launches,
    the 2^23-entry cap leaving each scale-20 graph alone."""
    import sys
    sys.path.insert(0, str(ROOT))
    import bench
    specs, _ = bench.batch_graph_specs(4)
    gn = [1 << sc for sc, _, _ in specs]
    gm = [2 * ef * (1 << sc) for sc, ef, _ in specs]
    queries = sorted(((i, i % 32) for i in range(256)), key=lambda t: t[1])
    head, launches = plan(driver, gn, gm, queries)
    check_invariants(gn, gm, queries, head, launches)
    assert len(launches) == 15
    for p in launches:
        if any(gn[g] == 1 << 20 for g, _ in p):
            assert len(p) == 1


@pytest.mark.parametrize("seed", range(12))
def test_plan_invariants_random(driver, seed):
    rng = np.random.default_rng(seed)
    G = int(rng.integers(1, 90))
    gn = [int(1 << rng.integers(4, 22)) for _ in range(G)]
    gm = [int(n * rng.integers(1, 40)) for n in gn]
    cap = int(1 << rng.integers(12, 26))
    maxg = int(rng.choice([2, 5, 64]))
    counts = rng.integers(0, 80, G) * (rng.random(G) < 0.7)
    queries, qi = [], 0
    for g in range(G):
        for _ in range(int(counts[g])):
            queries.append((qi, g))
            qi += 1
    if not queries:
        queries = [(0, 0)]
    head, launches = plan(driver, gn, gm, queries, cap=cap, maxg=maxg)
    check_invariants(gn, gm, queries, head, launches, cap=cap, maxg=maxg)
