"""Generate the committed golden fixtures in tests/golden/ (run in the build
container, where the Grus sources are present).

  *.gr                 hand-built Galois v1 graphs (path, star, two components
                       + isolated vertex, duplicate edges + self-loop, odd-m
                       weighted file exercising the padding rule, edgeless)
  known_answers.json   hand-computed BFS / SSSP / CC answers for them, each
                       asserted here against networkx before it is written
  ref_pin_<name>.txt   the reference's own graph_loader::ReadGraphGR and
                       csr_tocsc run on each file (oracle/_ref/ref_pin); pins
                       the oracle's .gr reader and transpose
  rmat_spec.json       RMAT edges / relabelling / weights from a pure-Python
                       restatement of the generator specification (independent
                       of the C++ oracle and the CUDA generator)

Usage: python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import struct
import subprocess
import sys
from pathlib import Path

import networkx as nx

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))
INF = 4294967294
M64 = (1 << 64) - 1


def write_gr(path: Path, n, edges, weights=None):
    """edges: list of (u, v) already in CSR order (sorted by u)."""
    offs = [0] * (n + 1)
    for u, _ in edges:
        offs[u + 1] += 1
    for i in range(n):
        offs[i + 1] += offs[i]
    m = len(edges)
    with open(path, "wb") as f:
        f.write(struct.pack("<4Q", 1, 4 if weights else 0, n, m))
        f.write(struct.pack(f"<{n}Q", *offs[1:]))
        f.write(struct.pack(f"<{m}I", *[v for _, v in edges]))
        if weights:
            if m % 2:
                f.write(struct.pack("<I", 0))
            f.write(struct.pack(f"<{m}I", *weights))


def nx_graph(n, edges, weights=None):
    G = nx.MultiDiGraph()
    G.add_nodes_from(range(n))
    for i, (u, v) in enumerate(edges):
        G.add_edge(u, v, weight=(weights[i] if weights else 1))
    return G


def nx_bfs(G, n, s):
    d = [INF] * n
    for k, v in nx.single_source_shortest_path_length(G, s).items():
        d[k] = v
    return d


def nx_sssp(G, n, s):
    d = [INF] * n
    for k, v in nx.single_source_dijkstra_path_length(G, s).items():
        d[k] = int(v)
    return d


def nx_cc(G, n):
    lab = [0] * n
    for comp in nx.connected_components(nx.Graph(G.to_undirected())):
        mn = min(comp)
        for x in comp:
            lab[x] = mn
    return lab


def sym(pairs):
    out = set()
    for u, v in pairs:
        out.add((u, v))
        out.add((v, u))
    return sorted(out)


# ---- pure-Python restatement of the generator specification ---------------
def mix64(x):
    x = (x + 0x9E3779B97F4A7C15) & M64
    x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & M64
    x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & M64
    return x ^ (x >> 31)


def rmat_edge(scale, seed, i):
    base = mix64(mix64(seed) ^ i)
    u = v = 0
    r = 0
    for lv in range(scale):
        if lv % 4 == 0:
            r = mix64((base + lv // 4) & M64)
        x = (r >> ((lv % 4) * 16)) & 0xFFFF
        if x < 37356:
            ub, vb = 0, 0
        elif x < 49807:
            ub, vb = 0, 1
        elif x < 62259:
            ub, vb = 1, 0
        else:
            ub, vb = 1, 1
        u = (u << 1) | ub
        v = (v << 1) | vb
    return u, v


def relabel(scale, seed, x):
    mask = (1 << scale) - 1
    k0 = mix64(seed ^ 0x5851F42D4C957F2D)
    sh = (scale + 1) // 2
    for rnd in range(3):
        kr = mix64((k0 + rnd) & M64)
        x = (x * ((kr & mask) | 1) + ((kr >> 32) & mask)) & mask
        x ^= x >> sh
    return x


def edge_weight(seed, u, v):
    lo, hi = min(u, v), max(u, v)
    return mix64(mix64(seed ^ 0x2545F4914F6CDD1D) ^ ((lo << 32) | hi)) % 255 + 1


def main():
    cases = {}

    # path 0-1-2-3-4 (symmetric)
    e = sym([(0, 1), (1, 2), (2, 3), (3, 4)])
    cases["path5"] = dict(n=5, edges=e, weights=None,
                          bfs={0: [0, 1, 2, 3, 4], 2: [2, 1, 0, 1, 2]},
                          cc=[0, 0, 0, 0, 0])
    # star: centre 0, leaves 1..6
    e = sym([(0, k) for k in range(1, 7)])
    cases["star7"] = dict(n=7, edges=e, weights=None,
                          bfs={0: [0, 1, 1, 1, 1, 1, 1], 3: [1, 2, 2, 0, 2, 2, 2]},
                          cc=[0] * 7)
    # triangle {0,1,2}, edge {3,4}, isolated 5
    e = sym([(0, 1), (1, 2), (0, 2), (3, 4)])
    cases["two_comp"] = dict(n=6, edges=e, weights=None,
                             bfs={0: [0, 1, 1, INF, INF, INF], 5: [INF] * 5 + [0],
                                  4: [INF, INF, INF, 1, 0, INF]},
                             cc=[0, 0, 0, 3, 3, 5])
    # directed, duplicate edge 0->1 twice, self-loop 1->1
    e = [(0, 1), (0, 1), (1, 1), (1, 2), (2, 0)]
    cases["dup_self"] = dict(n=3, edges=e, weights=None,
                             bfs={0: [0, 1, 2], 2: [1, 2, 0]}, cc=None)
    # directed weighted, odd m (padding before the weights)
    e = [(0, 1), (0, 2), (1, 3), (2, 1), (3, 0)]
    w = [4, 1, 5, 2, 1]
    cases["odd_weighted"] = dict(n=4, edges=e, weights=w,
                                 bfs={0: [0, 1, 1, 2]},
                                 sssp={0: [0, 3, 1, 8], 3: [1, 4, 2, 0]}, cc=None)
    # no edges at all
    cases["edgeless"] = dict(n=4, edges=[], weights=None,
                             bfs={2: [INF, INF, 0, INF]}, cc=[0, 1, 2, 3])

    answers = {}
    for name, c in cases.items():
        n, edges, weights = c["n"], c["edges"], c["weights"]
        write_gr(HERE / f"{name}.gr", n, edges, weights)
        G = nx_graph(n, edges, weights)
        for s, exp in c["bfs"].items():
            assert nx_bfs(G, n, s) == exp, (name, s)
        for s, exp in (c.get("sssp") or {}).items():
            assert nx_sssp(G, n, s) == exp, (name, s)
        if c["cc"] is not None:
            assert nx_cc(G, n) == c["cc"], name
        answers[name] = {
            "n": n, "m": len(edges),
            "bfs": {str(k): v for k, v in c["bfs"].items()},
            "sssp": {str(k): v for k, v in (c.get("sssp") or {}).items()},
            "cc": c["cc"],
        }
    (HERE / "known_answers.json").write_text(json.dumps(answers, indent=1))

    # reference pins
    from oracle import build as ob
    pin = ob.build_ref_pin()
    if pin is None:
        print("reference sources absent: ref_pin_*.txt not regenerated")
    else:
        for name in cases:
            gr = subprocess.run([str(pin), "gr", str(HERE / f"{name}.gr"), "1"],
                                capture_output=True, text=True, check=True).stdout
            csc = subprocess.run([str(pin), "csc", str(HERE / f"{name}.gr"), "0"],
                                 capture_output=True, text=True, check=True).stdout
            (HERE / f"ref_pin_{name}.txt").write_text("# gr\n" + gr + "# csc\n" + csc)

    # generator specification vectors
    spec = {"rmat_edges": [], "relabel": [], "weights": []}
    for scale, seed in ((8, 3), (16, 1), (24, 3)):
        for i in (0, 1, 2, 1000, 123457):
            u, v = rmat_edge(scale, seed, i)
            spec["rmat_edges"].append([scale, seed, i, u, v])
    for scale, seed in ((8, 3), (12, 1), (26, 9)):
        for x in (0, 1, 77, (1 << scale) - 1):
            spec["relabel"].append([scale, seed, x, relabel(scale, seed, x)])
        perm = sorted(relabel(8, seed, x) for x in range(256))
        assert perm == list(range(256)), "relabel must be a bijection"
    for seed, u, v in ((2, 0, 1), (2, 1, 0), (5, 123, 77777), (3, 4095, 4096)):
        spec["weights"].append([seed, u, v, edge_weight(seed, u, v)])
    (HERE / "rmat_spec.json").write_text(json.dumps(spec, indent=1))
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
