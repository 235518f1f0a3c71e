"""GPU: device generator and BFS against the CPU oracle, through the C ABI.

BFS depths are integer results and must match bit for bit (the fixpoint of
samples/bfs/bfs.cu:18-87), on the golden fixtures, on RMAT-16 (edge factor
16, seed 1, symmetrised), on directed and high-diameter graphs, and -- through the
size-independent checks that the serial oracle can afford -- on RMAT-22.
"""
import json

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu
INF = 4294967294
ANSWERS = json.loads((GOLDEN / "known_answers.json").read_text())


def host_csr(g):
    offs, cols, wts = g.copy_csr()
    import oracle
    return oracle.CSR(offs, cols, wts)


@pytest.mark.parametrize("scale,ef,seed,flags", [
    (8, 4, 3, 0), (10, 16, 1, 1 | 4), (12, 8, 2, 1 | 2 | 4), (11, 16, 3, 2 | 4), (14, 16, 1, 1 | 4),
])
def test_rmat_generator_matches_oracle(grus, oracle_mod, scale, ef, seed, flags):
    g = grus.Graph.rmat(scale, ef, seed, symmetric=bool(flags & 1), weighted=bool(flags & 2),
                        relabel=bool(flags & 4))
    ref = oracle_mod.rmat(scale, ef, seed, flags)
    offs, cols, wts = g.copy_csr()
    assert np.array_equal(offs, ref.offs)
    assert np.array_equal(cols, ref.cols)
    if flags & 2:
        assert np.array_equal(wts, ref.wts)
    assert g.max_degree_vertex == oracle_mod.max_degree_vertex(ref)
    g.free()


def test_grid_generator_matches_oracle(grus, oracle_mod):
    g = grus.Graph.grid2d(37, 53, seed=5, weighted=True)
    ref = oracle_mod.grid(37, 53, 5, 2)
    offs, cols, wts = g.copy_csr()
    assert np.array_equal(offs, ref.offs) and np.array_equal(cols, ref.cols)
    assert np.array_equal(wts, ref.wts)


@pytest.mark.parametrize("name", sorted(ANSWERS))
def test_bfs_golden_fixtures(grus, name):
    a = ANSWERS[name]
    g = grus.Graph.load_gr(GOLDEN / f"{name}.gr")
    for s, exp in a["bfs"].items():
        d, st = grus.bfs(g, int(s), stats=True)
        assert d.tolist() == exp
        assert st["vertices_reached"] == sum(x != INF for x in exp)
    g.free()


def _check_bfs(grus, oracle_mod, g, srcs):
    h = host_csr(g)
    for s in srcs:
        d, st = grus.bfs(g, int(s), stats=True)
        ref = oracle_mod.bfs(h, int(s))
        assert np.array_equal(d, ref), f"src {s}: {np.count_nonzero(d != ref)} mismatches"
        assert st["vertices_reached"] == int(np.count_nonzero(ref != INF))
        assert st["edges_reached"] == oracle_mod.reached_edges(h, ref)
        reached = ref[ref != INF]
        assert st["levels"] == int(reached.max()) + 1
    return h


def test_bfs_rmat16(grus, oracle_mod):
    """RMAT scale 16, ef 16, seed 1, symmetrised, source = max-degree vertex."""
    g = grus.Graph.rmat(16, 16, 1, symmetric=True)
    rng = np.random.default_rng(0)
    _check_bfs(grus, oracle_mod, g, [g.max_degree_vertex, *rng.integers(0, g.n, 4)])


@pytest.mark.parametrize("alpha,beta", [(15.0, 18.0), (1e9, 18.0), (1e-6, 1e9), (2.0, 2.0)])
def test_bfs_direction_policies(grus, oracle_mod, alpha, beta):
    """Push-only, pull-heavy and frequent-switch schedules all give the same depths."""
    g = grus.Graph.rmat(15, 16, 7, symmetric=True)
    g.set_tuning(alpha=alpha, beta=beta)
    _check_bfs(grus, oracle_mod, g, [g.max_degree_vertex, 5, 12345])


@pytest.mark.parametrize("huge,bu_scan,ctas,words", [(64, 4, 1, 2), (1 << 20, 64, 2, 4), (512, 1, 0, 2),
                                                     (2048, 12, 0, 4)])
def test_bfs_bins_and_launch_shapes(grus, oracle_mod, huge, bu_scan, ctas, words):
    g = grus.Graph.rmat(14, 32, 9, symmetric=True)
    g.set_tuning(huge_degree=huge, bu_scan=bu_scan, ctas_per_sm=ctas, bu_words=words)
    _check_bfs(grus, oracle_mod, g, [g.max_degree_vertex, 77])


def test_bfs_directed_rmat(grus, oracle_mod):
    """Directed graph: push-only without a CSC, direction-optimising with one."""
    g = grus.Graph.rmat(14, 16, 3, symmetric=False)
    srcs = [g.max_degree_vertex, 0, 999]
    _check_bfs(grus, oracle_mod, g, srcs)
    g.build_csc()
    g.set_tuning(alpha=2.0, beta=1e9)  # pull as early as possible
    _check_bfs(grus, oracle_mod, g, srcs)


def test_bfs_grid_high_diameter(grus, oracle_mod):
    g = grus.Graph.grid2d(300, 200)
    _check_bfs(grus, oracle_mod, g, [201, 0, 59999])


def test_bfs_device_output_and_stream(grus, oracle_mod):
    torch = pytest.importorskip("torch")
    g = grus.Graph.rmat(13, 16, 5, symmetric=True)
    out = torch.empty(g.n, dtype=torch.int32, device="cuda")
    s = torch.cuda.Stream()
    grus.bfs(g, g.max_degree_vertex, out=out, stream=s)
    s.synchronize()
    ref = oracle_mod.bfs(host_csr(g), g.max_degree_vertex)
    assert np.array_equal(out.cpu().numpy().view(np.uint32), ref)


def test_bfs_errors(grus):
    g = grus.Graph.rmat(8, 4, 1)
    with pytest.raises(grus.GrusError) as e:
        grus.bfs(g, g.n)
    assert e.value.status == grus.EINVAL
    with pytest.raises(grus.GrusError):
        grus.Graph.load_gr(GOLDEN / "does_not_exist.gr")


@pytest.mark.slow
def test_bfs_rmat22_full_size(grus, oracle_mod):
    g = grus.Graph.rmat(22, 16, 2, symmetric=True)
    _check_bfs(grus, oracle_mod, g, [g.max_degree_vertex])


@pytest.mark.slow
def test_bfs_rmat24_full_size_headline(grus, oracle_mod):
    """The benchmarked configuration: RMAT-24, edge factor 16, seed 3,
    symmetrised and relabelled, from the first max-degree vertex (the
    direction-optimising persistent kernel; two pull levels)."""
    g = grus.Graph.rmat(24, 16, 3, symmetric=True)
    _check_bfs(grus, oracle_mod, g, [g.max_degree_vertex])
    g.free()


@pytest.mark.slow
def test_bfs_grid4096_full_size(grus, oracle_mod):
    """The 4096 x 4096 grid from vertex 4097: 8,189 levels, all but the first
    16 in the cluster tail."""
    g = grus.Graph.grid2d(4096, 4096)
    h = _check_bfs(grus, oracle_mod, g, [4097])
    d, st = grus.bfs(g, 4097, stats=True)
    assert st["levels"] == 8189 and st["kernel_launches"] == 2
    g.free()


def _broom(path_len, leaves):
    """A path 0..path_len-1, a star of `leaves` leaves on its last vertex,
    and one further vertex behind every leaf (symmetric CSR)."""
    edges = [(i, i + 1) for i in range(path_len - 1)]
    hub = path_len - 1
    for k in range(leaves):
        leaf = path_len + k
        edges.append((hub, leaf))
        edges.append((leaf, path_len + leaves + k))
    n = path_len + 2 * leaves
    both = edges + [(v, u) for u, v in edges]
    both.sort()
    offs = np.zeros(n + 1, np.uint32)
    for u, _ in both:
        offs[u + 1] += 1
    offs = np.cumsum(offs).astype(np.uint32)
    cols = np.array([v for _, v in both], np.uint32)
    return offs, cols


def test_bfs_long_tail_wide_vertex_and_spill(grus, oracle_mod):
    """A traversal past the hand-over level with a small frontier finishes in
    the tail cluster; there the edges of a vertex of degree 100,001 are dealt
    to all the threads of its owner CTA and its 100,000 neighbours overflow
    the shared-memory frontiers (16 x 4,096 entries at most) into the spill
    list.  Depths and counts equal the oracle's."""
    offs, cols = _broom(200, 100000)
    g = grus.Graph.from_csr(offs, cols, symmetric=True)
    _check_bfs(grus, oracle_mod, g, [0, 150, 199, 200 + 100000 + 5])


def test_bfs_long_tail_with_sinks(grus, oracle_mod):
    """A directed comb: a 300-vertex path whose every vertex also points at a
    sink of out-degree 0, so the frontiers the single-CTA tail takes over and
    builds hold vertices without out-edges."""
    path = 300
    offs = np.zeros(2 * path + 1, np.uint32)
    cols = []
    for i in range(path):
        nb = [path + i] + ([i + 1] if i + 1 < path else [])
        cols.extend(nb)
        offs[i + 1] = offs[i] + len(nb)
    offs[path + 1:] = offs[path]
    g = grus.Graph.from_csr(offs, np.array(cols, np.uint32))
    _check_bfs(grus, oracle_mod, g, [0, 7, path - 1, path + 3])


def test_bfs_pull_index(grus, oracle_mod):
    """The pull index (one representative in-neighbour per vertex) is built
    once per graph, on demand or ahead of the first BFS, and BFS depths with
    it are exact on symmetric and directed graphs."""
    for sym in (True, False):
        g = grus.Graph.rmat(14, 16, 11, symmetric=sym)
        if not sym:
            g.build_csc()
        ms = g.build_index()
        assert ms >= 0.0
        assert g.build_index() == ms  # built once
        offs, cols, _ = g.copy_csr()
        h = oracle_mod.CSR(offs, cols)
        deg = np.diff(offs.astype(np.int64))
        for src in (g.max_degree_vertex, int(np.flatnonzero(deg > 0)[3])):
            d, st = grus.bfs(g, src, stats=True)
            assert np.array_equal(d, oracle_mod.bfs(h, src))
        if sym:
            assert st["bottom_up_levels"] >= 1
        g.free()


@pytest.mark.parametrize("mode", [1, 2])
def test_bfs_depth_planes(grus, oracle_mod, mode):
    """Depths kept as bit planes and written out at the end (1) or stored as
    vertices are found (2), forced on graphs below the automatic threshold:
    pull-heavy and push-only schedules, a directed graph with its CSC, a grid
    whose traversal hands over to the cluster tail (the planes are written
    out at the hand-over), and long tails with a spilling hub and sinks."""
    g = grus.Graph.rmat(15, 16, 7, symmetric=True)
    for alpha, beta in ((1e9, 18.0), (1e-6, 1e9), (15.0, 18.0)):
        g.set_tuning(alpha=alpha, beta=beta, depth_planes=mode)
        _check_bfs(grus, oracle_mod, g, [g.max_degree_vertex, 5])
    g.free()
    g = grus.Graph.rmat(14, 16, 3, symmetric=False)
    g.build_csc()
    g.set_tuning(alpha=2.0, beta=1e9, depth_planes=mode)
    _check_bfs(grus, oracle_mod, g, [g.max_degree_vertex, 999])
    g.free()
    g = grus.Graph.grid2d(300, 200)
    g.set_tuning(depth_planes=mode)
    _check_bfs(grus, oracle_mod, g, [201, 59999])
    g.free()
    offs, cols = _broom(200, 100000)
    g = grus.Graph.from_csr(offs, cols, symmetric=True)
    g.set_tuning(depth_planes=mode)
    _check_bfs(grus, oracle_mod, g, [0, 199])
    g.free()


def test_bfs_depth_planes_tuning_range(grus):
    g = grus.Graph.rmat(8, 4, 1)
    for field in ("depth_planes", "tail_cluster"):
        with pytest.raises(grus.GrusError):
            g.set_tuning(**{field: 3})
        g.set_tuning(**{field: 0})
        assert g.get_tuning()[field] == 0
    g.free()


def _path(n):
    """A symmetric path 0 - 1 - ... - n-1."""
    deg = np.full(n, 2, np.int64)
    deg[0] = deg[-1] = 1
    offs = np.zeros(n + 1, np.uint32)
    offs[1:] = np.cumsum(deg)
    cols = np.empty(int(offs[-1]), np.uint32)
    cols[offs[1:-1] - 1] = np.arange(1, n, dtype=np.uint32)        # right neighbour, last slot
    cols[offs[1:-1]] = np.arange(0, n - 1, dtype=np.uint32)        # left neighbour, first slot
    return offs, cols


@pytest.mark.parametrize("n,src", [(300 * 200, None), (70001, 0)])
def test_bfs_depth_planes_deep(grus, oracle_mod, n, src):
    """Every level in the persistent kernel (no cluster tail), so the planes
    hold depths of up to 9 bits (a 300 x 200 grid) and of 17 bits (a path of
    70,001 vertices, depths up to 70,000): the closing pass's wider forms."""
    if src is None:
        g = grus.Graph.grid2d(300, 200)
        srcs = [201, 59999]
    else:
        offs, cols = _path(n)
        g = grus.Graph.from_csr(offs, cols, symmetric=True)
        srcs = [src, n // 3]
    g.set_tuning(depth_planes=1, tail_cluster=2)
    _check_bfs(grus, oracle_mod, g, srcs)
    g.free()
