"""Persisted autotuning: results of grus_autotune keyed by graph signature,
and of grus_batch_autotune / grus_server_autotune keyed by the signature of
the graph set and of the query mix.

The signature (algorithm, n, m, flags, max-degree vertex and degree) names a
graph well enough that a tuning measured once is reused on later runs of the
same graph; a query mix is named by a hash of its (graph, algorithm, source)
list.  The cache is a small JSON file.
"""
from __future__ import annotations

import hashlib
import json
import os
from pathlib import Path

import grus_framework_gb300 as grus

DEFAULT_PATH = Path(os.environ.get("GRUS_TUNING_CACHE",
                                   Path.home() / ".cache" / "grus_gb300" / "tuning.json"))


def signature(g: "grus.Graph", algo: int) -> str:
    inf = g.info()
    return f"{algo}:{inf.n}:{inf.m}:{inf.flags}:{inf.max_degree_vertex}:{inf.max_degree}"


def load(path: Path = DEFAULT_PATH) -> dict:
    try:
        return json.loads(Path(path).read_text())
    except (OSError, ValueError):
        return {}


def _store(path: Path, key: str, entry: dict) -> bool:
    """Adds one entry to the cache file; an unwritable cache only costs the
    reuse (returns False), never the tuning just measured."""
    cache = load(path)
    cache[key] = entry
    path = Path(path)
    try:
        path.parent.mkdir(parents=True, exist_ok=True)
        tmp = path.with_suffix(".tmp")
        tmp.write_text(json.dumps(cache, indent=1))
        tmp.replace(path)
    except OSError:
        return False
    return True


def load_or_tune(g: "grus.Graph", algo: int = grus.ALGO_BFS, src=None, path: Path = DEFAULT_PATH,
                 reps: int = 2) -> dict:
    """Applies the cached tuning for `g`, or autotunes and caches it."""
    cache = load(path)
    key = signature(g, algo)
    if key in cache:
        g.set_tuning(**cache[key]["tuning"])
        return cache[key]
    tuning, ms = grus.autotune(g, algo, src, reps)
    entry = {"tuning": tuning, "device_ms": ms}
    _store(path, key, entry)
    return entry


def mix_signature(kind: str, graph_sigs, queries) -> str:
    """Key of a tuning for a graph set (signature() of each graph, algorithm
    field aside) and a query mix ((graph, algo, src) tuples)."""
    gsig = ",".join(s.split(":", 1)[1] for s in graph_sigs)
    qsig = hashlib.sha1(repr([tuple(int(x) for x in q) for q in queries]).encode()).hexdigest()[:16]
    return f"{kind}:{hashlib.sha1(gsig.encode()).hexdigest()[:16]}:{len(queries)}:{qsig}"


def load_or_tune_batch(graphs, queries, path: Path = DEFAULT_PATH, reps: int = 2) -> dict:
    """The cached batch-engine tuning for this graph set and query mix, or a
    fresh grus_batch_autotune of it (then cached).  Returns {"config":
    Batch keyword arguments, "device_ms": ..., "cached": bool}."""
    key = mix_signature("batch", [signature(g, 0) for g in graphs], queries)
    cache = load(path)
    if key in cache:
        return dict(cache[key], cached=True)
    cfg, ms = grus.batch_autotune(graphs, queries, reps)
    entry = {"config": cfg, "device_ms": ms}
    _store(path, key, entry)
    return dict(entry, cached=False)


def load_or_tune_server(graphs, queries, path: Path = DEFAULT_PATH, reps: int = 1) -> dict:
    """As load_or_tune_batch for the query server (grus_server_autotune);
    returns {"config": Server keyword arguments, "qps": ..., "cached": bool}."""
    key = mix_signature("server", [signature(g, 0) for g in graphs], queries)
    cache = load(path)
    if key in cache:
        return dict(cache[key], cached=True)
    cfg, qps = grus.server_autotune(graphs, queries, reps)
    entry = {"config": cfg, "qps": qps}
    _store(path, key, entry)
    return dict(entry, cached=False)
