"""Persisted autotuning: results of grus_autotune keyed by graph signature.

The signature (algorithm, n, m, flags, max-degree vertex and degree) names a
graph well enough that a tuning measured once is reused on later runs of the
same graph; the cache is a small JSON file.
"""
from __future__ import annotations

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


def load_or_tune(g: "grus.Graph", algo: int = grus.ALGO_BFS, src=None, path: Path = DEFAULT_PATH,
                 reps: int = 2) -> dict:
    """Applies the cached tuning for `g`, or autotunes and caches it."""
    cache = load(path)
    key = signature(g, algo)
    if key in cache:
        g.set_tuning(**cache[key]["tuning"])
        return cache[key]
    tuning, ms = grus.autotune(g, algo, src, reps)
    cache[key] = {"tuning": tuning, "device_ms": ms}
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    tmp = path.with_suffix(".tmp")
    tmp.write_text(json.dumps(cache, indent=1))
    tmp.replace(path)
    return cache[key]
