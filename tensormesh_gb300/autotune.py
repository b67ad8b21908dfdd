"""The project's autotuner: time launch-shape candidates with CUDA events on
the real inputs, keep the fastest, and cache the choice as JSON per
(device, kernel, problem signature).

Cache file: ``$TM_AUTOTUNE_CACHE`` or ~/.cache/tensormesh_gb300/autotune.json.
"""
from __future__ import annotations

import json
import os
from typing import Callable, Dict, Iterable, List, Tuple

import torch

_CACHE_ENV = "TM_AUTOTUNE_CACHE"


def cache_path() -> str:
    p = os.environ.get(_CACHE_ENV)
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "tensormesh_gb300", "autotune.json")


def load_cache() -> dict:
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except Exception:
        return {}


def store_cache(key: str, value: dict):
    data = load_cache()
    data[key] = value
    path = cache_path()
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + f".{os.getpid()}"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def time_ms(fn: Callable[[], None], reps: int = 3, warm: int = 1) -> float:
    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        fn()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def pick(candidates: Iterable, run: Callable[[object], None], reps: int = 3) -> Tuple[object, List[Dict]]:
    """Time ``run(c)`` for every candidate; returns (best, table)."""
    table = []
    for c in candidates:
        try:
            ms = time_ms(lambda: run(c), reps=reps)
        except Exception as exc:  # a candidate that does not fit (shared memory) is skipped
            table.append({"candidate": c, "error": str(exc)[:120]})
            continue
        table.append({"candidate": c, "ms": ms})
    ok = [t for t in table if "ms" in t]
    if not ok:
        raise RuntimeError("autotune: no candidate ran")
    best = min(ok, key=lambda t: t["ms"])
    return best["candidate"], table
