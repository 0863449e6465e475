"""Autotuner for grouped launches.

The grouped kernel has two launch parameters: ``columns`` (right-hand-side columns a thread
accumulates; more columns share each entry load, fewer keep registers and occupancy) and
``g1_avg`` (a warp sums one row per thread while its rows average at most ``g1_avg``
entries and doubles the lanes per row for each doubling beyond).  The best pair depends on
the row-length distribution and the number of right-hand sides, so it is measured once per
(device, element type, index type, k, row-length histogram bucket) on the batch itself and
kept in a JSON cache (``$GSA_AUTOTUNE_CACHE`` or ``~/.cache/genericsparsearrays_gb300/autotune.json``).
"""
from __future__ import annotations

import json
import math
import os
from typing import Dict, Sequence, Tuple

import numpy as np
import torch

CANDIDATE_G1 = (3, 6, 12)
CANDIDATE_COLUMNS = (1, 2, 4, 8)


def cache_path() -> str:
    p = os.environ.get("GSA_AUTOTUNE_CACHE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "genericsparsearrays_gb300", "autotune.json")


def _load() -> Dict[str, dict]:
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _save(d: Dict[str, dict]) -> None:
    p = cache_path()
    try:
        os.makedirs(os.path.dirname(p), exist_ok=True)
        tmp = p + f".tmp{os.getpid()}"
        with open(tmp, "w") as f:
            json.dump(d, f, indent=1, sort_keys=True)
        os.replace(tmp, p)
    except OSError:
        pass  # a read-only home: tune again next time


def histogram_key(products) -> str:
    """Bucket of the row-length distribution: log2 of the mean row length and of the spread of
    per-matrix means, plus the largest number of right-hand sides."""
    means = np.array([max(p[0].nzval.numel(), 1) / max(p[0].m, 1) for p in products])
    rows = np.array([p[0].m for p in products], dtype=np.float64)
    mean = float(np.average(means, weights=np.maximum(rows, 1)))
    spread = float(np.std(np.log2(means))) if means.size > 1 else 0.0
    kmax = max(1 if p[1].dim() == 1 else p[1].shape[1] for p in products)
    return f"len{int(round(math.log2(max(mean, 1.0))))}/sp{int(round(spread * 2))}/k{kmax}"


def key_for(products) -> str:
    A = products[0][0]
    dev = torch.cuda.get_device_name(A.device)
    return f"{dev}|{A.dtype}|{A.itype}|{histogram_key(products)}"


def tune(products: Sequence, reps: int = 3, use_cache: bool = True) -> Tuple[int, int]:
    """(columns, g1_avg) for this product list: from the cache, or measured on it."""
    from .batch import BatchedMul
    key = key_for(products)
    cache = _load() if use_cache else {}
    if key in cache:
        c = cache[key]
        return int(c["columns"]), int(c["g1_avg"])
    kmax = max(1 if p[1].dim() == 1 else p[1].shape[1] for p in products)
    columns = (1,) if kmax == 1 else CANDIDATE_COLUMNS
    best, results = None, []
    for col in columns:
        for g1 in CANDIDATE_G1:
            b = BatchedMul(products, columns=col, g1_avg=g1)
            b.run("grouped")
            torch.cuda.synchronize()
            ts = []
            for _ in range(reps):
                s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                s.record()
                b.run("grouped")
                e.record()
                e.synchronize()
                ts.append(s.elapsed_time(e))
            b.close()
            t = min(ts)
            results.append({"columns": col, "g1_avg": g1, "ms": t})
            if best is None or t < best[0]:
                best = (t, col, g1)
    cache = _load()
    cache[key] = {"columns": best[1], "g1_avg": best[2], "ms": best[0], "tried": results}
    _save(cache)
    return best[1], best[2]
