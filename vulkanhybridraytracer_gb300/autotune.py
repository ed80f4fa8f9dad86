"""Launch-shape autotuner for the hybrid pass.

Times a workload under each candidate launch shape — queue chunk (8x4 tiles
a warp pulls per atomic: 32..1024 pixels) and register cap of the shadow
kernel (5, 6 or 8 resident 128-thread blocks per SM, i.e. 96, 80 or 64
registers)
— and keeps the fastest.  Results are cached on disk per GPU name and
workload signature, so a workload is tuned once per machine.
"""
from __future__ import annotations

import json
import os
import time
from pathlib import Path

CHUNKS = (1, 2, 4, 8, 16, 32)       # tiles per queue pull: 32 .. 1024 pixels
MIN_BLOCKS = (5, 6, 8)

DEFAULT_CACHE = Path(os.environ.get("HY_AUTOTUNE_CACHE", Path.home() / ".cache" / "hybridrt_autotune.json"))


def _load(path: Path) -> dict:
    try:
        return json.loads(path.read_text())
    except Exception:
        return {}


def _save(path: Path, data: dict) -> None:
    try:
        path.parent.mkdir(parents=True, exist_ok=True)
        path.write_text(json.dumps(data, indent=1))
    except OSError:
        pass


def cached(signature: str, device_name: str, cache_path: Path | None = DEFAULT_CACHE) -> dict | None:
    """The cached winner for this GPU and workload, or None."""
    if not cache_path:
        return None
    hit = _load(cache_path).get(f"{device_name}|{signature}")
    if hit is None:
        return None
    out = dict(hit)
    out["cached"] = True
    return out


def autotune(run, signature: str, device_name: str, chunks=CHUNKS, min_blocks=MIN_BLOCKS, reps: int = 2,
             cache_path: Path | None = DEFAULT_CACHE, timer=None) -> dict:
    """run(chunk, min_blocks) executes the workload once.  timer(fn) returns
    seconds for one call of fn (default: wall clock around a synchronised call).
    Returns {"chunk", "min_blocks", "ms", "tried": [...], "cached": bool}."""
    key = f"{device_name}|{signature}"
    cache = _load(cache_path) if cache_path else {}
    if key in cache:
        out = dict(cache[key])
        out["cached"] = True
        return out
    if timer is None:
        def timer(fn):
            t0 = time.perf_counter()
            fn()
            return time.perf_counter() - t0
    tried = []
    for mb in min_blocks:
        for ch in chunks:
            run(ch, mb)  # warm-up (and graph capture for a new shape)
            t = min(timer(lambda: run(ch, mb)) for _ in range(reps))
            tried.append({"chunk": ch, "min_blocks": mb, "ms": 1e3 * t})
    best = min(tried, key=lambda r: r["ms"])
    out = {"chunk": best["chunk"], "min_blocks": best["min_blocks"], "ms": best["ms"], "tried": tried}
    if cache_path:
        cache[key] = out
        _save(cache_path, cache)
    out = dict(out)
    out["cached"] = False
    return out
