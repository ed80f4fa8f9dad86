"""Launch-shape autotuning of the batched pass, with an on-disk cache.

The search itself is the library's ``hy_batch_autotune`` (so a C++ caller of
``hy_batch_forward`` has it too): one axis at a time, the batch's tile-stream
shadow kernel is timed under each queue chunk (1..32 tiles = 32..1024 pixels),
block size (64, 128, 256 threads), register cap (6 or 8 resident 128-thread
blocks per SM = 80 or 64 registers) and shared-memory stack depth (0, 8, 16,
32 entries), keeping the fastest.  This module caches the winner per GPU name
and workload signature, so a workload is tuned once per machine.
"""
from __future__ import annotations

import json
import os
from pathlib import Path

DEFAULT_CACHE = Path(os.environ.get("HY_AUTOTUNE_CACHE", Path.home() / ".cache" / "hybridrt_autotune.json"))
DEFAULT = {"chunk": 1, "block": 256, "min_blocks": 8, "stack_depth": 0}  # hy_batch_forward's own default


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


def tuning_config(shape: dict):
    """The HyPassConfig a batch takes as its tuning for a shape dict."""
    from .hybrid import pass_config

    return pass_config(1, queue_chunk=shape["chunk"], block_size=shape["block"], min_blocks=shape["min_blocks"],
                       stack_depth=shape["stack_depth"])


def cached(signature: str, device_name: str, cache_path: Path | None = DEFAULT_CACHE) -> dict | None:
    """The cached shape for this GPU and workload, or None."""
    if not cache_path:
        return None
    hit = _load(cache_path).get(f"{device_name}|{signature}")
    if hit is None:
        return None
    out = dict(hit)
    out["cached"] = True
    return out


def autotune(runner, scenes, views, signature: str, device_name: str, reps: int = 2,
             cache_path: Path | None = DEFAULT_CACHE) -> dict:
    """The fastest launch shape of a batch (runner: a HybridContext; scenes, views as for
    batch_forward).  Returns {"chunk", "block", "min_blocks", "stack_depth", "ms", "cached"}.
    Tuning runs the batch many times: its histories and outputs are overwritten."""
    hit = cached(signature, device_name, cache_path)
    if hit is not None:
        return hit
    t, ms = runner.batch_autotune(scenes, views, reps)
    out = {"chunk": int(t.queue_chunk), "block": int(t.block_size), "min_blocks": int(t.min_blocks),
           "stack_depth": int(t.stack_depth), "ms": float(ms)}
    if cache_path:
        cache = _load(cache_path)
        cache[f"{device_name}|{signature}"] = out
        _save(cache_path, cache)
    out = dict(out)
    out["cached"] = False
    return out
