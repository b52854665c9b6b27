"""Schedule autotuner: picks, per device, variant, precision and grid, the fastest of the
engine's execution schedules (``laps_set_schedule`` bits) and caches the choice on disk.

The schedules change how the kernels are launched, never what they compute (every schedule
gives bit-identical results): pass B of FP32 lines as one-shot or persistent double-buffered
blocks, pass E's L2 prefetch on or off, the continuity update beside pass D or in line.  A
candidate is timed with ``laps_step_profiled`` (CUDA events on the engine's stream, after one
step that captures the schedule's graph and warms its kernels); the cache is a JSON file
(``LAPS_TUNE_CACHE``, else ``~/.cache/laps_gb300/schedules.json``) keyed by the device name
and the run's shape, so a later run of the same kind starts from the cached schedule.
"""
from __future__ import annotations

import json
import os
from pathlib import Path

from . import ffi

CANDIDATES = tuple(range(ffi.SCHED_ALL + 1))


def cache_path() -> Path:
    env = os.environ.get("LAPS_TUNE_CACHE")
    return Path(env) if env else Path.home() / ".cache" / "laps_gb300" / "schedules.json"


def key(p: ffi.laps_params, device_name: str) -> str:
    """The cache key of a run: the device and what the schedules' speed depends on."""
    return (f"{device_name}|variant={p.variant}|precision={p.precision}|grid={p.nx}x{p.ny}x{p.nz}"
            f"|hall={p.if_Hall}|aeb={p.if_AEB}|dealias={p.dealias_option}")


def load_cache(path: Path | None = None) -> dict:
    path = path or cache_path()
    try:
        return json.loads(path.read_text())
    except (OSError, ValueError):
        return {}


def save_cache(cache: dict, path: Path | None = None):
    path = path or cache_path()
    path.parent.mkdir(parents=True, exist_ok=True)
    tmp = path.with_suffix(".tmp")
    tmp.write_text(json.dumps(cache, indent=1, sort_keys=True))
    tmp.replace(path)


def choose(times: dict) -> int:
    """The fastest schedule; ties go to the smaller bit pattern (the default first)."""
    return min(times, key=lambda b: (times[b], b))


def device_name(dev: int = 0) -> str:
    try:
        import torch

        return torch.cuda.get_device_name(dev)
    except Exception:
        return f"cuda:{dev}"


def tune(run: ffi.Laps, steps: int = 3, candidates=CANDIDATES, cache: dict | None = None, name: str | None = None,
         retune: bool = False) -> dict:
    """Pick the schedule of `run` (a context with its state uploaded): from the cache when it
    holds the run's key, else by timing every candidate.  The run is left on the chosen
    schedule; its state has advanced by the timed steps.  Returns {"bits", "times_ms",
    "from_cache", "key"}."""
    own = cache is None
    cache = load_cache() if own else cache
    k = key(run.p, name or device_name(run.p.device))
    if not retune and k in cache:
        run.set_schedule(int(cache[k]["bits"]))
        return {"bits": int(cache[k]["bits"]), "times_ms": cache[k].get("times_ms", {}), "from_cache": True, "key": k}
    times = {}
    for bits in candidates:
        run.set_schedule(bits)
        run.step(1)  # captures the schedule's graph, warms its kernels
        _, total_ms, _ = run.step_profiled(steps)
        times[bits] = total_ms / steps
    best = choose(times)
    run.set_schedule(best)
    cache[k] = {"bits": best, "times_ms": {str(b): t for b, t in times.items()}}
    if own:
        save_cache(cache)
    return {"bits": best, "times_ms": times, "from_cache": False, "key": k}
