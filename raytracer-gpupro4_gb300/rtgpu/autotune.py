"""Launch-shape autotuner of the batched trace, with a JSON cache.

The batched trace (rt_batch_trace) has four launch knobs: threads per block,
a cap on resident blocks per SM, how many work items a warp takes per
increment of the work counter (grab), and the order of the work items
(scene-major or interleaved).  The best choice depends on the GPU and on the
batch's shape, so it is measured once per (GPU, size bucket) and kept in a
JSON file:

    { "<gpu key>|<size bucket>": {"threads": 128, "blocks_per_sm": 0,
                                  "grab": 2, "order": 0, "ms": 11.3}, ... }

gpu key = device name, compute capability and SM count; size bucket =
scene count, log2 of the total triangle count and log2 of the pixels per
scene, so batches of similar shape share an entry.  The cache path is
$RTGPU_TUNE_CACHE, else ~/.cache/rtgpu/batch_tuning.json.
"""
from __future__ import annotations

import itertools
import json
import math
import os
import tempfile
from pathlib import Path
from typing import Callable, Iterable

THREADS = (64, 128, 256)
GRABS = (1, 2, 4, 8)
ORDERS = (0, 1)
DEFAULT = {"threads": 128, "blocks_per_sm": 0, "grab": 1, "order": 0}


def default_cache_path() -> Path:
    env = os.environ.get("RTGPU_TUNE_CACHE")
    if env:
        return Path(env)
    return Path.home() / ".cache" / "rtgpu" / "batch_tuning.json"


def gpu_key(name: str, capability: tuple[int, int], sms: int) -> str:
    return f"{name.strip().replace('|', '/')}:sm{capability[0]}{capability[1]}:{sms}sm"


def size_bucket(n_scenes: int, total_tris: int, width: int, height: int) -> str:
    lt = int(math.floor(math.log2(max(1, total_tris))))
    lp = int(math.floor(math.log2(max(1, width * height))))
    return f"S{n_scenes}:T2^{lt}:P2^{lp}"


def candidates(threads: Iterable[int] = THREADS, grabs: Iterable[int] = GRABS,
               orders: Iterable[int] = ORDERS) -> list[dict]:
    return [{"threads": t, "blocks_per_sm": 0, "grab": g, "order": o}
            for t, g, o in itertools.product(threads, grabs, orders)]


class TuneCache:
    """JSON file of tuned launch shapes; writes are atomic (temp file + rename)."""

    def __init__(self, path: Path | str | None = None):
        self.path = Path(path) if path is not None else default_cache_path()
        self.entries: dict[str, dict] = {}
        if self.path.exists():
            try:
                data = json.loads(self.path.read_text())
                if isinstance(data, dict):
                    self.entries = {k: v for k, v in data.items() if _valid(v)}
            except (OSError, ValueError):
                self.entries = {}  # a damaged cache is re-measured, not trusted

    def get(self, key: str) -> dict | None:
        return self.entries.get(key)

    def put(self, key: str, cfg: dict) -> None:
        self.entries[key] = dict(cfg)
        self.path.parent.mkdir(parents=True, exist_ok=True)
        fd, tmp = tempfile.mkstemp(prefix=".tune", dir=str(self.path.parent))
        with os.fdopen(fd, "w") as f:
            json.dump(self.entries, f, indent=1, sort_keys=True)
        os.replace(tmp, self.path)


def _valid(cfg) -> bool:
    return (isinstance(cfg, dict) and cfg.get("threads") in THREADS and isinstance(cfg.get("grab"), int)
            and 1 <= cfg["grab"] <= 16 and cfg.get("order") in ORDERS)


def pick(timings: list[tuple[dict, float]]) -> dict:
    """Fastest candidate; ties keep the earlier one (candidates() order)."""
    if not timings:
        raise ValueError("no candidate was timed")
    best_cfg, best_ms = timings[0]
    for cfg, ms in timings[1:]:
        if ms < best_ms:
            best_cfg, best_ms = cfg, ms
    out = dict(best_cfg)
    out["ms"] = float(best_ms)
    return out


def tune(key: str, timer: Callable[[dict], float], cache: TuneCache | None = None,
         cands: list[dict] | None = None, force: bool = False) -> dict:
    """Cached best launch shape for `key`; `timer(cfg)` returns milliseconds."""
    cache = cache if cache is not None else TuneCache()
    if not force:
        hit = cache.get(key)
        if hit is not None:
            return hit
    timings = [(c, float(timer(c))) for c in (cands if cands is not None else candidates())]
    best = pick(timings)
    cache.put(key, best)
    return best


def autotune_batch(batch, hits, vis=None, cache: TuneCache | None = None, reps: int = 3,
                   force: bool = False) -> dict:
    """Tunes rt_batch_trace for `batch` (an rtgpu.api.Batch with views set),
    applies the best shape to it and returns it."""
    import torch

    dev = batch.ctx.torch_device
    props = torch.cuda.get_device_properties(dev)
    key = gpu_key(props.name, (props.major, props.minor), props.multi_processor_count) + "|" + size_bucket(
        batch.n_scenes, batch.total, batch.width, batch.height)
    stream = batch.ctx.stream

    def timer(cfg: dict) -> float:
        batch.tuning = cfg
        batch.trace(hits, vis)  # warm-up
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        stream.synchronize()
        start.record(stream)
        for _ in range(reps):
            batch.trace(hits, vis)
        end.record(stream)
        end.synchronize()
        batch.ctx.check()
        return start.elapsed_time(end) / reps

    best = tune(key, timer, cache, force=force)
    batch.tuning = best
    return best
