"""Autotuner for the batched rasterizer's launch configuration.

FB fixes bucket size 128, 16x16 tiles and 128-tile sub-tasks at compile time
(rasterizer_imp.h:24, :40-41; __init__.py:109).  Their best values depend on
the scene (footprint spread, Gaussians per tile) and the camera set, so the
batched path picks them per workload: every candidate ``TuneConfig`` is
planned, captured as a CUDA graph of one step (forward, or forward +
backward) and timed by replaying it; the fastest wins.  Results are cached
per (Gaussian-count range, camera resolutions, SH degree, step kind) in
memory and, when ``cache_path`` (or ``FGS_TUNE_CACHE``) names a file, on
disk as JSON.
"""
from __future__ import annotations

import dataclasses
import itertools
import json
import math
import os
import time
from pathlib import Path
from typing import Iterable, Sequence

import torch

from .batched import BatchedRasterizer, CapturedStep, TuneConfig

BUCKETS = (16, 32, 64)
TILES = ((16, 16), (8, 32))
PACKETS = (2, 4, 8)

_MEMO: dict = {}


def search_space(buckets=BUCKETS, tiles=TILES, packets=PACKETS, include_default: bool = True) -> list[TuneConfig]:
    """bucket x tile x packet, plus FB's fixed choice (bucket 128, 16x16, packet 4)."""
    space = [TuneConfig(b, bx, by, p) for b, (bx, by), p in itertools.product(buckets, tiles, packets)]
    if include_default and TuneConfig() not in space:
        space.append(TuneConfig())
    return space


def cache_key(P: int, sizes: Sequence[tuple[int, int]], sh_degree: int, backward: bool) -> str:
    prange = 1 << max(0, math.ceil(math.log2(max(P, 1))))  # next power of two
    res = ",".join(f"{w}x{h}" for h, w in sizes)
    return f"P<={prange}|{res}|deg{sh_degree}|{'fwdbwd' if backward else 'fwd'}"


def _load(path: Path | None) -> dict:
    if path is None or not path.exists():
        return {}
    try:
        return json.loads(path.read_text())
    except (OSError, ValueError):
        return {}


def _store(path: Path | None, table: dict) -> None:
    if path is None:
        return
    tmp = path.with_suffix(path.suffix + ".tmp")
    tmp.write_text(json.dumps(table, indent=1, sort_keys=True))
    os.replace(tmp, path)


def time_config(settings, params: dict, sh_degree: int, tune: TuneConfig, backward: bool = True, reps: int = 5,
                warmup: int = 2, headroom: float = 1.15) -> tuple[float, int]:
    """Milliseconds per replay of one captured step with this config, and its pair count."""
    P = params["means3D"].shape[0]
    rast = BatchedRasterizer(settings, P, tune=tune)
    pairs = rast.fit(params["means3D"], params["opacities"], params.get("dc"), params.get("shs"),
                     params.get("colors_precomp"), params["scales"], params["rotations"], params.get("culling"),
                     sh_degree, headroom=headroom)
    dL = torch.ones(rast.out_color.numel(), device=rast.device)
    step = CapturedStep(rast, params, dL, sh_degree=sh_degree, with_backward=backward)
    for _ in range(warmup):
        step.replay()
    s = torch.cuda.current_stream(rast.device)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(rast.device)
    e0.record(s)
    for _ in range(reps):
        step.replay()
    e1.record(s)
    torch.cuda.synchronize(rast.device)
    rast.status()  # raises if a replay overflowed its planned capacity
    ms = e0.elapsed_time(e1) / reps
    del step, rast
    return ms, pairs


def autotune(settings, params: dict, sh_degree: int = 3, candidates: Iterable[TuneConfig] | None = None,
             backward: bool = True, reps: int = 5, warmup: int = 2, cache_path: str | os.PathLike | None = None,
             force: bool = False, verbose: bool = False) -> tuple[TuneConfig, list[dict]]:
    """Pick the fastest TuneConfig for this scene and camera set.

    Returns (best config, table of {config, ms, pairs}); a cached answer
    returns an empty table unless force=True.
    """
    P = params["means3D"].shape[0]
    sizes = [(int(s.image_height), int(s.image_width)) for s in settings]
    key = cache_key(P, sizes, sh_degree, backward)
    path = Path(cache_path or os.environ.get("FGS_TUNE_CACHE", "")) if (cache_path or
                                                                         os.environ.get("FGS_TUNE_CACHE")) else None
    if not force:
        if key in _MEMO:
            return _MEMO[key], []
        disk = _load(path)
        if key in disk:
            cfg = TuneConfig(**disk[key]["config"])
            _MEMO[key] = cfg
            return cfg, []
    table = []
    t0 = time.time()
    for cfg in (list(candidates) if candidates is not None else search_space()):
        ms, pairs = time_config(settings, params, sh_degree, cfg, backward, reps, warmup)
        table.append(dict(config=dataclasses.asdict(cfg), ms=ms, pairs=pairs))
        if verbose:
            print(f"  {cfg}: {ms:.3f} ms  ({pairs} pairs)")
        torch.cuda.empty_cache()
    best = min(table, key=lambda r: r["ms"])
    cfg = TuneConfig(**best["config"])
    _MEMO[key] = cfg
    if path is not None:
        disk = _load(path)
        disk[key] = dict(config=best["config"], ms=best["ms"], seconds=time.time() - t0)
        _store(path, disk)
    return cfg, table
