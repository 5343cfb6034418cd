"""Autotuner for the batched rasterizer's launch configuration.

FB fixes bucket size 128, 16x16 tiles and one candidate tile per lane at compile time
(rasterizer_imp.h:24, :40-41; __init__.py:109).  Their best values depend on
the scene (footprint spread, Gaussians per tile) and the camera set, so the
batched path picks them per workload: every candidate ``TuneConfig`` is
planned, captured as a CUDA graph of one step (forward, or forward +
backward) and timed by replaying it; the fastest wins.  The search sweeps
bucket x tile x packet, then the forward's fold-chain length (``chain``,
which leaves the results bit-identical) for the winner.  Results are cached
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
PACKETS = (1, 2, 4, 8)
CHAINS = (2, 4, 8, 16, 32)

_MEMO: dict = {}


def search_space(buckets=BUCKETS, tiles=TILES, packets=PACKETS, include_default: bool = True) -> list[TuneConfig]:
    """bucket x tile x packet, plus FB's fixed choice (bucket 128, 16x16, packet 1)."""
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

    def sweep(cands):
        for cfg in cands:
            ms, pairs = time_config(settings, params, sh_degree, cfg, backward, reps, warmup)
            table.append(dict(config=dataclasses.asdict(cfg), ms=ms, pairs=pairs))
            if verbose:
                print(f"  {cfg}: {ms:.3f} ms  ({pairs} pairs)")
            torch.cuda.empty_cache()

    sweep(list(candidates) if candidates is not None else search_space())
    if candidates is None:  # second stage: the fold-chain length of the winner
        lead = TuneConfig(**min(table, key=lambda r: r["ms"])["config"])
        sweep([dataclasses.replace(lead, chain=c) for c in CHAINS if c != lead.chain])
    best = min(table, key=lambda r: r["ms"])
    cfg = TuneConfig(**best["config"])
    _MEMO[key] = cfg
    if path is not None:
        disk = _load(path)
        disk[key] = dict(config=best["config"], ms=best["ms"], seconds=time.time() - t0)
        _store(path, disk)
    return cfg, table


def autotune_native(settings, params: dict, sh_degree: int = 3, candidates: Iterable[TuneConfig] | None = None,
                    backward: bool = True, reps: int = 5, headroom: float = 1.15) -> tuple[TuneConfig, list[dict]]:
    """The same search through the library's own tuner (fgs_tune): plain launches timed with CUDA
    events instead of graph replays, for callers that drive the C ABI without Python.  Returns
    (best config, table of {config, ms}); ms is -1 for a config whose workspace did not fit and -2
    for one whose frame outgrew the planned pair capacity."""
    import ctypes as C

    from . import _lib
    from ._C import _f32, _ptr, _stream

    cands = list(candidates) if candidates is not None else search_space()
    P = params["means3D"].shape[0]
    probe = BatchedRasterizer(settings, P, tune=TuneConfig())
    pairs = probe.fit(params["means3D"], params["opacities"], params.get("dc"), params.get("shs"),
                      params.get("colors_precomp"), params["scales"], params["rotations"], params.get("culling"),
                      sh_degree, headroom=headroom)
    dev = probe.device
    cap = int(pairs * headroom) + (1 << 16)
    need = 0
    for cfg in cands:
        out = C.c_size_t(0)
        if _lib.load().fgs_batch_workspace_bytes(P, probe.V, probe._cams, C.byref(cfg.as_c()), cap, C.byref(out)) == 0:
            need = max(need, int(out.value))
    probe.workspace = None
    workspace = torch.empty(max(need, 256), dtype=torch.uint8, device=dev)
    dev_ = lambda k: _f32(k, params.get(k), dev)
    shs = dev_("shs")
    M = shs.size(1) if shs.numel() else 0
    dL = torch.ones(probe.out_color.numel(), device=dev) if backward else None
    gbytes = int(_lib.load().fgs_tune_grad_bytes(P, M))
    arena = torch.empty(max(gbytes, 256), dtype=torch.uint8, device=dev) if backward else None
    arr = (_lib.TuneConfig * len(cands))(*[c.as_c() for c in cands])
    ms = (C.c_float * len(cands))()
    best = C.c_int(-1)
    cull = params.get("culling")
    cull_t = cull.to(device=dev, dtype=torch.uint8).contiguous() if cull is not None and cull.numel() else None
    _lib.call("fgs_tune", P, int(sh_degree), int(M), _ptr(dev_("means3D")), _ptr(dev_("colors_precomp")),
              _ptr(dev_("dc")), _ptr(shs), _ptr(dev_("opacities")), _ptr(dev_("scales")), _ptr(dev_("rotations")),
              _ptr(cull_t), probe.V, probe._cams, arr, len(cands), cap, workspace.data_ptr(), workspace.numel(),
              probe.out_color.data_ptr(), probe.radii.data_ptr(), _ptr(dL), _ptr(arena), gbytes, int(reps),
              C.byref(best), ms, _stream(dev))
    table = [dict(config=dataclasses.asdict(c), ms=float(ms[i])) for i, c in enumerate(cands)]
    return cands[best.value], table
