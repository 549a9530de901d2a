"""Autotuner of the split-BF16 contraction's schedule per PD size class.

The tensor-core contraction of D (include/manifoldem_gb300.h, ``mem_contraction_config``) runs
the tiles of each size class of PDs in one launch with the class's schedule: tiles of 128 x 128
or 128 x 256 entries of D on one SM, or 256 x 128 on a pair of SMs sharing one MMA stream (the
larger tiles read a quarter fewer operand bytes per MMA but pad small PDs more), one CTA per
tile or one persistent CTA per SM walking its tiles, with two or four TMEM accumulators (how
many accumulation groups the MMA issuer may run ahead of the epilogue, across tile
boundaries).  Which is fastest depends on the PD size (padding, tiles per PD, the tail of the
last wave) and on the box size (K, the length of each tile's main loop), so the choice is
measured: for each class a synthetic batch of PDs of the class's typical size is planned once
per candidate schedule and its contraction phase timed with the library's phase events (median
of a few executes); the simplest schedule is kept unless another is clearly faster, and
adjacent classes that chose the same schedule are merged into one launch.

Results are cached in a JSON file keyed by GPU name, box size and contraction form
(``MEM_AUTOTUNE_CACHE`` names the file; default ``autotune_cache.json`` beside this module);
``pipeline.Plan`` applies a cached table when it creates a plan.  The reference has no
counterpart: its D is one float64 GEMM per PD on the CPU
(modules/getDistanceCTF_local_Conj9combinedS2.py:391-397).
"""
from __future__ import annotations

import ctypes
import json
import os
import threading
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import _lib

HERE = os.path.dirname(os.path.abspath(__file__))

# size classes (largest PD of each; the last takes every larger PD) and the PD size the class
# is tuned on
CLASS_MAX_N = (192, 640, 1536, 2 ** 31 - 1)
CLASS_REP_N = (160, 400, 1000, 2500)
# candidate schedules, simplest first: (persistent, accumulators, tile width, tile height);
# height 256 = a pair of SMs sharing one MMA stream
CANDIDATES = ((0, 2, 128, 128), (1, 2, 128, 128), (1, 4, 128, 128), (0, 2, 256, 128),
              (1, 2, 256, 128), (0, 2, 128, 256), (1, 2, 128, 256), (1, 4, 128, 256))
TARGET_TILES = 1216         # about eight waves of 128 x 128 tiles on 152 SMs
# a schedule later in CANDIDATES (more machinery) must beat the current choice by this fraction
TIE_MARGIN = 0.03

_lock = threading.Lock()


def cache_path() -> str:
    return os.environ.get('MEM_AUTOTUNE_CACHE', os.path.join(HERE, 'autotune_cache.json'))


def cache_key(gpu_name: str, N: int, precision: str) -> str:
    return '%s|N=%d|%s' % (gpu_name, int(N), precision)


def _read_cache() -> Dict[str, dict]:
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _write_cache(d: Dict[str, dict]) -> None:
    path = cache_path()
    tmp = path + '.tmp.%d' % os.getpid()
    with open(tmp, 'w') as f:
        json.dump(d, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def lookup(gpu_name: str, N: int, precision: str) -> Optional[List[dict]]:
    """The cached class table for this GPU, box size and form, or None."""
    with _lock:
        ent = _read_cache().get(cache_key(gpu_name, N, precision))
    return None if ent is None else ent['classes']


def to_c(classes: Sequence[dict]):
    arr = (_lib.MemContractionConfig * len(classes))()
    for i, c in enumerate(classes):
        arr[i].max_n = int(c['max_n'])
        arr[i].persistent = int(c['persistent'])
        arr[i].accumulators = int(c['accumulators'])
        arr[i].tile_n = int(c.get('tile_n', 128))
        arr[i].tile_m = int(c.get('tile_m', 128))
        arr[i].reserved = 0
    return arr


def _class_batch(rep_n: int) -> List[int]:
    nb = -(-rep_n // 128)
    tiles_per_pd = nb * (nb + 1) // 2
    n_pd = max(1, -(-TARGET_TILES // tiles_per_pd))
    return [rep_n] * n_pd


def _time_schedule(params, counts, sched: Tuple[int, int, int, int], device,
                   reps: int = 5) -> float:
    """Median contraction-phase time (ms) of a plan of `counts` random PDs with one schedule."""
    import torch
    from .pipeline import Plan
    cfg = [dict(max_n=2 ** 31 - 1, persistent=sched[0], accumulators=sched[1],
                tile_n=sched[2], tile_m=sched[3])]
    plan = Plan(params, counts, [0.0] * len(counts), device, contraction=cfg)
    n_img = plan.n_images
    g = torch.Generator(device=device).manual_seed(1)
    N = params.N
    stack = torch.randn((n_img, N, N), generator=g, device=device, dtype=torch.float32)
    sidx = torch.arange(n_img, device=device, dtype=torch.int64)
    flip = torch.zeros(n_img, device=device, dtype=torch.uint8)
    psi = torch.rand(n_img, generator=g, device=device, dtype=torch.float64) * 6.2
    df = 1e4 + 2e4 * torch.rand(n_img, generator=g, device=device, dtype=torch.float64)
    outs = plan.allocate_outputs(('D',))
    lib = plan.lib
    plan.execute(stack, sidx, flip, psi, df, outs)          # warm-up
    lib.mem_plan_set_timing(plan.handle, 1)
    times = []
    phase = (ctypes.c_float * 9)()
    for _ in range(reps):
        plan.execute(stack, sidx, flip, psi, df, outs)
        lib.mem_plan_phase_times(plan.handle, phase, 9)
        times.append(float(phase[8]))
    lib.mem_plan_set_timing(plan.handle, 0)
    torch.cuda.synchronize(device)
    plan.device_status()
    del plan, stack, outs
    return float(np.median(times))


def tune(params, device=None, force: bool = False) -> List[dict]:
    """Measure every candidate schedule for every size class at params.N and params.precision
    (split-BF16 only; the FP32 form has one schedule), cache and return the class table."""
    import dataclasses
    import torch
    device = torch.device(device or 'cuda')
    name = torch.cuda.get_device_name(device)
    if params.precision != 'bf16x3':
        return []
    if not force:
        got = lookup(name, params.N, params.precision)
        if got is not None:
            return got
    p = dataclasses.replace(params, avg_only=False)
    classes = []
    for max_n, rep_n in zip(CLASS_MAX_N, CLASS_REP_N):
        counts = _class_batch(rep_n)
        ms = {s: _time_schedule(p, counts, s, device) for s in CANDIDATES}
        best = pick(ms)
        classes.append(dict(max_n=int(max_n), persistent=best[0], accumulators=best[1],
                            tile_n=best[2], tile_m=best[3], rep_n=rep_n, pds=len(counts),
                            ms={'%d,%d,%d,%d' % s: round(v, 4) for s, v in ms.items()}))
        torch.cuda.empty_cache()
    classes = merge_classes(classes)
    with _lock:
        d = _read_cache()
        d[cache_key(name, params.N, params.precision)] = dict(classes=classes)
        _write_cache(d)
    return classes


def pick(ms: Dict[tuple, float]) -> tuple:
    """The schedule of a class from its measured times: walking CANDIDATES in order (simplest
    first), a later schedule replaces the current choice only when it is faster by more than
    TIE_MARGIN."""
    order = [c for c in CANDIDATES if c in ms]
    best = order[0]
    for cand in order[1:]:
        if ms[cand] < ms[best] * (1.0 - TIE_MARGIN):
            best = cand
    return best


def merge_classes(classes: List[dict]) -> List[dict]:
    """Adjacent classes with the same schedule become one (one launch instead of two, one
    tail instead of two); the merged class keeps the larger max_n and both measurements."""
    key = lambda c: (c['persistent'], c['accumulators'], c.get('tile_n', 128),
                     c.get('tile_m', 128))
    out: List[dict] = []
    for c in classes:
        if out and key(out[-1]) == key(c):
            prev = out[-1]
            prev['max_n'] = c['max_n']
            prev['merged'] = prev.get('merged', [dict(rep_n=prev.get('rep_n'),
                                                      ms=prev.get('ms'))])
            prev['merged'].append(dict(rep_n=c.get('rep_n'), ms=c.get('ms')))
        else:
            out.append(dict(c))
    return out
