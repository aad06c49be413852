"""Tile-shape autotuner for the fused step kernel.

For a mesh shape and arithmetic scheme it times every (tile_j, x_segment)
candidate on the device (CUDA events around a chunk of steps, from the zero
state, on a scratch simulation of the same shape) and keeps the fastest.  The
result is cached per (scheme, mesh, device) in a JSON file next to the built
library, so a shape is tuned once per machine.

tile_j sets the block (32 x tile_j threads, shared memory per block); the
x segment sets how many x planes a block marches and thereby the number of
blocks (several waves of the 152 SMs vs. the re-read of three halo planes per
segment).
"""
from __future__ import annotations

import json
import os
from pathlib import Path

import numpy as np

CACHE = Path(__file__).resolve().parent / "_build" / "autotune.json"
TILE_J = (4, 8, 16)
X_SEGMENTS = (16, 24, 32, 40, 48, 64)
DEFAULT = (8, 32)


def _device_name():
    try:
        import torch

        return torch.cuda.get_device_name()
    except Exception:
        return "cuda"


def _key(precision, shape):
    return f"{precision}:{shape[0]}x{shape[1]}x{shape[2]}:{_device_name()}"


def _load():
    try:
        return json.loads(CACHE.read_text())
    except (OSError, ValueError):
        return {}


def _store(d):
    CACHE.parent.mkdir(exist_ok=True)
    tmp = CACHE.with_suffix(".tmp")
    tmp.write_text(json.dumps(d, indent=1, sort_keys=True))
    os.replace(tmp, CACHE)


def tune(spacing, mat, table, dt, precision="f32k", steps=None, candidates=None, use_cache=True, verbose=False):
    """Best (tile_j, x_segment) for this mesh and scheme; times each candidate."""
    from .device import DeviceSimulation

    shape = tuple(int(s) for s in np.shape(mat))
    key = _key(precision, shape)
    cache = _load() if use_cache else {}
    if key in cache:
        return tuple(cache[key]["best"])
    if steps is None:
        steps = 48 if precision == "f32k" else 12
    cands = candidates or [(tj, xs) for tj in TILE_J for xs in X_SEGMENTS]
    src = np.zeros(steps + 12)
    results = []
    for tj, xs in cands:
        with DeviceSimulation(spacing, mat, table, dt, precision=precision, surface_mode="corrected",
                              max_steps=steps + 12, tile_j=tj, x_segment=xs) as sim:
            sim.set_source(src)
            sim.step(12)  # warm up: graph capture, first-touch
            sim.sync()
            sim.step(steps)
            ms = sim.last_step_ms() / steps
            results.append((ms, tj, xs))
            if verbose:
                print(f"autotune {precision} {shape} tile_j={tj} x_segment={xs}: {ms:.4f} ms/step")
    results.sort()
    best = (results[0][1], results[0][2])
    if use_cache:
        cache = _load()
        cache[key] = {"best": list(best), "ms_per_step": results[0][0],
                      "all": [[tj, xs, round(ms, 5)] for ms, tj, xs in results]}
        _store(cache)
    return best
