"""Tile-shape autotuner for the fused step kernel, single meshes and batches.

``tune``: for one mesh shape and arithmetic scheme it times every
(tile_j, x_segment) candidate on a scratch simulation of that shape (CUDA
events around a chunk of steps from the zero state; ``phono_set_tiling``
switches the candidate in place) and keeps the fastest.

``tune_batch``: for a mix of mesh shapes stepped as one batch it picks the
batch's tile height and each instance's x segment, i.e. how many
(instance, tile) work items every instance contributes to the persistent
launch.  Stage 1 times the whole mix for every tile height and one common
x segment; stage 2 revisits the x segment of each group of instances with
the same x extent, keeping a change only when the whole batch gets faster.

Timing uses scratch simulations (zero material ids and zero source: the
kernel's work does not depend on the values), so tuning never touches the
caller's state.  Results are cached per (scheme, shapes, device) in a JSON
file next to the built library, so a mesh or a mix is tuned once per machine.

tile_j sets the block (a 32 x tile_j tile: 32 x tile_j threads at height 4,
two rows a thread at 8 and 16 in FP32; shared memory per block); the x
segment sets how many x planes a block marches and thereby the number of
blocks (several waves of the 152 SMs vs. the re-read of two halo planes per
segment).  Blocks are dispatched segment by segment, so segments that
shorten towards the end of the list (tapered or listed) make the blocks that
run while the GPU drains at the end of a launch short.
"""
from __future__ import annotations

import hashlib
import json
import os
from pathlib import Path

import numpy as np

CACHE = Path(__file__).resolve().parent / "_build" / "autotune.json"
TILE_J = (4, 8, 16)
X_SEGMENTS = (12, 16, 20, 24, 28, 32, 40, 48, 64)
X_TAPERED = (16, 20, 24, 28, 32, 48)  # -L: L-plane segments shortening towards the end (see phono_desc.x_segment)
# listed segments (phono_set_segments): L-plane segments, then one of these
# shortening tails, so that the last blocks of a launch are short
LISTED_L = (24, 28, 30, 32, 36)
TAILS = ((16, 12, 8, 6, 4), (10, 8, 6, 4, 4), (12, 8, 4, 4, 4), (20, 16, 12, 8, 4), (6, 6, 6, 6, 4, 4))
_HOST_ROW = np.array([[224e9, 64e9, 64e9, 64e9, 224e9, 64e9, 64e9, 64e9, 224e9, 80e9, 80e9, 80e9, 2330.0]])


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


def _store(key, value):
    d = _load()
    d[key] = value
    CACHE.parent.mkdir(exist_ok=True)
    tmp = CACHE.with_suffix(f".tmp{os.getpid()}")
    tmp.write_text(json.dumps(d, indent=1, sort_keys=True))
    os.replace(tmp, CACHE)


def _scratch(shape, precision, max_steps, tile_j=8, x_segment=32):
    """Simulation of the given mesh shape with zero ids, uniform 10 um spacing and a zero source."""
    from .device import DeviceSimulation

    nx, ny, nz = shape
    sp = {f"fd{a}": np.full(n - 1, 1e-5) for a, n in zip("xyz", shape)}
    sp.update({f"sd{a}": np.full(n - 2, 1e-5) for a, n in zip("xyz", shape)})
    sim = DeviceSimulation(sp, np.zeros(shape, np.uint8), _HOST_ROW, 1e-10, precision=precision,
                           surface_mode="corrected", max_steps=max_steps, tile_j=tile_j, x_segment=x_segment)
    sim.set_source(np.zeros(max_steps))
    return sim


def listed_segments(planes, length, tail):
    """Segment lengths: length-plane segments, then the tail; the planes left
    over are spread over the long segments.  None if they do not fit."""
    rest = planes - sum(tail)
    full = rest // length if rest > 0 else 0
    if full < 1 or full + len(tail) > 64:
        return None
    extra = rest - full * length
    return tuple(length + extra // full + (1 if q < extra % full else 0) for q in range(full)) + tuple(tail)


def tapered_count(planes, length):
    """Segments of x_segment = -length over `planes` planes: length-plane
    segments while more than 2 * length planes are left, then the rest in
    four parts (phono_desc.x_segment)."""
    p = n = 0
    while planes - p > 2 * length:
        p += length
        n += 1
    rest = planes - p
    return n + (4 if rest >= 4 else rest)


def candidates_for(shape, tile_js=TILE_J):
    """(tile_j, x_segment) candidates of a mesh: even, tapered and listed
    segments; tapered and listed ones only where they take at most 64
    segments (the most a launch describes by table)."""
    planes = int(shape[0]) - 1
    cands = [(tj, xs) for tj in tile_js for xs in X_SEGMENTS]
    cands += [(tj, -xs) for tj in tile_js for xs in X_TAPERED if tapered_count(planes, xs) <= 64]
    for tj in tile_js:
        for length in LISTED_L:
            for tail in TAILS:
                seg = listed_segments(planes, length, tail)
                if seg is not None and (tj, seg) not in cands:
                    cands.append((tj, seg))
    return cands


def tune(spacing, mat, table, dt, precision="f32k", steps=None, candidates=None, use_cache=True, verbose=False):
    """Best (tile_j, x_segment) for this mesh and scheme; times each candidate."""
    shape = tuple(int(s) for s in np.shape(mat))
    key = _key(precision, shape)
    if use_cache:
        hit = _load().get(key)
        if hit:
            tj, xs = hit["best"]
            return int(tj), (tuple(xs) if isinstance(xs, list) else int(xs))
    if steps is None:
        steps = 48 if precision == "f32k" else 12
    cands = candidates or candidates_for(shape)
    results = []
    sim = _scratch(shape, precision, (steps + 12) * len(cands) + 12)
    try:
        for tj, xs in cands:
            sim.set_tiling(tj, xs)
            sim.step(12)  # warm up: graph capture
            sim.sync()
            sim.step(steps)
            ms = sim.last_step_ms() / steps
            results.append((ms, tj, xs))
            if verbose:
                print(f"autotune {precision} {shape} tile_j={tj} x_segment={xs}: {ms:.4f} ms/step")
    finally:
        sim.close()
    results.sort(key=lambda r: r[0])
    best = (results[0][1], results[0][2])
    if use_cache:
        _store(key, {"best": [best[0], list(best[1]) if isinstance(best[1], tuple) else best[1]],
                     "ms_per_step": results[0][0],
                     "all": [[tj, list(xs) if isinstance(xs, tuple) else xs, round(ms, 5)] for ms, tj, xs in results]})
    return best


def _batch_key(precision, shapes):
    h = hashlib.sha1(json.dumps(sorted(map(list, shapes))).encode()).hexdigest()[:16]
    return f"batch:{precision}:{len(shapes)}:{h}:{_device_name()}"


def tune_batch(shapes, precision="f32k", steps=24, tile_js=TILE_J, use_cache=True, verbose=False, streams=0):
    """Tile height of a batch and the x segment of each instance.

    shapes: mesh node counts (nx, ny, nz) of the instances, in batch order.
    streams: 0 times the persistent scheme, W > 0 the streams scheme on W
    worker streams (every instance at the chosen tile height).
    Returns (tile_j, [x_segment per instance]).
    """
    from .batch import Batch

    shapes = [tuple(int(v) for v in s) for s in shapes]
    key = _batch_key(precision, shapes) + ":" + ",".join(map(str, tile_js)) + (f":streams{streams}" if streams else "")
    if use_cache:
        hit = _load().get(key)
        if hit:
            by_nx = {int(k): v for k, v in hit["x_segment_by_nx"].items()}
            return int(hit["tile_j"]), [by_nx[s[0]] for s in shapes]
    groups = sorted({s[0] for s in shapes})
    seg_cands = {nx: sorted({xs for xs in X_SEGMENTS if xs < nx - 1} | {nx - 1}) for nx in groups}
    n_timings = len(tile_js) * (len(X_SEGMENTS) + 1) + sum(len(c) for c in seg_cands.values())
    budget = (steps + 12) * (n_timings + 2)
    sims = [_scratch(s, precision, budget) for s in shapes]
    log = []

    def time_mix(tj, seg_by_nx):
        for sim in sims:
            sim.set_tiling(tj, seg_by_nx[sim.nx])
        with Batch(len(sims), precision=precision, tile_j=tj, streams=streams) as b:
            for sim in sims:
                b.add(sim, steps + 12)
            b.step(12)  # work list upload, graph capture
            b.sync()
            b.step(steps)
            ms = b.last_step_ms() / steps
        log.append([tj, {str(k): v for k, v in seg_by_nx.items()}, round(ms, 5)])
        if verbose:
            print(f"autotune batch streams={streams} tile_j={tj} x_segment={seg_by_nx}: {ms:.4f} ms/step")
        return ms

    try:
        best = None
        for tj in tile_js:
            for xs in list(X_SEGMENTS) + [0]:  # 0: one segment per block column
                seg = {nx: (min(xs, nx - 1) if xs else nx - 1) for nx in groups}
                ms = time_mix(tj, seg)
                if best is None or ms < best[0]:
                    best = (ms, tj, dict(seg))
        ms_best, tj, seg = best
        for nx in reversed(groups):  # per-group refinement, largest x extent first
            for xs in seg_cands[nx]:
                if xs == seg[nx]:
                    continue
                trial = dict(seg)
                trial[nx] = xs
                ms = time_mix(tj, trial)
                if ms < 0.99 * ms_best:
                    ms_best, seg = ms, trial
    finally:
        for sim in sims:
            sim.close()
    if use_cache:
        _store(key, {"tile_j": tj, "x_segment_by_nx": {str(k): v for k, v in seg.items()},
                     "ms_per_step": ms_best, "timings": log})
    return tj, [seg[s[0]] for s in shapes]
