"""Run one seeded crystal on the GPU: ``python -m phonomena_gb300 --cells 256,256,128 --steps 2000``.

Builds the crystal (lattice a=16, radii U[0.2a, 0.4a], 25% tungsten, 42 MHz
line source), steps it with the chosen scheme and tile shape, and prints the
device time, Gcell-updates/s and the energy.  With ``--batch N`` it runs N
crystals of the batching mix in one batch instead (``--batch-streams W``:
the streams scheme on W worker streams).  Used as the fixed command
for profiling the kernels.
"""
from __future__ import annotations

import argparse
import json
import sys
import time


def main(argv=None):
    p = argparse.ArgumentParser(prog="python -m phonomena_gb300")
    p.add_argument("--cells", default="256,256,128")
    p.add_argument("--steps", type=int, default=2000)
    p.add_argument("--precision", default="f32k", choices=["f64", "f32k", "f64v"])
    p.add_argument("--tile-j", type=int, default=8)
    p.add_argument("--x-segment", type=int, default=32)
    p.add_argument("--x-segments", default="", help="explicit x segment lengths, comma separated (phono_set_segments)")
    p.add_argument("--batch", type=int, default=0, help="run this many crystals of the batching mix instead")
    p.add_argument("--batch-streams", type=int, default=0,
                   help="with --batch: worker streams of the streams scheme (0: the persistent kernel)")
    p.add_argument("--seed", type=int, default=0)
    a = p.parse_args(argv)

    from . import build, crystal

    build.build()
    from .device import DeviceSimulation

    if a.batch:
        from .batch import Batch

        specs = crystal.config4_specs(n=a.batch, seed=a.seed, steps=a.steps)
        sims = []
        for sp in specs:
            g, m = crystal.build(sp)
            s = DeviceSimulation(g.spacing(), m.ids, m.table, m.dt, precision=a.precision, surface_mode="corrected",
                                 max_steps=a.steps, record_every=10, tile_j=a.tile_j, x_segment=a.x_segment)
            s.set_source(crystal.sin_source(sp.freq, m.dt, a.steps))
            sims.append(s)
        with Batch(len(sims), precision=a.precision, tile_j=a.tile_j, streams=a.batch_streams) as b:
            for s in sims:
                b.add(s, a.steps)
            b.step(a.steps)
            b.sync()
            ms = b.last_step_ms()
        nodes = sum(sp.n_nodes for sp in specs)
        for s in sims:
            s.close()
        print(json.dumps({"instances": a.batch, "batch_streams": a.batch_streams, "nodes": nodes, "steps": a.steps,
                          "ms": round(ms, 3),
                          "gcell_updates_per_s": round(nodes * a.steps / ms / 1e6, 3)}))
        return 0

    cells = tuple(int(c) for c in a.cells.split(","))
    xs = [int(v) for v in a.x_segments.split(",")] if a.x_segments else a.x_segment
    spec = crystal.CrystalSpec(cells=cells, lattice=16, radius=(0.2, 0.4), depth=10, tungsten_frac=0.25,
                               seed=a.seed, steps=a.steps)
    g, m = crystal.build(spec)
    t0 = time.perf_counter()
    with DeviceSimulation(g.spacing(), m.ids, m.table, m.dt, precision=a.precision, surface_mode="corrected",
                          max_steps=a.steps, record_every=10, tile_j=a.tile_j, x_segment=xs) as sim:
        sim.set_source(crystal.sin_source(spec.freq, m.dt, a.steps))
        sim.step(a.steps)
        sim.sync()
        ms = sim.last_step_ms()
        e = sim.energy()
    wall = time.perf_counter() - t0
    print(json.dumps({"cells": list(cells), "nodes": spec.n_nodes, "steps": a.steps, "precision": a.precision,
                      "ms": round(ms, 3), "gcell_updates_per_s": round(spec.n_nodes * a.steps / ms / 1e6, 3),
                      "wall_s": round(wall, 3), "energy": list(e)}))
    return 0


if __name__ == "__main__":
    sys.exit(main())
