"""Benchmark: Gcell-updates/s of the GB300 FDTD solver on the 256x256x128 crystal.

One bench step = one complete simulation of the seeded 256 x 256 x 128-cell
crystal (257*257*129 = 8,520,321 mesh nodes, 2000 time steps, lattice a=16,
radii U[0.2a, 0.4a], 25% tungsten, 42 MHz line source, uz surface recorded
every 10 steps) starting from the zero state, on the FP32 Kahan path (the
headline) with the plain FP64 path measured beside it on the same crystal.
Gcell-updates/s = mesh nodes x time steps / s (nodes = (cells+1)^3, the
reference's "points", tests/test_speed.py:52).

value: device time (CUDA events on the solver's stream) with all state
resident in HBM; the state (770 MB) is larger than L2.  e2e: wall time
through the public API with pinned host buffers: per step the material ids
and source go host->device and the surface records and final uz come back.

--impl reference times the reference algorithm on the host cores: the C
restatement of phonomena's NumPy solver (oracle/cpu_ref.c, FP64, bit-identical
to the reference), all host threads, a bounded number of time steps per step.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

GRAPH_CHUNK = 12
BYTES_PER_NODE = 73  # algorithmic: 3 components x (u, v, c) read + write x 4 B, + 1 B material id (FP64: u, u_old read, u_new write x 8 B + 1)


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="crystal", choices=["crystal", "batch", "serve", "precision"],
                   help="crystal: the 256x256x128 crystal (default); batch: 64 uneven crystals in one persistent "
                        "launch; serve: Poisson request stream; precision: 1024x1024x256 FP32K vs FP64 error")
    p.add_argument("--fdtd-steps", type=int, default=None)
    p.add_argument("--instances", type=int, default=64)
    p.add_argument("--batch-streams", type=int, default=64,
                   help="batch and serving: worker streams of the streams batch scheme (0: the persistent scheme only)")
    p.add_argument("--requests", type=int, default=2000, help="serve: FP32K requests")
    p.add_argument("--rate", type=float, default=0.0, help="serve: FP32K arrivals per second (0: 70%% load)")
    p.add_argument("--requests-f64", type=int, default=40, help="serve: plain FP64 requests")
    p.add_argument("--budget-gb", type=float, default=150.0, help="serve: device memory budget")
    p.add_argument("--cells", default="256,256,128")
    p.add_argument("--tile-j", type=int, default=0)
    p.add_argument("--x-segment", type=int, default=0)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--cpu-seconds", type=float, default=12.0)
    p.add_argument("--no-precision", action="store_true",
                   help="crystal: leave out the 1024x1024x256 FP32K-vs-FP64 error study (precision_config3)")
    p.add_argument("--precision-cells", default="1024,1024,256")
    p.add_argument("--precision-steps", type=int, default=4000)
    p.add_argument("--no-serve", action="store_true", help="crystal: leave out the served-latency streams (serve)")
    p.add_argument("--serve-requests", type=int, default=500, help="crystal: FP32K requests per served stream")
    p.add_argument("--serve-loads", default="0.7,0.9", help="crystal: FP32K offered loads (fractions of 45 Gcell/s)")
    p.add_argument("--serve-requests-f64", type=int, default=200, help="crystal: plain FP64 served requests")
    p.add_argument("--no-reference-numpy", action="store_true",
                   help="reference: leave out the timing of phonomena's own NumPy solvers")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("pci.bus_id,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, bus_id):
        self.bus = (bus_id or "").lower()[-12:]
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        return self

    def __exit__(self, *exc):
        if self.p is not None:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()

    def summary(self):
        self.f.flush()
        rows = []
        for line in open(self.f.name):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9 or (self.bus and not parts[0].lower().endswith(self.bus)):
                continue
            rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["clock sampling unavailable"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[q] for r in rows for q in range(4) if r[5 + q].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows),
                "power_w_max": max((float(r[3]) for r in rows if r[3].replace(".", "").isdigit()), default=None)}


def graph_launches(nsteps, separate_faces=True):
    """Kernels launched by phono_step(nsteps): per step the tile pass and the
    face pass, plus one step-counter update per 12-step graph and remainder."""
    per = 2 if separate_faces else 1
    full, rem = divmod(nsteps, GRAPH_CHUNK)
    return full * (per * GRAPH_CHUNK + 1) + per * rem + (1 if rem else 0)


def workload(cells, seed, fdtd_steps):
    from phonomena_gb300 import crystal

    spec = crystal.CrystalSpec(cells=cells, lattice=16, radius=(0.2, 0.4), depth=10, tungsten_frac=0.25,
                               seed=seed, steps=fdtd_steps)
    g, m = crystal.build(spec)
    src = crystal.sin_source(spec.freq, m.dt, fdtd_steps)
    return spec, g, m, src


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_per_node(kernel):
    """DRAM bytes per node-update of a kernel from the committed ncu summary."""
    p = ROOT / "profiles" / "traffic.json"
    if not p.exists():
        return None
    d = json.load(open(p))
    return d.get(kernel, {}).get("dram_bytes_per_node")


def traffic_bounds(scheme, nodes):
    """DRAM bytes per batch step bounded from the committed ncu summary where
    the scheme's traffic is not observable directly (streams: ncu serialises
    the side-by-side launches); None for the persistent scheme."""
    if scheme == "persistent":
        return None
    p = ROOT / "profiles" / "traffic.json"
    if not p.exists():
        return None
    b = json.load(open(p)).get("fdtd_step_kernel_f32k_batch", {}).get("bounds_bytes_per_node")
    return [round(v * nodes) for v in b] if b else None


def cpu_oracle_rate(cells, seconds, seed=0):
    """FP64 reference restatement on all host threads: (Gcell-updates/s, threads, steps)."""
    from oracle import cpu_oracle

    spec, g, m, src = workload(cells, seed, 4096)
    prob = cpu_oracle.OracleProblem(g.spacing(), m.ids, m.table, m.dt, src, surface_mode=1)
    st = cpu_oracle.F64State(prob)
    threads = cpu_oracle.max_threads()
    cpu_oracle.run_f64(prob, st, t0=0, nsteps=1)  # warm caches / page in
    done, t = 1, 0.0
    while t < seconds and done < 4000:
        t0 = time.perf_counter()
        cpu_oracle.run_f64(prob, st, t0=done, nsteps=2)
        t += time.perf_counter() - t0
        done += 2
    return spec.n_nodes * (done - 1) / t / 1e9, threads, done - 1, t


def reference_numpy(cases=(("config1", 500), ("config2", 20)), solvers=("default", "threading")):
    """phonomena's own NumPy solvers (the reference itself, from the
    baseline/_ref install) timed on this host: solver_default (NumPy
    elementwise, one core) and solver_threading (cfg num_threads = 6,
    solver_threading.py:10), FP64, writer off, through oracle/ref_harness.py.
    config1: the 40x40x20-cell void crystal for its full 500 steps; config2:
    the 256x256x128-cell crystal for 20 of its 2000 steps (a bounded sample;
    its per-node 6x6 C array alone is 2.45 GB).  Time = BaseSolver.run only
    (init, which fills C and P, is not timed)."""
    from oracle import ref_harness as H
    from phonomena_gb300 import crystal

    if not H.available():
        return {"unavailable": f"reference application not installed under {H.REF_ROOT}"}
    H.import_reference()
    mats = [dict(crystal.HOST), dict(crystal.VOID), dict(crystal.TUNGSTEN)]
    out = {"cpu_count": os.cpu_count(),
           "affinity": len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else None,
           "arithmetic": "FP64, the reference's own NumPy code (no FMA, reference op order)"}
    for name, steps in cases:
        spec = crystal.config1(seed=0) if name == "config1" else crystal.config2(seed=0)
        ids = crystal.material_ids(spec)
        g, m = H.make_uniform_case(spec.cells, 10e-6, mats, ids, c_max=0.5 / 10e-6, primary=0, secondary=2)
        for solver in solvers:
            R = H.import_reference()
            mod = {"default": R.solver_default, "threading": R.solver_threading}[solver]
            sv = mod.Solver()
            sv.cfg.update(write_mode="off", wave="sin", wave_args={"f": spec.freq})
            sv.init(g, m, steps)
            H._install_id_constants(sv.m, ids, [mm["name"] for mm in mats])
            sv.m.update()
            t0 = time.perf_counter()
            sv.run()
            el = time.perf_counter() - t0
            out[f"{name}_{solver}"] = {
                "value": round(spec.n_nodes * steps / el / 1e9, 6), "unit": "Gcell-updates/s",
                "seconds": round(el, 3), "time_steps": steps, "nodes": spec.n_nodes,
                "threads": 1 if solver == "default" else int(sv.cfg.get("num_threads", 6)),
                "sample": "full run" if name == "config1" else f"{steps} of the 2000 time steps"}
            del sv
    return out


def reference_arm(args, rank, world):
    if rank != 0:
        return
    cells = tuple(int(c) for c in args.cells.split(","))
    from oracle import cpu_oracle

    spec, g, m, src = workload(cells, 0, 4096)
    prob = cpu_oracle.OracleProblem(g.spacing(), m.ids, m.table, m.dt, src, surface_mode=1)
    st = cpu_oracle.F64State(prob)
    threads = cpu_oracle.max_threads()
    per_step = 4  # time steps of the 256^2 x 128 crystal per bench step (bounded sample)
    t_done = 0
    for _ in range(args.warmup):
        cpu_oracle.run_f64(prob, st, t0=t_done, nsteps=per_step)
        t_done += per_step
    t0 = time.perf_counter()
    for _ in range(args.steps):
        cpu_oracle.run_f64(prob, st, t0=t_done, nsteps=per_step)
        t_done += per_step
    el = time.perf_counter() - t0
    val = spec.n_nodes * per_step * args.steps / el / 1e9
    line = {
        "impl": "reference", "metric": "Gcell-updates/s", "value": round(val, 6), "unit": "Gcell-updates/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(el / args.steps * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"crystal {cells[0]}x{cells[1]}x{cells[2]} cells ({spec.n_nodes} nodes), "
                               f"{per_step} time steps per bench step (bounded sample of the 2000-step run)",
                   "parallelism": "host threads"},
        "cpu_baseline": {"value": round(val, 6), "unit": "Gcell-updates/s", "cores": threads, "kind": "port",
                         "sample": f"{per_step * args.steps} time steps of the {cells} crystal, FP64 reference "
                                   "arithmetic (oracle/cpu_ref.c, OpenMP)"},
        "e2e": {"value": round(val, 6), "unit": "Gcell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if not args.no_reference_numpy:
        try:
            line["reference_numpy"] = reference_numpy()
        except Exception as e:  # noqa: BLE001 - the port's value stands without it
            line["reference_numpy"] = {"error": f"{type(e).__name__}: {e}"[:500]}
    print(json.dumps(line), flush=True)


def bench_batch(args, rank, world, local, torch, dist):
    """64 uneven seeded crystals (sizes {64..192}^2 x {32..96} cells, a in
    {8,12,16}, f ~ U[20, 60] MHz), 1500 steps each, FP32 Kahan, with a
    graph-captured step loop, in both batch schemes: one persistent tile
    launch per time step, and every instance's own kernels on worker streams;
    tile height and per-instance x segments from the batch autotuner for
    each.  The faster scheme is the line's value.  One bench step = the whole
    batch from the zero state to its last step."""
    from phonomena_gb300 import autotune, crystal
    from phonomena_gb300.batch import Batch
    from phonomena_gb300.device import DeviceSimulation

    S = args.fdtd_steps or 1500
    specs = crystal.config4_specs(n=args.instances, seed=rank, steps=S)
    built = [crystal.build(sp) for sp in specs]
    shapes = [sp.nodes for sp in specs]
    node_sum = sum(sp.n_nodes for sp in specs)
    srcs = [crystal.sin_source(sp.freq, m.dt, S) for sp, (g, m) in zip(specs, built)]

    def make(prec, tj, segs):
        sims = []
        for (g, m), xs, src in zip(built, segs, srcs):
            sim = DeviceSimulation(g.spacing(), m.ids, m.table, m.dt, precision=prec, surface_mode="corrected",
                                   max_steps=S, record_every=10, tile_j=tj, x_segment=xs)
            sim.set_source(src)
            sims.append(sim)
        return sims

    def run_once(b, sims):
        for s in sims:
            s.reset()
        slots = [b.add(s, S) for s in sims]
        b.step(S)
        ms = b.last_step_ms()
        b.sync()
        for q in slots:
            b.remove(q)
        return ms

    schemes = {"persistent": 0}
    if args.batch_streams > 0:
        schemes["streams"] = args.batch_streams
    timed = {}
    bus = getattr(torch.cuda.get_device_properties(local), "pci_bus_id", "")
    for name, streams in schemes.items():
        tj, segs = autotune.tune_batch(shapes, "f32k", streams=streams)
        sims = make("f32k", tj, segs)
        batch = Batch(len(sims), precision="f32k", tile_j=tj, streams=streams)
        for _ in range(args.warmup):
            run_once(batch, sims)
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        with ClockSampler(bus) as clk:
            times = [run_once(batch, sims) for _ in range(args.steps)]
        ms = sum(times)
        if dist is not None:
            t = torch.tensor([ms], dtype=torch.float64, device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        timed[name] = dict(ms=ms, tj=tj, segs=segs, sims=sims, batch=batch, streams=streams, clocks=clk.summary(),
                           value=world * node_sum * S * args.steps / (ms / 1e3) / 1e9)
    scheme = min(timed, key=lambda k: timed[k]["ms"])
    for name, t in timed.items():
        if name != scheme:
            t["batch"].close()
            for s_ in t["sims"]:
                s_.close()
    best = timed[scheme]
    ms, tj, segs, sims, batch, clocks, value = (best[k] for k in ("ms", "tj", "segs", "sims", "batch", "clocks", "value"))
    surf32 = [s.read_surface().astype(np.float64) for s in sims]

    # the same instances one after another, each alone on its own handle
    seq_ms = 0.0
    for s in sims:
        s.reset()
        s.step(S)
        s.sync()
        seq_ms += s.last_step_ms()
    same = all(np.array_equal(s.read_surface().astype(np.float64), r) for s, r in zip(sims, surf32))

    # e2e: per bench step, materials and sources host->device, the batch run,
    # every instance's surface records device->host (pinned buffers)
    def pinned(shape, dtype):
        return torch.empty(shape, dtype=dtype, pin_memory=True).numpy()

    ids_h = [pinned(m.ids.shape, torch.uint8) for g, m in built]
    src_h = [pinned((S,), torch.float64) for _ in built]
    surf_h = [pinned((S // 10, sh[0], sh[1]), torch.float32) for sh in shapes]
    for (g, m), a, b_, src in zip(built, ids_h, src_h, srcs):
        a[...] = m.ids
        b_[...] = src
    h2d = sum(a.nbytes + b_.nbytes + m.table.nbytes for a, b_, (g, m) in zip(ids_h, src_h, built))
    d2h = sum(x.nbytes for x in surf_h)

    def e2e_once():
        for s, a, b_, (g, m) in zip(sims, ids_h, src_h, built):
            s.set_materials(a, m.table)
            s.set_source(b_)
            s.reset()
        slots = [batch.add(s, S) for s in sims]
        batch.step(S)
        batch.sync()
        for s, out in zip(sims, surf_h):
            s.read_surface(0, S // 10, out=out)
        for q in slots:
            batch.remove(q)

    e2e_once()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_once()
    wall = time.perf_counter() - t0
    e2e = world * node_sum * S * args.steps / wall / 1e9
    batch.close()
    for s in sims:
        s.close()

    # plain FP64 batch of the same instances, one run in two halves: throughput,
    # error, and the energy growth that marks an instance whose reference
    # scheme is unstable (exponential growth amplifies every rounding
    # difference, so its FP32/FP64 difference says nothing about FP32)
    tj64, segs64 = autotune.tune_batch(shapes, "f64", steps=4, tile_js=(8, 16), streams=best["streams"])
    sims64 = make("f64", tj64, segs64)
    b64 = Batch(len(sims64), precision="f64", tile_j=tj64, streams=best["streams"])
    slots = [b64.add(s, S) for s in sims64]
    half = S // 2
    b64.step(half)
    ms64 = b64.last_step_ms()
    b64.sync()
    e_half = [sum(s.energy()) for s in sims64]
    b64.step(S - half)
    ms64 += b64.last_step_ms()
    b64.sync()
    e_end = [sum(s.energy()) for s in sims64]
    errs, growing = [], []
    for q, (s, r) in enumerate(zip(sims64, surf32)):
        ref = s.read_surface()
        errs.append(float(np.linalg.norm(r - ref) / np.linalg.norm(ref)))
        if e_end[q] > 16.0 * e_half[q]:
            growing.append(q)
    stable = [e for q, e in enumerate(errs) if q not in growing]
    b64.close()
    for s in sims64:
        s.close()

    launch_ms = ms / (args.steps * S)
    hbm_peak, peak_kind = measured_peaks()
    achieved = BYTES_PER_NODE * node_sum / (launch_ms / 1e3) / 1e9
    tpn = traffic_per_node("batch_step_kernel_f32k" if scheme == "persistent" else "fdtd_step_kernel_f32k_batch")
    if rank == 0:
        line = {
            "metric": "Gcell-updates/s", "value": round(value, 4), "unit": "Gcell-updates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded crystals)",
            "config": {"workload": f"batch of {len(specs)} uneven crystals ({node_sum} nodes in all), {S} time steps "
                                   f"each, {scheme} batch scheme, graph-captured step loop, FP32 Kahan",
                       "instances": len(specs), "nodes": node_sum, "fdtd_steps": S, "scheme": scheme,
                       "worker_streams": best["streams"], "tile_j": tj, "x_segment_by_instance": segs,
                       "l2": f"inputs larger than L2 (state {node_sum * 72 / 1e9:.1f} GB)",
                       "parallelism": f"replicas x{world}"},
            "schemes": {k: {"value": round(t["value"], 4), "unit": "Gcell-updates/s",
                            "ms_per_step": round(t["ms"] / args.steps, 3), "tile_j": t["tj"],
                            "x_segments": sorted(set(map(str, t["segs"])))} for k, t in timed.items()},
            "sequential": {"value": round(world * node_sum * S / (seq_ms / 1e3) / 1e9, 4), "unit": "Gcell-updates/s",
                           "ms": round(seq_ms, 3), "speedup_batch_over_sequential":
                               round(seq_ms / (ms / args.steps), 3), "bit_identical_to_batch": bool(same)},
            "fp64": {"value": round(world * node_sum * S / (ms64 / 1e3) / 1e9, 4), "unit": "Gcell-updates/s",
                     "ms": round(ms64, 3), "speedup_f32k_over_f64": round(ms64 / (ms / args.steps), 3),
                     "tile_j": tj64},
            "error_vs_fp64": {"rel_l2_surface_uz_max": max(errs), "rel_l2_surface_uz_median": float(np.median(errs)),
                              "fdtd_steps": S, "instances_with_energy_growth": growing,
                              "energy_growth_rule": f"energy after {S} steps > 16x energy after {half} steps (FP64; "
                                                    "a steady drive gives about 2x, a resonance 4x)",
                              "energy_ratio_by_instance": [round(e / h, 2) if h > 0 else None
                                                           for e, h in zip(e_end, e_half)],
                              "rel_l2_surface_uz_max_without_growth": max(stable) if stable else None,
                              "rel_l2_surface_uz_median_without_growth": float(np.median(stable)) if stable else None},
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm_peak, "unit": "GB/s",
                         "frac": round(achieved / hbm_peak, 4), "peak_kind": peak_kind,
                         "traffic": (round(tpn * node_sum) if tpn else None),
                         "traffic_bounds_per_launch": traffic_bounds(scheme, node_sum),
                         "algorithmic_bytes_per_launch": BYTES_PER_NODE * node_sum,
                         "avg_launch_ms": round(launch_ms, 5),
                         "launch_timing": ("one time step = persistent tile launch + batched face launch "
                                           "(+1/12 counter update)" if scheme == "persistent" else
                                           "one time step = every instance's tile and face launches on the worker "
                                           "streams (+1/12 counter update)")
                                          + "; the whole step is charged to the stencil kernel"},
            "cpu_baseline": None,
            "e2e": {"value": round(e2e, 4), "unit": "Gcell-updates/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h)},
            "gpu_launches": (graph_launches(S, True) if scheme == "persistent"
                             else len(specs) * 2 * S + -(-S // GRAPH_CHUNK)) * args.steps,
            "clocks": clocks,
        }
        print(json.dumps(line), flush=True)


SERVE_GCELL = {"f32k": 45.0, "f64": 4.0}  # batched throughputs the offered loads refer to


def serve_stream(precision, n, rate, seed, budget_gb, streams=0):
    """One Poisson stream of crystal-simulation requests (config-4 size mix
    plus 5% 512x512x128-cell jobs, 500-3000 steps each, surface uz every 10
    steps) served by continuous batching under a device-memory budget:
    latency percentiles, served throughput and admission statistics."""
    from phonomena_gb300 import serve

    reqs = serve.poisson_stream(n, rate, seed=seed)
    be = serve.GpuBackend(precision=precision, capacity=256, max_steps=3000, streams=streams)
    srv = serve.Server(be, budget_bytes=budget_gb * 1e9, capacity=256, chunk=60)
    streamed = []
    srv.on_result = lambda r: streamed.append(r.surface.nbytes)
    t0 = time.perf_counter()
    res = srv.run(reqs, realtime=True)
    wall = time.perf_counter() - t0
    srv.close()
    be.close()
    out = serve.summarize(res)
    out.update({"rate_per_s": round(rate, 4), "offered_gcell_per_s": round(rate * serve.mean_work() / 1e9, 3),
                "wall_s": round(wall, 2), "peak_resident_gb": round(srv.stats.peak_bytes / 1e9, 2),
                "peak_active": srv.stats.peak_active, "chunks": srv.stats.chunks,
                "rejected": len(srv.stats.rejected), "streamed_surface_bytes": int(sum(streamed))})
    return out


def serve_summary(r, load):
    """The served-stream figures of the benchmark line."""
    return {"load": load, "rate": r["rate_per_s"], "requests": r["requests"], "p50": round(r["p50_s"], 4),
            "p95": round(r["p95_s"], 4), "p99": round(r["p99_s"], 4),
            "gcell_per_s": round(r["gcell_updates_per_s"], 4), "offered_gcell_per_s": r["offered_gcell_per_s"],
            "failed": r["failed"], "rejected": r["rejected"], "peak_active": r["peak_active"],
            "peak_resident_gb": r["peak_resident_gb"], "wall_s": r["wall_s"]}


def bench_serve(args, rank, world, local, torch, dist):
    """FP32K and plain FP64 request streams, each at about 70% of its own
    batched throughput (serve_stream)."""
    from phonomena_gb300 import serve

    rate32 = args.rate or serve.rate_for_load(SERVE_GCELL["f32k"], 0.7)
    rate64 = rate32 * SERVE_GCELL["f64"] / SERVE_GCELL["f32k"]
    bus = getattr(torch.cuda.get_device_properties(local), "pci_bus_id", "")
    with ClockSampler(bus) as clk:
        r32 = serve_stream("f32k", args.requests, rate32, rank, args.budget_gb, streams=args.batch_streams)
    clocks = clk.summary()
    r64 = serve_stream("f64", args.requests_f64, rate64, rank + 1000, args.budget_gb, streams=args.batch_streams)
    if rank == 0:
        line = {
            "metric": "served Gcell-updates/s", "value": round(r32["gcell_updates_per_s"], 4),
            "unit": "Gcell-updates/s", "n_gpus": world, "steps": 1, "warmup": 0,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded request stream)",
            "config": {"workload": f"Poisson stream of {args.requests} requests at {rate32:.3f}/s (70% of "
                                   f"{SERVE_GCELL['f32k']} Gcell/s offered), sizes {{64..192}}^2 x {{32..96}} cells "
                                   "plus 5% 512x512x128, 500-3000 steps, uz surface every 10 steps, "
                                   f"{args.budget_gb:.0f} GB device budget, continuous batching",
                       "parallelism": f"replicas x{world}"},
            "latency_s": {"p50": round(r32["p50_s"], 4), "p95": round(r32["p95_s"], 4), "p99": round(r32["p99_s"], 4)},
            "f32k": r32, "fp64": r64, "clocks": clocks,
        }
        print(json.dumps(line), flush=True)


def serve_study(args, rank):
    """The serve object of the default line: FP32K streams at the offered
    loads of --serve-loads, a plain FP64 stream at 70% of its throughput."""
    from phonomena_gb300 import serve

    loads = [float(v) for v in args.serve_loads.split(",") if v]
    out = {"workload": "Poisson request streams: sizes {64..192}^2 x {32..96} cells plus 5% 512x512x128, "
                       "500-3000 steps, uz surface every 10 steps, continuous batching, "
                       f"{args.budget_gb:.0f} GB device budget; load = offered work / the scheme's batched "
                       f"throughput ({SERVE_GCELL['f32k']} Gcell/s FP32K, {SERVE_GCELL['f64']} FP64)",
           "f32k": [], "fp64": []}
    for q, load in enumerate(loads):
        rate = serve.rate_for_load(SERVE_GCELL["f32k"], load)
        out["f32k"].append(serve_summary(serve_stream("f32k", args.serve_requests, rate, rank + 10 * q,
                                                      args.budget_gb, streams=args.batch_streams), load))
    rate64 = serve.rate_for_load(SERVE_GCELL["f64"], 0.7)
    out["fp64"].append(serve_summary(serve_stream("f64", args.serve_requests_f64, rate64, rank + 1000,
                                                  args.budget_gb, streams=args.batch_streams), 0.7))
    out["batch_scheme"] = "streams" if args.batch_streams > 0 else "persistent"
    return out


def precision_study(cells, S, seed, torch):
    """Seeded crystal of the config-2 recipe on a cells grid, S steps: FP32
    fields with Kahan-compensated u against the plain FP64 path (the
    reference arithmetic) on the same inputs; relative L2 error of surface
    uz and relative error of the total energy after S/4, S/2 and S steps, and
    the device throughput of both runs."""
    from phonomena_gb300 import autotune
    from phonomena_gb300.device import DeviceSimulation

    marks = [m for m in (S // 4, S // 2, S) if m > 0]
    spec, g, m, src = workload(cells, seed, S)
    sp = g.spacing()
    every = S // 4

    def run(prec):
        tj, xs = autotune.tune(sp, m.ids, m.table, m.dt, precision=prec,
                               candidates=None if prec == "f32k" else [(8, 32), (16, 32)])
        sim = DeviceSimulation(sp, m.ids, m.table, m.dt, precision=prec, surface_mode="corrected", max_steps=S,
                               record_every=every, tile_j=tj, x_segment=xs)
        sim.set_source(src)
        stream = torch.cuda.ExternalStream(sim.stream_ptr)
        energy, ms, done = {}, 0.0, 0
        for mk in marks:
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            sim.step(mk - done)
            e1.record(stream)
            e1.synchronize()
            ms += e0.elapsed_time(e1)
            done = mk
            energy[mk] = sum(sim.energy())
        sim.sync()
        surf = sim.read_surface()
        sim.close()
        return {"ms": ms, "energy": energy, "surf": surf, "tile": [tj, xs]}

    r32 = run("f32k")
    r64 = run("f64")
    per = {}
    for mk in marks:
        rec = mk // every - 1
        a, b = r32["surf"][rec].astype(np.float64), r64["surf"][rec]
        per[str(mk)] = {"rel_l2_surface_uz": float(np.linalg.norm(a - b) / np.linalg.norm(b)),
                        "rel_energy": float(abs(r32["energy"][mk] - r64["energy"][mk]) / abs(r64["energy"][mk])),
                        "energy_f64": r64["energy"][mk]}
    nodes = spec.n_nodes
    v32 = nodes * S / (r32["ms"] / 1e3) / 1e9
    v64 = nodes * S / (r64["ms"] / 1e3) / 1e9
    worst = max(max(v["rel_l2_surface_uz"], v["rel_energy"]) for v in per.values())
    return {"workload": f"crystal {cells[0]}x{cells[1]}x{cells[2]} cells ({nodes} nodes), {S} time steps, "
                        "FP32K vs plain FP64 on the same inputs (config-2 recipe, seed 0)",
            "nodes": nodes, "fdtd_steps": S, "errors_at_step": per, "max_error": worst, "tolerance": 1e-5,
            "within_tolerance": bool(worst <= 1e-5),
            "f32k": {"value": round(v32, 4), "unit": "Gcell-updates/s", "ms": round(r32["ms"], 1),
                     "tile": r32["tile"]},
            "fp64": {"value": round(v64, 4), "unit": "Gcell-updates/s", "ms": round(r64["ms"], 1),
                     "tile": r64["tile"]},
            "speedup_f32k_over_f64": round(v32 / v64, 3)}


def bench_precision(args, rank, world, local, torch, dist):
    """The precision study (precision_study) as its own benchmark line."""
    cells = (1024, 1024, 256) if args.cells == "256,256,128" else tuple(int(c) for c in args.cells.split(","))
    S = args.fdtd_steps or 4000
    r = precision_study(cells, S, rank, torch)
    if rank == 0:
        line = {"metric": "rel L2 error FP32K vs FP64",
                "value": max(v["rel_l2_surface_uz"] for v in r["errors_at_step"].values()),
                "unit": "relative L2", "higher_is_better": False, "n_gpus": world, "steps": 1, "warmup": 0,
                "dtype": "f32", "data": "synthetic (seeded crystal)",
                "config": {"workload": r["workload"], "nodes": r["nodes"]},
                "errors_at_step": r["errors_at_step"], "f32k": r["f32k"], "fp64": r["fp64"],
                "speedup_f32k_over_f64": r["speedup_f32k_over_f64"]}
        print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        reference_arm(args, rank, world)
        return
    import torch

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import __graft_entry__

    __graft_entry__.build()
    if args.workload != "crystal":
        {"batch": bench_batch, "serve": bench_serve, "precision": bench_precision}[args.workload](
            args, rank, world, local, torch, dist)
        if dist is not None:
            dist.destroy_process_group()
        return
    from phonomena_gb300.device import DeviceSimulation

    cells = tuple(int(c) for c in args.cells.split(","))
    S = args.fdtd_steps or 2000
    spec, g, m, src = workload(cells, rank, S)
    nodes = spec.n_nodes
    sp = g.spacing()
    # tile shapes: the project autotuner (untimed, cached per mesh and device)
    shapes = {}
    for prec in ("f32k", "f64v", "f64"):
        if args.tile_j:
            shapes[prec] = (args.tile_j, args.x_segment)
        else:
            from phonomena_gb300 import autotune

            cands = None if prec == "f32k" else [(tj, xs) for tj in (8, 16) for xs in (24, 32, 40)]
            shapes[prec] = autotune.tune(sp, m.ids, m.table, m.dt, precision=prec, candidates=cands)

    def kw(prec):
        return dict(surface_mode="corrected", max_steps=S, record_every=10, tile_j=shapes[prec][0],
                    x_segment=shapes[prec][1])

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    def max_over_ranks(x):
        from phonomena_gb300 import replicas

        return replicas.aggregate(x, 0.0, dist)[0]

    # ---- FP32 Kahan: device-resident throughput ----
    sim = DeviceSimulation(sp, m.ids, m.table, m.dt, precision="f32k", **kw("f32k"))
    separate_faces = g.y.size >= 4
    sim.set_source(src)
    stream = torch.cuda.ExternalStream(sim.stream_ptr)
    for _ in range(args.warmup):
        sim.reset()
        sim.step(S)
    sim.sync()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    bus = torch.cuda.get_device_properties(local).pci_bus_id if hasattr(torch.cuda.get_device_properties(local),
                                                                         "pci_bus_id") else ""
    with ClockSampler(bus) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            sim.reset()
            sim.step(S)
        e1.record(stream)
        e1.synchronize()
    sim.sync()
    ms = max_over_ranks(e0.elapsed_time(e1))
    barrier()
    clocks = clk.summary()
    value = world * nodes * S * args.steps / (ms / 1e3) / 1e9
    surf32 = sim.read_surface().astype(np.float64)
    u32 = [sim.download(k).astype(np.float64) for k in ("ux", "uy", "uz")]
    e32 = sim.energy()
    step_ms = ms / (args.steps * S)
    # the stencil kernel alone: CUDA events around each tile launch (and
    # apart, each face launch) of KT steps, launched back to back
    KT = min(240, S)
    sim.reset()
    tile_ms, face_ms = sim.time_kernels(KT)
    sim.sync()
    launch_ms = tile_ms / KT
    hbm_peak, peak_kind = measured_peaks()
    achieved = BYTES_PER_NODE * nodes / (launch_ms / 1e3) / 1e9
    step_achieved = BYTES_PER_NODE * nodes / (step_ms / 1e3) / 1e9
    tpn = traffic_per_node("fdtd_step_kernel_f32k")

    # ---- FP64 on the same crystal, one full run each: the reference
    # arithmetic (plain FP64 path, bit-identical to phonomena) and the FP64
    # velocity form (the same scheme as the FP32 path) ----
    def run_fp64(prec):
        s = DeviceSimulation(sp, m.ids, m.table, m.dt, precision=prec, **kw(prec))
        s.set_source(src)
        st = torch.cuda.ExternalStream(s.stream_ptr)
        s.step(GRAPH_CHUNK)
        s.sync()
        s.reset()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(st)
        s.step(S)
        f1.record(st)
        f1.synchronize()
        s.sync()
        t = max_over_ranks(f0.elapsed_time(f1))
        out = (t, world * nodes * S / (t / 1e3) / 1e9, s.read_surface(),
               [s.download(k) for k in ("ux", "uy", "uz")], s.energy())
        s.close()
        return out

    def errors(ref):
        _, _, surf64, u64, e64 = ref
        return {"rel_l2_surface_uz": float(np.linalg.norm(surf32 - surf64) / np.linalg.norm(surf64)),
                "rel_l2_u": float(math.sqrt(sum(np.linalg.norm(a - b) ** 2 for a, b in zip(u32, u64)))
                                  / math.sqrt(sum(np.linalg.norm(b) ** 2 for b in u64))),
                "rel_energy": float(abs(sum(e32) - sum(e64)) / abs(sum(e64))), "fdtd_steps": S}

    r64 = run_fp64("f64")
    r64v = run_fp64("f64v")
    ms64, value64 = r64[0], r64[1]

    # ---- e2e through the public API with pinned host buffers ----
    def pinned(shape, dtype):
        t = torch.empty(shape, dtype=dtype, pin_memory=True)
        return t.numpy()

    ids_h = pinned(m.ids.shape, torch.uint8)
    ids_h[...] = m.ids
    src_h = pinned(src.shape, torch.float64)
    src_h[...] = src
    nrec = S // 10
    surf_h = pinned((nrec, g.x.size, g.y.size), torch.float32)
    uz_h = pinned((g.x.size, g.y.size, g.z.size - 1), torch.float32)
    h2d = ids_h.nbytes + m.table.nbytes + src_h.nbytes
    d2h = surf_h.nbytes + uz_h.nbytes
    for _ in range(max(1, min(args.warmup, 2))):
        sim.set_materials(ids_h, m.table)
        sim.set_source(src_h)
        sim.reset()
        sim.step(S)
        sim.read_surface(0, nrec, out=surf_h)
        sim.download("uz", out=uz_h)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        sim.set_materials(ids_h, m.table)
        sim.set_source(src_h)
        sim.reset()
        sim.step(S)
        sim.read_surface(0, nrec, out=surf_h)
        sim.download("uz", out=uz_h)
    sim.sync()
    wall = max_over_ranks(time.perf_counter() - t0)
    e2e = world * nodes * S * args.steps / wall / 1e9
    sim.close()

    # ---- the untimed studies of the line: config-3 error table, served latency ----
    # a failure inside a study is reported in the line instead of losing it
    def study(fn, *a):
        try:
            return fn(*a)
        except Exception as e:  # noqa: BLE001
            try:
                torch.cuda.synchronize()
            except Exception:  # noqa: BLE001
                pass
            return {"error": f"{type(e).__name__}: {e}"[:500]}

    prec3 = None
    if not args.no_precision:
        pc = tuple(int(c) for c in args.precision_cells.split(","))
        prec3 = study(precision_study, pc, args.precision_steps, rank, torch)
    served = None if args.no_serve else study(serve_study, args, rank)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        rate, threads, nst, secs = cpu_oracle_rate(cells, args.cpu_seconds)
        cpu = {"value": round(rate, 6), "unit": "Gcell-updates/s", "cores": threads, "kind": "port",
               "sample": f"{nst} time steps of the same crystal in {secs:.1f} s, FP64 reference arithmetic "
                         "(oracle/cpu_ref.c, OpenMP, bit-identical to phonomena's solver_default)"}

    if rank == 0:
        line = {
            "metric": "Gcell-updates/s", "value": round(value, 4), "unit": "Gcell-updates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded crystal, one per rank)",
            "config": {"workload": f"crystal {cells[0]}x{cells[1]}x{cells[2]} cells ({nodes} nodes), {S} time steps "
                                   "per bench step from the zero state, FP32 velocity form with Kahan-compensated u, "
                                   "corrected z=0 row, absorbing walls, uz surface every 10 steps",
                       "nodes": nodes, "fdtd_steps": S, "l2": "inputs larger than L2 (state 770 MB)",
                       "parallelism": f"replicas x{world}"},
            "fp64": {"value": round(value64, 4), "unit": "Gcell-updates/s", "fdtd_steps": S,
                     "ms": round(ms64, 3), "speedup_f32k_over_f64": round(value / value64, 3),
                     "arithmetic": "reference leapfrog, IEEE quotients (divisor table), bit-identical to phonomena",
                     "tile": list(shapes["f64"])},
            "fp64_velocity_form": {"value": round(r64v[1], 4), "unit": "Gcell-updates/s", "ms": round(r64v[0], 3),
                                   "speedup_f32k_over_f64v": round(value / r64v[1], 3),
                                   "tile": list(shapes["f64v"])},
            "error_vs_fp64": errors(r64),
            "error_vs_fp64_velocity_form": errors(r64v),
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm_peak, "unit": "GB/s",
                         "frac": round(achieved / hbm_peak, 4), "peak_kind": peak_kind,
                         "traffic": (round(tpn * nodes) if tpn else None),
                         "algorithmic_bytes_per_launch": BYTES_PER_NODE * nodes,
                         "avg_launch_ms": round(launch_ms, 5),
                         "launch_timing": f"fdtd_step_kernel<F32K> alone: CUDA events on the solver's stream around "
                                          f"each tile launch of {KT} back-to-back steps (phono_time_kernels)",
                         "face_launch_ms": round(face_ms / KT, 5),
                         "whole_step": {"ms": round(step_ms, 5), "achieved": round(step_achieved, 1),
                                        "frac": round(step_achieved / hbm_peak, 4),
                                        "note": "graph-replayed step of the timed region: tile + face launch "
                                                "(+1/12 counter update), all charged to the stencil"}},
            "tile": list(shapes["f32k"]),
            "cpu_baseline": cpu,
            "e2e": {"value": round(e2e, 4), "unit": "Gcell-updates/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h)},
            "gpu_launches": graph_launches(S, separate_faces) * args.steps,
            "clocks": clocks,
            "precision_config3": prec3,
            "serve": served,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
