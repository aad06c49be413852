"""Continuous-batching request loop for crystal simulations.

Requests (a crystal to build, a step count, a surface-record interval) arrive
over time.  One loop thread owns the GPU work: it admits waiting requests
while a batch slot is free and their device footprint fits the memory budget,
uploads their materials and source into device-resident simulations, steps
every admitted simulation together in chunks of time steps (one persistent
launch per step for the whole mix, ``phonomena_gb300.batch``), and at each
chunk boundary streams out the surface traces of the requests that finished
and frees their memory for the next ones.  Requests that arrive while others
are on the GPU join the running batch at the next chunk boundary; each
instance keeps its own step counter and budget, so its result does not
depend on what else is in the mix.

Host-side preparation (material ids, source samples) runs on a small thread
pool as requests arrive, so the loop thread only uploads and steps.

The reference runs one simulation per solver object to completion
(simulation/base_solver.py:224-280) and has no request loop; the per-request
result here is that of ``DeviceSimulation.step`` on the same inputs, bit for
bit.

Backends: ``GpuBackend`` (the C ABI) and any object with the same methods
(the CPU tests drive the scheduler with a fake backend).
"""
from __future__ import annotations

import hashlib

import heapq
import queue
import threading
import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Request:
    rid: int
    spec: object                 # crystal.CrystalSpec (cells, lattice, radii, seed, freq, steps)
    steps: int
    arrival: float = 0.0         # seconds after the stream start
    record_every: int = 10


@dataclass
class Result:
    rid: int
    nodes: int
    steps: int
    arrival: float
    admitted: float
    finished: float
    surface: np.ndarray          # (steps // record_every, nx, ny) uz at z = 0
    error: str = None            # set when the run stopped early (non-finite values)

    @property
    def latency(self):
        return self.finished - self.arrival

    @property
    def wait(self):
        return self.admitted - self.arrival


@dataclass
class Prepared:
    """Host inputs of a request, built off the loop thread."""
    req: Request
    shape: tuple
    spacing: dict
    ids: np.ndarray
    table: np.ndarray
    dt: float
    source: np.ndarray


def prepare(req: Request) -> Prepared:
    from . import crystal

    g, m = crystal.build(req.spec)
    src = crystal.sin_source(req.spec.freq, m.dt, req.steps)
    return Prepared(req, req.spec.nodes, g.spacing(), m.ids, m.table, m.dt, src)


class GpuBackend:
    """Device simulations and one batch behind the C ABI.

    Finished simulations are kept (zeroed, not freed) in a pool keyed by mesh
    shape and record layout, and reused for the next request of that key:
    no cudaMalloc / cudaFree (a device synchronisation) on the serving path
    once the pool is warm.  Every simulation is created with room for
    ``max_steps`` steps so that requests of any length share a key.
    """

    def __init__(self, precision="f32k", capacity=128, tile_j=16, x_segment=0, max_steps=3000, streams=0):
        from .batch import Batch

        self.precision = precision
        self.tile_j = tile_j
        self.x_segment = x_segment
        self.max_steps = int(max_steps)
        self.batch = Batch(capacity, precision=precision, tile_j=tile_j, streams=streams)
        self.pool = {}  # key -> [DeviceSimulation], least recently used first
        self._lru = []  # keys of pooled simulations, least recently used first

    def key(self, p: Prepared):
        """Pool key: what a simulation keeps across requests (mesh, spacing,
        time step, record layout); materials and source are replaced.  The
        spacings enter as the SHA-256 digest of their bytes: two meshes share
        a key only when every spacing value is the same (a pooled handle keeps
        its spacings and divisor table, so a collision would change results)."""
        h = hashlib.sha256()
        for k in ("fdx", "fdy", "fdz", "sdx", "sdy", "sdz"):
            h.update(np.ascontiguousarray(p.spacing[k], np.float64).tobytes())
        return (tuple(int(v) for v in p.shape), max(self.max_steps, int(p.req.steps)), int(p.req.record_every),
                float(p.dt), h.hexdigest())

    def footprint(self, shape, steps, record_every):
        from .device import footprint

        return footprint(shape, self.precision, max(self.max_steps, int(steps)), record_every)

    def _key_bytes(self, k):
        return self.footprint(k[0], k[1], k[2])

    def has_pooled(self, key):
        return bool(self.pool.get(key))

    def evict_one(self, keep=None):
        """Free the least recently pooled simulation (not of key `keep`);
        returns its footprint, or 0 if there is none."""
        for q, k in enumerate(self._lru):
            if k == keep:
                continue
            sim = self.pool[k].pop(0)
            del self._lru[q]
            sim.close()
            return self._key_bytes(k)
        return 0

    def admit(self, p: Prepared):
        from .device import DeviceSimulation

        k = self.key(p)
        if self.pool.get(k):
            sim = self.pool[k].pop()
            self._lru.reverse()
            self._lru.remove(k)  # the most recent entry of this key
            self._lru.reverse()
            sim.set_materials(p.ids, p.table)
        else:
            sim = DeviceSimulation(p.spacing, p.ids, p.table, p.dt, precision=self.precision,
                                   surface_mode="corrected", max_steps=k[1], record_every=k[2], tile_j=self.tile_j,
                                   x_segment=self.x_segment or _x_segment(p.shape[0]))
        sim.set_source(p.source)
        sim.pool_key = k
        slot = self.batch.add(sim, p.req.steps)
        return slot, sim

    def step(self, nsteps):
        self.batch.step(nsteps)

    def sync(self):
        """Wait for the batch; returns the slots whose simulation reported
        non-finite values (its own error flag; the others are unaffected)."""
        from ._lib import PhonoError

        try:
            self.batch.sync()
            return []
        except PhonoError as e:
            if e.code != -5:
                raise
        bad = []
        for slot, sim in self.batch.members.items():
            try:
                sim.sync()
            except PhonoError as e:
                if e.code != -5:
                    raise
                bad.append(slot)
        return bad

    def remaining(self, slot):
        return self.batch.remaining(slot)

    def finish(self, slot, sim):
        """Surface records of a finished instance; the simulation goes back to the pool."""
        self.batch.remove(slot)
        out = sim.read_surface()
        sim.reset()
        k = sim.pool_key
        self.pool.setdefault(k, []).append(sim)
        self._lru.append(k)
        return out

    def pooled_bytes(self):
        return sum(self._key_bytes(k) for k in self._lru)

    def close(self):
        self.batch.close()
        for sims in self.pool.values():
            for sim in sims:
                sim.close()
        self.pool.clear()
        self._lru.clear()


def _x_segment(nx):
    """Default x segment: about 32 planes, evened out over the x extent."""
    nseg = max(1, round((nx - 1) / 32))
    return -(-(nx - 1) // nseg)


@dataclass
class ServerStats:
    results: list = field(default_factory=list)
    peak_bytes: int = 0
    peak_active: int = 0
    chunks: int = 0
    rejected: list = field(default_factory=list)


class Server:
    """Continuous batching under a device-memory budget.

    budget_bytes: device memory the resident simulations may hold together.
    capacity: batch slots.  chunk: time steps between admission points.
    on_result(Result) is called on the loop thread as each request finishes
    (the streamed surface trace).
    """

    def __init__(self, backend, budget_bytes=150e9, capacity=128, chunk=60, prepare_fn=prepare, workers=4,
                 on_result=None, clock=time.perf_counter):
        self.backend = backend
        self.budget = int(budget_bytes)
        self.capacity = int(capacity)
        self.chunk = int(chunk)
        self.prepare_fn = prepare_fn
        self.pool = ThreadPoolExecutor(max_workers=workers)
        self.on_result = on_result
        self.clock = clock
        self.inbox = queue.Queue()
        self.stats = ServerStats()
        self._stop = False
        self._t0 = None

    # -- client side -----------------------------------------------------
    def submit(self, req: Request):
        """Hand a request to the loop (thread-safe); preparation starts now."""
        self.inbox.put((req, self.pool.submit(self.prepare_fn, req)))

    def close(self):
        self._stop = True
        self.pool.shutdown(wait=True)

    # -- the loop ----------------------------------------------------------
    def now(self):
        return self.clock() - self._t0

    def run(self, requests, realtime=True):
        """Serve a whole request stream (arrival times relative to now) and
        return the results in completion order.  realtime=False submits every
        request at once (arrival times are then only used for latency)."""
        self._t0 = self.clock()
        stream = sorted(requests, key=lambda r: (r.arrival, r.rid))
        feeder = None
        if realtime:
            feeder = threading.Thread(target=self._feed, args=(stream,), daemon=True)
            feeder.start()
        else:
            for r in stream:
                self.submit(r)
        self.serve(len(stream))
        if feeder is not None:
            feeder.join()
        return self.stats.results

    def _feed(self, stream):
        for r in stream:
            dt = r.arrival - self.now()
            if dt > 0:
                time.sleep(dt)
            self.submit(r)

    def serve(self, n_expected):
        waiting = []  # FIFO of (arrival, rid, request, future)
        active = {}   # slot -> (request, sim, admitted time, footprint)
        used = 0
        done = 0
        while done < n_expected and not self._stop:
            # collect arrivals (block briefly only when there is nothing to step)
            block = not active and not waiting
            try:
                while True:
                    req, fut = self.inbox.get(block=block, timeout=0.05 if block else None)
                    heapq.heappush(waiting, (req.arrival, req.rid, req, fut))
                    block = False
            except queue.Empty:
                pass
            # admission: FIFO, as long as a slot and the memory budget allow;
            # `used` counts active and pooled simulations
            while waiting and len(active) < self.capacity:
                arrival, rid, req, fut = waiting[0]
                need = self.backend.footprint(req.spec.nodes, req.steps, req.record_every)
                if need > self.budget:
                    heapq.heappop(waiting)
                    self.stats.rejected.append(rid)
                    done += 1
                    continue
                if not fut.done() and active:
                    break  # inputs still being built: step the others meanwhile
                prep = fut.result()
                key = self.backend.key(prep)
                extra = 0 if self.backend.has_pooled(key) else need
                while used + extra > self.budget:
                    freed = self.backend.evict_one(keep=key)
                    if not freed:
                        break
                    used -= freed
                if used + extra > self.budget:
                    break
                heapq.heappop(waiting)
                slot, sim = self.backend.admit(prep)
                active[slot] = (req, sim, self.now(), need)
                used += extra
            self.stats.peak_bytes = max(self.stats.peak_bytes, used)
            self.stats.peak_active = max(self.stats.peak_active, len(active))
            if not active:
                continue
            # step the mix up to the next finish or the chunk length
            n = min(self.chunk, min(self.backend.remaining(s) for s in active))
            n = max(n, 1)
            self.backend.step(n)
            self.stats.chunks += 1
            finished = [s for s in active if self.backend.remaining(s) == 0]
            if finished:
                failed = set(self.backend.sync())
                t = self.now()
                # a simulation that produced non-finite values ends now, with
                # the records it has; the rest of the mix goes on
                for s in sorted(failed | set(finished)):
                    req, sim, admitted, need = active.pop(s)
                    ran = req.steps - self.backend.remaining(s)
                    surf = self.backend.finish(s, sim)  # memory stays held by the pool
                    res = Result(req.rid, int(np.prod(req.spec.nodes)), ran, req.arrival, admitted, t, surf,
                                 error="non-finite values" if s in failed else None)
                    self.stats.results.append(res)
                    if self.on_result is not None:
                        self.on_result(res)
                    done += 1
        return self.stats.results


def poisson_stream(n, rate, seed=0, large_frac=0.05, steps=(500, 3000), large_cells=(512, 512, 128)):
    """Request stream: config-4-style crystals plus a share of large jobs,
    step counts uniform in ``steps``, exponential inter-arrival times."""
    from . import crystal

    rng = np.random.default_rng(seed)
    base = crystal.config4_specs(n=n, seed=seed + 1, steps=steps[1])
    out = []
    t = 0.0
    for q in range(n):
        t += rng.exponential(1.0 / rate) if rate > 0 else 0.0
        st = int(rng.integers(steps[0], steps[1] + 1))
        sp = base[q]
        if rng.uniform() < large_frac:
            sp = crystal.CrystalSpec(cells=large_cells, lattice=16, radius=(0.2, 0.4), depth=10, tungsten_frac=0.25,
                                     seed=sp.seed, freq=sp.freq, steps=st)
        sp.steps = st
        out.append(Request(q, sp, st, t))
    return out


def summarize(results, makespan=None):
    """Latency percentiles (s) and aggregate Gcell-updates/s of a served stream."""
    if not results:
        return {}
    lat = np.array([r.latency for r in results])
    work = sum(r.nodes * r.steps for r in results)
    if makespan is None:
        makespan = max(r.finished for r in results) - min(r.arrival for r in results)
    return {"requests": len(results), "p50_s": float(np.percentile(lat, 50)),
            "p95_s": float(np.percentile(lat, 95)), "p99_s": float(np.percentile(lat, 99)),
            "mean_wait_s": float(np.mean([r.wait for r in results])),
            "gcell_updates_per_s": work / makespan / 1e9, "makespan_s": makespan,
            "cell_updates": int(work), "failed": sum(1 for r in results if r.error)}


def mean_work(n=4000, seed=0, **kw):
    """Mean node-steps per request of the stream distribution (for choosing a rate)."""
    reqs = poisson_stream(n, 1.0, seed=seed, **kw)
    return float(np.mean([r.spec.n_nodes * r.steps for r in reqs]))


def rate_for_load(gcells_per_s, load=0.7, **kw):
    """Arrival rate (requests/s) that offers `load` of a throughput."""
    return load * gcells_per_s * 1e9 / mean_work(**kw)


__all__ = ["Request", "Result", "Server", "GpuBackend", "poisson_stream", "summarize", "rate_for_load", "prepare"]
