"""GB300 solver plugin for phonomena (drop-in ``Solver`` class).

Copy or symlink this module into ``phonomena/simulation/solvers/`` (or import
it from there): ``common.findSolvers`` (phonomena/common.py:93-110) then
finds a solver named ``gb300`` and ``common.loadSettings`` selects it with
``"solver": "gb300"``.  Inside phonomena the class subclasses the
reference's ``simulation.base_solver.BaseSolver``; standalone it subclasses
``phonomena_gb300.base.BaseSolver`` with the same skeleton.

Behaviour mirrors ``BaseSolver`` (simulation/base_solver.py:172-292):
``Solver()`` takes no arguments; ``init(grid, material, steps)`` deep-copies
the inputs, rebuilds mesh and material and moves everything to the GPU;
``run(signals=...)`` blocks until the steps are done, emitting
``signals.status`` and integer ``signals.progress`` 0..100, honouring
``cancel()`` between chunks, and leaves the final displacement in
``self.g.ux / uy / uz`` as float64 arrays.  ``step(n)`` advances n steps.

Extra ``cfg`` keys (merged like solver_default.py:19):
  precision     'f64' (reference arithmetic, bit-identical) | 'f32k'
  surface_mode  'reference' (base_solver.py:516 as written) | 'corrected'
  bc            'absorbing' (reference faces) | 'rigid'
  source_mode   'line' (uz[0,:,0], reference) | 'wall' (uz[0,:,:])
  record_every  surface uz[:,:,0] sampling period in steps (0 = off)
  tile_j, x_segment  kernel tile shape (0: tuned once per mesh above 2M nodes, else the default)
"""
from __future__ import annotations

import copy
import logging
import time

import numpy as np

try:  # inside the phonomena application
    from simulation import base_solver as _ref_base  # type: ignore

    _Base = _ref_base.BaseSolver
    _WorkerSignals = _ref_base.WorkerSignals
except Exception:  # standalone
    from .base import BaseSolver as _Base
    from .base import WorkerSignals as _WorkerSignals

from .device import DeviceSimulation
from .model import solver_inputs

TUNE_MIN_NODES = 2_000_000  # below this the default tile shape is used without tuning
logger = logging.getLogger(__name__)

cfg = {"precision": "f64", "surface_mode": "reference", "bc": "absorbing", "source_mode": "line",
       "record_every": 10, "tile_j": 0, "x_segment": 0}

GRAPH_CHUNK = 12  # steps per captured graph replay


class Solver(_Base):
    def __init__(self):
        super().__init__(logger)
        self.name = "gb300"
        self.description = ("<p>GB300 solver: one fused sm_103a kernel per time step, graph-replayed, "
                            "fields resident in HBM. precision f64 matches the default solver bit for bit; "
                            "f32k is FP32 with Kahan-compensated displacement.</p>")
        self.cfg = {**cfg, **self.cfg}
        self.sim = None
        self.surface = None

    # -- BaseSolver.init (base_solver.py:194-222) ----------------------------
    def init(self, grid, material, steps):
        self.g = copy.deepcopy(grid)
        self.m = copy.deepcopy(material)
        self.t = copy.deepcopy(steps)
        logger.info("Initializing %s with settings: %s", self.name, self.cfg)
        self.g.buildMesh()
        self.g.update()
        self.m.update()
        if self.sim is not None:
            self.sim.close()
            self.sim = None
        spacing, ids, table, dt = solver_inputs(self.g, self.m)
        c = self.cfg
        self.record_every = int(c.get("record_every", 0) or 0)
        tj, xs = int(c.get("tile_j", 0) or 0), int(c.get("x_segment", 0) or 0)
        if not tj and ids.size >= TUNE_MIN_NODES:  # large meshes: the tuner's shape (cached per mesh)
            from . import autotune

            tj, xs = autotune.tune(spacing, ids, table, dt, precision=c["precision"])
        self.sim = DeviceSimulation(spacing, ids, table, dt, precision=c["precision"],
                                    surface_mode=c["surface_mode"], bc=c["bc"], source_mode=c["source_mode"],
                                    max_steps=max(int(self.t), 1), record_every=self.record_every,
                                    tile_j=tj, x_segment=xs)
        wave_fn = {"sin": self.update_sin, "ricker": self.update_ricker}[c["wave"]]
        samples = np.array([wave_fn(tt=tt, **c["wave_args"]) for tt in range(int(self.t))], dtype=np.float64)
        self.sim.set_source(samples)
        self.surface = None

    # -- step entry point ----------------------------------------------------
    def step(self, n=1):
        """Advance n time steps on the device (asynchronous)."""
        self.sim.step(int(n))

    def results(self):
        """Copy the current displacement into self.g.ux/uy/uz (float64) and
        the surface records into self.surface (records, nx, ny)."""
        self.sim.sync()
        for f in ("ux", "uy", "uz"):
            setattr(self.g, f, self.sim.download(f).astype(np.float64, copy=False))
        if self.record_every > 0:
            self.surface = self.sim.read_surface().astype(np.float64, copy=False)
        return self.g.ux, self.g.uy, self.g.uz

    # -- BaseSolver.run (base_solver.py:224-280) -----------------------------
    def run(self, *args, **kwargs):
        signals = kwargs.get("signals") or _WorkerSignals()
        signals.status.emit("Solver starting..")
        self.running.set()
        signals.status.emit("Running simulation.")
        stime = time.time()
        total = int(self.t) - self.sim.steps_done
        chunk = max(GRAPH_CHUNK, (total // 100) // GRAPH_CHUNK * GRAPH_CHUNK)
        signals.progress.emit(0)
        done = 0
        progress = 0
        while done < total:
            if not self.running.is_set():
                logger.warning("Simulation cancelled.")
                break
            n = min(chunk, total - done)
            self.sim.step(n)
            self.sim.sync()
            done += n
            if progress < 99:
                progress = min(99, int((done / total) * 100))
                signals.progress.emit(progress)
        self.running.clear()
        self.results()
        if self.cfg.get("write_mode", "off") != "off":
            from .output import write_results
            write_results(self.file, self)
        signals.status.emit("Simulation finished in {:.2f}s.".format(time.time() - stime))
        signals.progress.emit(100)

    def release(self):
        if self.sim is not None:
            self.sim.close()
            self.sim = None
