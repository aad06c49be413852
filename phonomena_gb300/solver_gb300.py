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
  record_every  sampling period of the output in steps (0 = surface records off)
  output        'surface' (uz[:,:,0] every record_every steps) | 'volume'
                (ux, uy, uz every record_every steps, the reference writer's
                layout: record_every = 1 gives the reference's file)
  material_builder  'device' (ids of the inclusion model built on the GPU,
                phono_set_inclusions; no per-node C / P arrays on the host) |
                'host' (Material.update on the host, then compressed to ids)
  tile_j, x_segment  kernel tile shape (0: tuned once per mesh above 2M nodes, else the default)

With ``write_mode`` other than 'off' the result file is written when the run
ends (phonomena_gb300/output.py); ``self.file`` then names that file
(``.npz`` appended when h5py is absent).
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
from .model import inclusion_inputs, solver_inputs

TUNE_MIN_NODES = 2_000_000  # below this the default tile shape is used without tuning
logger = logging.getLogger(__name__)

cfg = {"precision": "f64", "surface_mode": "reference", "bc": "absorbing", "source_mode": "line",
       "record_every": 10, "output": "surface", "material_builder": "device", "tile_j": 0, "x_segment": 0}

VOLUME_OUTPUT_MAX_BYTES = 8 << 30  # host memory a volume-layout result may take

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
        if self.sim is not None:
            self.sim.close()
            self.sim = None
        c = self.cfg
        incl = inclusion_inputs(self.g, self.m) if c.get("material_builder", "device") == "device" else None
        if incl is not None:  # ids built on the GPU from the inclusion list
            spacing, table, dt, targets = incl
            ids = np.zeros((self.g.x.size, self.g.y.size, self.g.z.size), dtype=np.uint8)
        else:
            self.m.update()
            spacing, ids, table, dt = solver_inputs(self.g, self.m)
        self.record_every = int(c.get("record_every", 0) or 0)
        tj, xs = int(c.get("tile_j", 0) or 0), int(c.get("x_segment", 0) or 0)
        if not tj and ids.size >= TUNE_MIN_NODES and incl is None:  # large meshes: the tuner's shape (per mesh)
            from . import autotune

            tj, xs = autotune.tune(spacing, ids, table, dt, precision=c["precision"])
        self.sim = DeviceSimulation(spacing, ids, table, dt, precision=c["precision"],
                                    surface_mode=c["surface_mode"], bc=c["bc"], source_mode=c["source_mode"],
                                    max_steps=max(int(self.t), 1), record_every=self.record_every,
                                    tile_j=tj, x_segment=xs)
        if incl is not None:
            self.sim.set_inclusions(self.g.x, self.g.y, self.g.z, targets, table, inside=1, host=0)
        wave_fn = {"sin": self.update_sin, "ricker": self.update_ricker}[c["wave"]]
        samples = np.array([wave_fn(tt=tt, **c["wave_args"]) for tt in range(int(self.t))], dtype=np.float64)
        self.sim.set_source(samples)
        self.surface = None
        self.volume = None

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

    def material_ids(self):
        """(nx, ny, nz) uint8 node material ids as held on the device."""
        return self.sim.host_ids()

    def material_table(self):
        """(nmat, 13) table rows: C00 C01 C02 C10 C11 C12 C20 C21 C22 C33 C44 C55 rho."""
        return self.sim.table

    def _writing(self):
        return self.cfg.get("write_mode", "off") != "off"

    def _volume_buffers(self, total):
        """Host arrays of the volume layout, (component shape..., records)."""
        k = max(self.record_every, 1)
        nrec = total // k
        nx, ny, nz = self.g.x.size, self.g.y.size, self.g.z.size
        shapes = {"ux": (nx - 1, ny, nz), "uy": (nx, ny - 1, nz), "uz": (nx, ny, nz - 1)}
        need = sum(int(np.prod(sh)) for sh in shapes.values()) * nrec * 8
        if need > VOLUME_OUTPUT_MAX_BYTES:
            raise MemoryError(f"volume output of {need / 2**30:.1f} GiB exceeds the limit; use output='surface' "
                              f"or a larger record_every")
        return {f: np.zeros(sh + (nrec,), dtype=np.float64) for f, sh in shapes.items()}

    # -- BaseSolver.run (base_solver.py:224-280) -----------------------------
    def run(self, *args, **kwargs):
        signals = kwargs.get("signals") or _WorkerSignals()
        signals.status.emit("Solver starting..")
        self.running.set()
        signals.status.emit("Running simulation.")
        stime = time.time()
        total = int(self.t) - self.sim.steps_done
        volume = self._writing() and self.cfg.get("output", "surface") == "volume"
        k = max(self.record_every, 1)
        if volume:  # one chunk per record: the whole state is read back after every k-th step
            self.volume = self._volume_buffers(total)
            chunk = k
        else:
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
            if volume and n == k:
                r = done // k - 1
                for f in ("ux", "uy", "uz"):
                    self.volume[f][..., r] = self.sim.download(f)
            if progress < 99:
                progress = min(99, int((done / total) * 100))
                signals.progress.emit(progress)
        self.running.clear()
        self.results()
        if self._writing():
            from .output import write_results
            self.file = write_results(self.file, self)
        signals.status.emit("Simulation finished in {:.2f}s.".format(time.time() - stime))
        signals.progress.emit(100)

    def release(self):
        if self.sim is not None:
            self.sim.close()
            self.sim = None
