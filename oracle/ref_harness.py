"""Headless runner for the reference phonomena solver.

TEST AND BENCHMARK INFRASTRUCTURE ONLY.  This module imports the reference's
own Python solver read-only and runs it unmodified through
``BaseSolver.init`` / ``run``: to freeze its outputs as golden fixtures, to
run the GB300 plugin inside the reference application in the tests, and to
time the reference's NumPy solvers in bench.py's reference arm.  The
reference is found under $PHONO_REFERENCE_ROOT, else in the
``baseline/_ref`` install made by ``oracle/install_reference.py``.  The
product package never imports it.

Shims (the reference imports packages that this environment lacks):
  * ``gui.worker.WorkerSignals`` -> a stub with ``status/progress.emit``
    (imported at simulation/grid.py:19 and simulation/base_solver.py:21);
  * ``h5py`` -> an empty module (simulation/base_solver.py:3; the writer is
    turned off with ``write_mode='off'``);
  * ``np.float`` -> ``float`` (simulation/grid.py:258,301, removed from NumPy).

Hooks installed on instances (never on the reference sources):
  * ``Material.setConstants`` can fill C and P from a uint8 id grid and a
    per-id (C 6x6, rho) list, so crystals with any number of materials can be
    expressed on a uniform mesh (the stock method knows two materials and
    vertical cylinders, simulation/material.py:55-63);
  * ``surface_mode='corrected'`` recomputes the z=0 row of uz_new with the
    parenthesisation fixed (simulation/base_solver.py:516);
  * ``bc='rigid'`` zeroes the four absorbing faces instead of
    simulation/base_solver.py:525-554;
  * ``time_step`` is wrapped to record uz[:, :, 0] every ``record_every`` steps.
"""
from __future__ import annotations

import copy
import os
import sys
import types
from pathlib import Path

import numpy as np

REF_ROOT = Path(os.environ.get("PHONO_REFERENCE_ROOT") or Path(__file__).resolve().parents[1] / "baseline" / "_ref")

_mods = None


def available() -> bool:
    return (REF_ROOT / "phonomena" / "simulation" / "base_solver.py").exists()


def install_shims(h5py_module=None):
    """Put the stand-ins for the reference's missing imports into sys.modules:
    ``gui.worker`` (WorkerSignals stub), ``h5py`` (the given module, else the
    real h5py if present, else an empty module) and ``np.float``."""
    if not hasattr(np, "float"):
        np.float = float  # noqa: NPY001 - the reference still uses the alias
    if "gui.worker" not in sys.modules:
        class _Sig:
            def emit(self, *a, **k):
                pass

        class WorkerSignals:
            def __init__(self):
                for n in ("finished", "success", "error", "warning", "result", "progress", "status", "quit"):
                    setattr(self, n, _Sig())

        gui = types.ModuleType("gui")
        worker = types.ModuleType("gui.worker")
        worker.WorkerSignals = WorkerSignals
        gui.worker = worker
        sys.modules["gui"] = gui
        sys.modules["gui.worker"] = worker
    if h5py_module is not None:
        sys.modules["h5py"] = h5py_module
    elif "h5py" not in sys.modules:
        try:
            import h5py  # noqa: F401
        except ImportError:
            sys.modules["h5py"] = types.ModuleType("h5py")


def import_reference():
    """Import the reference's simulation package with the shims above."""
    global _mods
    if _mods is not None:
        return _mods
    if not available():
        raise RuntimeError(f"reference sources not found under {REF_ROOT}")
    install_shims()
    path = str(REF_ROOT / "phonomena")
    if path not in sys.path:
        sys.path.insert(0, path)
    from simulation import base_solver, grid, material  # noqa: E402
    from simulation.solvers import solver_default, solver_threading  # noqa: E402
    _mods = types.SimpleNamespace(grid=grid, material=material, base_solver=base_solver,
                                  solver_default=solver_default, solver_threading=solver_threading)
    return _mods


def _props_from_materials(materials):
    """materials: list of dicts {name, c (6x6 in 1e10 Pa as the reference's JSON), p}."""
    return {m["name"]: {"name": m["name"], "c": [list(map(float, r)) for r in m["c"]], "p": m["p"]}
            for m in materials}


def make_uniform_case(size, SI, materials, ids, c_max, primary=0, secondary=None):
    """Build a reference Grid + Material for a uniform mesh of ``size`` cells.

    ``ids`` (nx, ny, nz) node material ids index ``materials``.  The time step
    comes from the reference's own ``setTimeStep`` over primary/secondary.
    """
    R = import_reference()
    g = R.grid.Grid()
    g.SI_conversion = SI
    g.init(*size)
    m = R.material.Material()
    m.init(grid=g, properties=_props_from_materials(materials))
    m.c_max = c_max
    m.setPrimary(materials[primary]["name"])
    m.setSecondary(materials[primary if secondary is None else secondary]["name"])
    ids = np.asarray(ids, np.uint8)
    assert ids.shape == (g.x.size, g.y.size, g.z.size), (ids.shape, g.x.size, g.y.size, g.z.size)
    names = [mm["name"] for mm in materials]
    _install_id_constants(m, ids, names)
    return g, m


def _install_id_constants(m, ids, names):
    def set_constants(self=m):
        self.C[:, :, :] = 0
        self.P[:, :, :] = 0
        for mid, name in enumerate(names):
            sel = self._phono_ids == mid
            self.C[sel] = np.array(self.properties[name]["c"])
            self.P[sel] = float(self.properties[name]["p"])
    m._phono_ids = ids
    m.setConstants = types.MethodType(lambda self: set_constants(self), m)


def load_settings_case(path):
    """Mirror of common.loadSettings (common.py:112-156) without the solver registry."""
    import json
    R = import_reference()
    cfg = json.load(open(path))
    g = R.grid.Grid()
    g.init(size_x=cfg["grid"]["size_x"], size_y=cfg["grid"]["size_y"], size_z=cfg["grid"]["size_z"])
    for key in ("min_d", "max_dx", "max_dy", "max_dz", "slope"):
        setattr(g, key, cfg["grid"][key])
    for t in cfg["inclusions"]:
        g.addInclusion(x=t["x"], y=t["y"], z=t["z"], r=t["r"])
    g.buildMesh()
    g.update()
    m = R.material.Material()
    m.init(grid=g, properties=cfg["material"]["properties"])
    m.c_max = cfg["simulation"]["courant"]
    m.setPrimary(cfg["material"]["primary"])
    m.setSecondary(cfg["material"]["secondary"])
    m.update()
    return g, m, cfg


def _corrected_tfbc(self):
    """z=0 row of uz_new with (T3[...,1] - T3[...,0]) / fdz taken together."""
    type(self).apply_u_tfbc(self)
    g, m = self.g, self.m
    a = (g.T5[1:, 1:-1, 0] - g.T5[:-1, 1:-1, 0]) / g.sdx[0, :, :]
    b = (g.T4[1:-1, 1:, 0] - g.T4[1:-1, :-1, 0]) / g.sdy[:, 0, :]
    c = (g.T3[1:-1, 1:-1, 1] - g.T3[1:-1, 1:-1, 0]) / g.fdz[:, :, 0]
    g.uz_new[1:-1, 1:-1, 0] = 2 * g.uz[1:-1, 1:-1, 0] - g.uz_old[1:-1, 1:-1, 0] \
        + (m.dt ** 2 / m.P[1:-1, 1:-1, 0]) * (a + b + c)


def _rigid_faces(self):
    g = self.g
    for arr in (g.ux_new, g.uy_new, g.uz_new):
        arr[-1, :, :] = 0
    for arr in (g.ux_new, g.uy_new, g.uz_new):
        arr[:, 0, :] = 0
    for arr in (g.ux_new, g.uy_new, g.uz_new):
        arr[:, -1, :] = 0
    for arr in (g.ux_new, g.uy_new, g.uz_new):
        arr[:, :, -1] = 0


def run_reference(g, m, steps, wave="sin", wave_args=None, surface_mode="reference", bc="reference",
                  record_every=0, solver="default"):
    """Run the reference solver; returns a dict of inputs and outputs."""
    R = import_reference()
    mod = {"default": R.solver_default, "threading": R.solver_threading}[solver]
    s = mod.Solver()
    s.cfg["write_mode"] = "off"
    s.cfg["wave"] = wave
    s.cfg["wave_args"] = dict(wave_args or {"f": 100})
    s.init(g, m, steps)
    if hasattr(m, "_phono_ids"):
        # init deep-copied the material; re-install the id hook and refill C, P
        _install_id_constants(s.m, m._phono_ids, list(s.m.properties.keys()))
        s.m.update()
    if surface_mode == "corrected":
        s.apply_u_tfbc = types.MethodType(_corrected_tfbc, s)
    if bc == "rigid":
        s.apply_u_abc = types.MethodType(_rigid_faces, s)
    records = []
    counter = {"tt": 0}
    orig_ts = s.time_step

    def time_step():
        orig_ts()
        counter["tt"] += 1
        if record_every and counter["tt"] % record_every == 0:
            records.append(np.copy(s.g.uz[:, :, 0]))
    s.time_step = time_step
    wave_fn = {"sin": s.update_sin, "ricker": s.update_ricker}[wave]
    src = np.array([wave_fn(tt=tt, **s.cfg["wave_args"]) for tt in range(steps)], dtype=np.float64)
    s.run()
    out = dict(
        x=np.array(s.g.x, np.float64), y=np.array(s.g.y, np.float64), z=np.array(s.g.z, np.float64),
        SI=float(s.g.SI_conversion),
        fdx=s.g.fdx.ravel().copy(), fdy=s.g.fdy.ravel().copy(), fdz=s.g.fdz.ravel().copy(),
        sdx=s.g.sdx.ravel().copy(), sdy=s.g.sdy.ravel().copy(), sdz=s.g.sdz.ravel().copy(),
        dt=float(s.m.dt), dt2=float(s.m.dt ** 2), src=src,
        ux=s.g.ux.copy(), uy=s.g.uy.copy(), uz=s.g.uz.copy(),
        surf=np.array(records) if records else np.zeros((0, s.g.x.size, s.g.y.size)),
    )
    out["ids"], out["table"] = ids_from_CP(s.m.C, s.m.P)
    return out


def ids_from_CP(C, P):
    """Compress per-node (C 6x6, P) into a uint8 id grid + (nmat, 13) table."""
    sel = [(0, 0), (0, 1), (0, 2), (1, 0), (1, 1), (1, 2), (2, 0), (2, 1), (2, 2), (3, 3), (4, 4), (5, 5)]
    rows = np.stack([C[..., a, b] for a, b in sel] + [P], axis=-1)
    flat = rows.reshape(-1, 13)
    table, inv = np.unique(flat, axis=0, return_inverse=True)
    assert table.shape[0] <= 256
    return inv.reshape(P.shape).astype(np.uint8), table


def copy_state(x):
    return copy.deepcopy(x)
