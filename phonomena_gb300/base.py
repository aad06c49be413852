"""Stand-in for phonomena's BaseSolver skeleton when the reference is absent.

Inside the phonomena application the GPU plugin subclasses the reference's
own ``simulation.base_solver.BaseSolver``; elsewhere it subclasses this class,
which keeps the same constructor, attributes and helper methods
(simulation/base_solver.py:172-312): name, description, file, running,
writer, logger, cfg, cancel(), test(), update_sin(), update_ricker().
"""
from __future__ import annotations

import os
import tempfile
import threading

import numpy as np

from .model import Grid, Material


class _Signal:
    def __init__(self):
        self.calls = []

    def emit(self, *args):
        self.calls.append(args)


class WorkerSignals:
    """Duck type of gui/worker.py:WorkerSignals: status.emit(str), progress.emit(int 0..100)."""

    def __init__(self):
        for n in ("finished", "success", "error", "warning", "result", "progress", "status", "quit"):
            setattr(self, n, _Signal())


class TestDefaults:
    """Minimal test setup of simulation/base_solver.py:28-70 (GaAs, 4 x 5 x 6 cells)."""

    properties = {"GaAs": {"name": "Gallium Arsenide", "p": 5307,
                           "c": np.array([[11.88, 5.87, 5.38, 0, 0, 0], [5.87, 11.88, 5.38, 0, 0, 0],
                                          [5.87, 5.38, 11.88, 0, 0, 0], [0, 0, 0, 5.94, 0, 0],
                                          [0, 0, 0, 0, 5.94, 0], [0, 0, 0, 0, 0, 5.94]]) * 1e10}}

    @classmethod
    def make(cls):
        g = Grid()
        g.init(size_x=4, size_y=5, size_z=6)
        m = Material()
        m.init(grid=g, properties=cls.properties)
        g.min_d = g.max_dx = g.max_dy = g.max_dz = 1
        g.slope = 0
        g.buildMesh()
        m.setPrimary("GaAs")
        m.setSecondary("GaAs")
        return g, m


class BaseSolver:
    def __init__(self, logger):
        self.name = "default"
        self.description = "<p>Base Solver. This string should be overwritten by the child class</p>"
        with tempfile.NamedTemporaryFile() as f:
            self.file = os.path.realpath(f.name)
        self.running = threading.Event()
        self.writer = None
        self.logger = logger
        self.cfg = {"wave": "ricker", "wave_args": {"f": 100}, "write_mode": "process"}

    def cancel(self):
        if self.running.is_set():
            self.running.clear()

    def test(self):
        g, m = TestDefaults.make()
        self.init(grid=g, material=m, steps=10)
        self.run()

    def update_sin(self, tt, f, **kwargs):
        return np.sin(2 * np.pi * f * tt * self.m.dt)

    def update_ricker(self, tt, f, source_delay=0, **kwargs):
        arg = (np.pi * f * (self.m.dt * tt - source_delay)) ** 2
        return (1 - 2 * arg) * np.exp(-arg)
