"""ctypes front end of the C oracle (``oracle/cpu_ref.c``).

TEST INFRASTRUCTURE ONLY: the checker for the GPU solver.  Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` import
this module.  The product package never does.

Arrays follow the reference shapes (``simulation/grid.py:88-110``):
ux (nx-1, ny, nz), uy (nx, ny-1, nz), uz (nx, ny, nz-1), C order.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "cpu_ref.c"
BUILD = HERE / "_build"
LIB = BUILD / "libphono_oracle.so"


def build(force: bool = False) -> Path:
    """Compile the C restatement (no FMA contraction, OpenMP when present)."""
    BUILD.mkdir(exist_ok=True)
    newest = max(SRC.stat().st_mtime, (HERE / "velocity_form.inc").stat().st_mtime)
    if LIB.exists() and not force and LIB.stat().st_mtime >= newest:
        return LIB
    base = ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-shared", "-fPIC", "-std=c11",
            "-o", str(LIB) + ".tmp", str(SRC), "-lm"]
    try:
        subprocess.run(base[:1] + ["-fopenmp"] + base[1:], check=True, capture_output=True)
    except subprocess.CalledProcessError:
        subprocess.run(base, check=True, capture_output=True)
    os.replace(str(LIB) + ".tmp", LIB)
    return LIB


class _Problem(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
        ("fdx", ctypes.c_void_p), ("fdy", ctypes.c_void_p), ("fdz", ctypes.c_void_p),
        ("sdx", ctypes.c_void_p), ("sdy", ctypes.c_void_p), ("sdz", ctypes.c_void_p),
        ("mat", ctypes.c_void_p), ("table", ctypes.c_void_p), ("nmat", ctypes.c_int),
        ("dt", ctypes.c_double), ("src", ctypes.c_void_p), ("nsrc", ctypes.c_int),
        ("surface_mode", ctypes.c_int), ("bc", ctypes.c_int), ("source_mode", ctypes.c_int),
    ]


class _F64State(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in
                ("ux", "uy", "uz", "ux_old", "uy_old", "uz_old", "ux_new", "uy_new", "uz_new")]


class _F32State(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ("ux", "uy", "uz", "vx", "vy", "vz", "cx", "cy", "cz")]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(str(build()))
        _lib.ora_f64_run.restype = ctypes.c_int
        _lib.ora_f64_run.argtypes = [ctypes.POINTER(_Problem), ctypes.POINTER(_F64State), ctypes.c_int,
                                     ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int]
        for name in ("ora_run_f32k", "ora_run_f64v"):
            fn = getattr(_lib, name)
            fn.restype = ctypes.c_int
            fn.argtypes = [ctypes.POINTER(_Problem), ctypes.POINTER(_F32State), ctypes.c_int,
                           ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int]
        _lib.ora_abc_coeffs.restype = None
        _lib.ora_abc_coeffs.argtypes = [ctypes.POINTER(_Problem), ctypes.c_void_p]
        _lib.ora_max_threads.restype = ctypes.c_int
    return _lib


def max_threads() -> int:
    return int(lib().ora_max_threads())


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


class OracleProblem:
    """Inputs of one simulation, in the oracle's terms.

    ``spacing`` is the dict of per-axis arrays fdx, fdy, fdz, sdx, sdy, sdz (SI);
    ``mat`` the (nx, ny, nz) uint8 node material ids; ``table`` (nmat, 13) rows
    C00 C01 C02 C10 C11 C12 C20 C21 C22 C33 C44 C55 P; ``src`` the source
    sample of every global step.
    """

    def __init__(self, spacing, mat, table, dt, src, surface_mode=0, bc=0, source_mode=0):
        self.mat = _c(mat, np.uint8)
        self.nx, self.ny, self.nz = self.mat.shape
        self.sp = {k: _c(spacing[k], np.float64).ravel() for k in ("fdx", "fdy", "fdz", "sdx", "sdy", "sdz")}
        self.table = _c(table, np.float64).reshape(-1, 13)
        self.dt = float(dt)
        self.src = _c(src, np.float64).ravel()
        self.p = _Problem(self.nx, self.ny, self.nz,
                          *(self.sp[k].ctypes.data for k in ("fdx", "fdy", "fdz", "sdx", "sdy", "sdz")),
                          self.mat.ctypes.data, self.table.ctypes.data, self.table.shape[0],
                          self.dt, self.src.ctypes.data, self.src.size,
                          int(surface_mode), int(bc), int(source_mode))

    def shapes(self):
        nx, ny, nz = self.nx, self.ny, self.nz
        return (nx - 1, ny, nz), (nx, ny - 1, nz), (nx, ny, nz - 1)

    def abc_coeffs(self):
        out = np.zeros(8, np.float64)
        lib().ora_abc_coeffs(ctypes.byref(self.p), out.ctypes.data)
        return out


class F64State:
    """Reference leapfrog state: u, u_old and the persistent u_new."""

    def __init__(self, prob: OracleProblem):
        shp = prob.shapes()
        self.u = [np.zeros(s) for s in shp]
        self.u_old = [np.zeros(s) for s in shp]
        self.u_new = [np.zeros(s) for s in shp]

    def _c(self):
        arrs = self.u + self.u_old + self.u_new
        return _F64State(*(a.ctypes.data for a in arrs))


class F32KState:
    """Velocity-form state (u, v, Kahan term); dtype float32 (F32K) or float64 (F64V)."""

    dtype = np.float32

    def __init__(self, prob: OracleProblem):
        shp = prob.shapes()
        self.u = [np.zeros(s, self.dtype) for s in shp]
        self.v = [np.zeros(s, self.dtype) for s in shp]
        self.c = [np.zeros(s, self.dtype) for s in shp]

    def _c(self):
        arrs = self.u + self.v + self.c
        return _F32State(*(a.ctypes.data for a in arrs))


def run_f64(prob: OracleProblem, state: F64State | None = None, t0=0, nsteps=None, record_every=0,
            nthreads=0):
    """Run the FP64 reference restatement; returns (state, surface records)."""
    state = state or F64State(prob)
    nsteps = prob.src.size - t0 if nsteps is None else nsteps
    nrec = (t0 + nsteps) // record_every - t0 // record_every if record_every > 0 else 0
    surf = np.zeros((max(nrec, 0), prob.nx, prob.ny))
    st = state._c()
    rc = lib().ora_f64_run(ctypes.byref(prob.p), ctypes.byref(st), t0, nsteps, record_every,
                           surf.ctypes.data if nrec > 0 else None, nthreads)
    if rc != 0:
        raise ValueError(f"oracle f64 run failed: {rc}")
    return state, surf


class F64VState(F32KState):
    dtype = np.float64


def _run_velocity(fn, state_cls, prob, state, t0, nsteps, record_every, nthreads):
    state = state or state_cls(prob)
    nsteps = prob.src.size - t0 if nsteps is None else nsteps
    nrec = (t0 + nsteps) // record_every - t0 // record_every if record_every > 0 else 0
    surf = np.zeros((max(nrec, 0), prob.nx, prob.ny), state_cls.dtype)
    st = state._c()
    rc = getattr(lib(), fn)(ctypes.byref(prob.p), ctypes.byref(st), t0, nsteps, record_every,
                            surf.ctypes.data if nrec > 0 else None, nthreads)
    if rc != 0:
        raise ValueError(f"oracle {fn} failed: {rc}")
    return state, surf


def run_f32k(prob: OracleProblem, state: F32KState | None = None, t0=0, nsteps=None, record_every=0,
             nthreads=0):
    """FP32 velocity form with Kahan-compensated u (the GPU F32K scheme)."""
    return _run_velocity("ora_run_f32k", F32KState, prob, state, t0, nsteps, record_every, nthreads)


def run_f64v(prob: OracleProblem, state: F64VState | None = None, t0=0, nsteps=None, record_every=0,
             nthreads=0):
    """The same velocity-form scheme in FP64 (the GPU F64V scheme)."""
    return _run_velocity("ora_run_f64v", F64VState, prob, state, t0, nsteps, record_every, nthreads)
