"""One simulation resident on the GPU, driven through the C ABI.

``DeviceSimulation`` owns a ``phono_handle``: field buffers, material ids and
table, spacing arrays, source samples and the surface-record buffer all live
in device memory; ``step(n)`` enqueues n fused step launches (graph replays)
on the handle's stream.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import check


def field_shape(nx, ny, nz, comp):
    """Reference shape of a displacement component (simulation/grid.py:88-90)."""
    return (nx - (comp == 0), ny - (comp == 1), nz - (comp == 2))


def footprint(shape, precision="f32k", max_steps=0, record_every=0):
    """Device bytes a DeviceSimulation of this mesh shape allocates (phono_footprint)."""
    L = _lib.load()
    out = ctypes.c_size_t()
    nx, ny, nz = (int(v) for v in shape)
    check(L.phono_footprint(nx, ny, nz, _lib.PRECISIONS[precision], int(max_steps), int(record_every),
                            ctypes.byref(out)))
    return int(out.value)


def inclusion_columns(targets):
    """(tx, ty, tz, tr) float32 columns of an inclusion list: a NumPy record
    array with fields x, y, z, r (the reference's Grid.targets) or a sequence
    of (x, y, z, r) rows."""
    t = np.asarray(targets)
    if t.dtype.names and all(k in t.dtype.names for k in ("x", "y", "z", "r")):
        t = np.atleast_1d(t)
        return tuple(np.ascontiguousarray(t[k], dtype=np.float32) for k in ("x", "y", "z", "r"))
    t = np.asarray(targets, dtype=np.float64).reshape(-1, 4)
    return tuple(np.ascontiguousarray(t[:, q], dtype=np.float32) for q in range(4))


class DeviceSimulation:
    """Device-resident FDTD state behind ``phono_create`` / ``phono_step``.

    spacing: dict with fdx, fdy, fdz (n-1) and sdx, sdy, sdz (n-2) arrays (SI).
    mat: (nx, ny, nz) uint8 node material ids.  table: (nmat, 13) rows
    C00 C01 C02 C10 C11 C12 C20 C21 C22 C33 C44 C55 rho.
    """

    def __init__(self, spacing, mat, table, dt, *, precision="f64", surface_mode="reference", bc="absorbing",
                 source_mode="line", max_steps=0, record_every=0, tile_j=0, x_segment=0):
        L = _lib.load()
        self._L = L
        self.mat = np.ascontiguousarray(mat, dtype=np.uint8)
        if self.mat.ndim != 3:
            raise ValueError("mat must be a 3-D (nx, ny, nz) array")
        self.nx, self.ny, self.nz = map(int, self.mat.shape)
        self._sp = {k: np.ascontiguousarray(np.ravel(spacing[k]), dtype=np.float64)
                    for k in ("fdx", "fdy", "fdz", "sdx", "sdy", "sdz")}
        for k, n in (("fdx", self.nx - 1), ("fdy", self.ny - 1), ("fdz", self.nz - 1),
                     ("sdx", self.nx - 2), ("sdy", self.ny - 2), ("sdz", self.nz - 2)):
            if self._sp[k].size != n:
                raise ValueError(f"{k} has {self._sp[k].size} values, expected {n}")
        self.table = np.ascontiguousarray(table, dtype=np.float64).reshape(-1, 13)
        self.dt = float(dt)
        self.precision = precision
        self.record_every = int(record_every)
        self.max_steps = int(max_steps)
        self.dtype = np.float32 if precision == "f32k" else np.float64
        segments = None
        if np.ndim(x_segment):  # a list of segment lengths: set after creation
            segments, x_segment = x_segment, 0
        d = _lib.PhonoDesc(
            self.nx, self.ny, self.nz,
            *(self._sp[k].ctypes.data for k in ("fdx", "fdy", "fdz", "sdx", "sdy", "sdz")),
            self.mat.ctypes.data, self.table.ctypes.data, self.table.shape[0], self.dt,
            _lib.PRECISIONS[precision], _lib.SURFACE_MODES[surface_mode], _lib.BCS[bc],
            _lib.SOURCE_MODES[source_mode], self.max_steps, self.record_every, int(tile_j), int(x_segment))
        h = ctypes.c_void_p()
        check(L.phono_create(ctypes.byref(d), ctypes.byref(h)))
        self._h = h
        self.tile_j = int(tile_j) or (4 if precision == "f32k" else 8)
        self.x_segment = int(x_segment) or 24
        self.surface_mode, self.bc, self.source_mode = surface_mode, bc, source_mode
        self._source = None
        if segments is not None:
            try:
                self.set_tiling(0, segments)
            except Exception:
                self.close()
                raise

    # -- control ----------------------------------------------------------
    def set_source(self, samples):
        s = np.ascontiguousarray(samples, dtype=np.float64)
        check(self._L.phono_set_source(self._h, s.ctypes.data, s.size))
        self._source = s

    def step(self, n):
        check(self._L.phono_step(self._h, int(n)))

    def reset(self):
        """Zero the state, records and step counter (materials and source kept)."""
        check(self._L.phono_reset(self._h))

    def set_materials(self, mat, table):
        m = np.ascontiguousarray(mat, dtype=np.uint8)
        if m.shape != (self.nx, self.ny, self.nz):
            raise ValueError("material ids must match the mesh shape")
        t = np.ascontiguousarray(table, dtype=np.float64).reshape(-1, 13)
        check(self._L.phono_set_materials(self._h, m.ctypes.data, t.ctypes.data, t.shape[0]))
        self.mat, self.table = m, t

    def set_tiling(self, tile_j=0, x_segment=0):
        """Change the tile shape (0 keeps a value); results do not depend on it.

        x_segment: planes per block segment, -L for tapered L-plane segments,
        or a list of segment lengths adding up to nx - 1 (phono_set_segments).
        """
        if np.ndim(x_segment):
            seg = np.ascontiguousarray(x_segment, dtype=np.int32)
            check(self._L.phono_set_segments(self._h, int(tile_j), seg.ctypes.data, seg.size))
            self.x_segment = tuple(int(v) for v in seg)
        else:
            check(self._L.phono_set_tiling(self._h, int(tile_j), int(x_segment)))
            self.x_segment = int(x_segment) or self.x_segment
        self.tile_j = int(tile_j) or self.tile_j

    def set_lattice(self, lat, table):
        """Material ids built on the device from a hole lattice (crystal.lattice)
        and a new table; same ids as set_materials(crystal.ids_from_lattice(...))."""
        radius = np.ascontiguousarray(lat["radius"], dtype=np.float64)
        kind = np.ascontiguousarray(lat["kind"], dtype=np.uint8)
        if radius.ndim != 2 or kind.shape != radius.shape:
            raise ValueError("radius and kind must be (ncx, ncy) arrays of one shape")
        t = np.ascontiguousarray(table, dtype=np.float64).reshape(-1, 13)
        d = _lib.PhonoLattice(int(lat["pitch"]), radius.shape[0], radius.shape[1], radius.ctypes.data,
                              kind.ctypes.data, int(lat["depth"]), int(lat.get("host", 0)))
        check(self._L.phono_set_lattice(self._h, ctypes.byref(d), t.ctypes.data, t.shape[0]))
        self.mat = None  # ids live on the device; host_ids() rebuilds them when asked
        self._lattice = lat
        self.table = t

    def set_inclusions(self, x, y, z, targets, table, inside=1, host=0, ids=None):
        """Material ids of the reference's inclusion model built on the device
        (phono_set_inclusions): node coordinates x, y, z and the inclusion list
        ``targets`` as the reference's Grid.targets holds it (fields or columns
        x, y, z, r, stored as float32); ``ids`` optionally gives each inclusion
        its own material id (default: all ``inside``)."""
        x, y, z = (np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, z))
        if (x.size, y.size, z.size) != (self.nx, self.ny, self.nz):
            raise ValueError("node coordinates do not match the mesh")
        cols = inclusion_columns(targets)
        n = cols[0].size
        idv = None if ids is None else np.ascontiguousarray(ids, dtype=np.uint8)
        if idv is not None and idv.size != n:
            raise ValueError("one material id per inclusion")
        t = np.ascontiguousarray(table, dtype=np.float64).reshape(-1, 13)
        d = _lib.PhonoInclusions(x.ctypes.data, y.ctypes.data, z.ctypes.data, n,
                                 *(c.ctypes.data for c in cols), None if idv is None else idv.ctypes.data,
                                 int(inside), int(host))
        check(self._L.phono_set_inclusions(self._h, ctypes.byref(d), t.ctypes.data, t.shape[0]))
        self.mat = None  # ids live on the device; host_ids() reads them back when asked
        self._lattice = None
        self.table = t

    def test_wait_timeout(self, polls=0, skip_plane=-1):
        """Test hook of the tile pass's bounded waits (phono_test_wait_timeout):
        with skip_plane >= 0 the waits on that plane run out after ``polls``
        polls and the next sync() raises PHONO_ERR_TIMEOUT; (0, -1) turns it off."""
        check(self._L.phono_test_wait_timeout(self._h, int(polls), int(skip_plane)))

    def download_materials(self):
        """The node material ids held on the device, (nx, ny, nz) uint8."""
        out = np.empty((self.nx, self.ny, self.nz), dtype=np.uint8)
        check(self._L.phono_download_materials(self._h, out.ctypes.data, out.nbytes))
        return out

    def host_ids(self):
        """The node material ids on the host (read back from the device if they were built there)."""
        if self.mat is None:
            self.mat = self.download_materials()
        return self.mat

    @property
    def stream_ptr(self):
        """cudaStream_t of the handle (for CUDA events recorded by the caller)."""
        return int(self._L.phono_stream(self._h) or 0)

    def sync(self):
        check(self._L.phono_sync(self._h))

    @property
    def steps_done(self):
        return int(self._L.phono_steps_done(self._h))

    def time_kernels(self, n):
        """Advance n steps with the tile and face launches timed apart by CUDA
        events (phono_time_kernels): (tile ms, face ms) summed over the steps."""
        t, f = ctypes.c_float(), ctypes.c_float()
        check(self._L.phono_time_kernels(self._h, int(n), ctypes.byref(t), ctypes.byref(f)))
        return float(t.value), float(f.value)

    def last_step_ms(self):
        ms = ctypes.c_float()
        check(self._L.phono_last_step_ms(self._h, ctypes.byref(ms)))
        return float(ms.value)

    # -- data ------------------------------------------------------------
    @property
    def n_records(self):
        return self.max_steps // self.record_every if self.record_every > 0 else 0

    def read_surface(self, first=0, count=None, out=None):
        if count is None:
            count = self.steps_done // self.record_every - first if self.record_every > 0 else 0
        shape = (max(count, 0), self.nx, self.ny)
        if out is None:
            out = np.empty(shape, dtype=self.dtype)
        elif out.shape != shape or out.dtype != self.dtype or not out.flags.c_contiguous:
            raise ValueError(f"out must be a C-contiguous {self.dtype.__name__} array of shape {shape}")
        check(self._L.phono_read_surface(self._h, int(first), int(max(count, 0)), out.ctypes.data))
        return out

    def download(self, field, out=None):
        f = _lib.FIELDS[field]
        shape = field_shape(self.nx, self.ny, self.nz, f % 3)
        if out is None:
            out = np.empty(shape, dtype=self.dtype)
        elif out.shape != shape or out.dtype != self.dtype or not out.flags.c_contiguous:
            raise ValueError(f"out must be a C-contiguous {self.dtype.__name__} array of shape {shape}")
        check(self._L.phono_download(self._h, f, out.ctypes.data, out.nbytes))
        return out

    def upload(self, field, arr):
        f = _lib.FIELDS[field]
        a = np.ascontiguousarray(arr, dtype=self.dtype)
        if a.shape != field_shape(self.nx, self.ny, self.nz, f % 3):
            raise ValueError(f"{field} must have shape {field_shape(self.nx, self.ny, self.nz, f % 3)}")
        check(self._L.phono_upload(self._h, f, a.ctypes.data, a.nbytes))

    # -- checkpoint / resume ------------------------------------------------
    @property
    def state_fields(self):
        """Fields that make up the state of this scheme (all others are derived)."""
        if self.precision == "f64":
            return ("ux", "uy", "uz", "ux_old", "uy_old", "uz_old")
        return ("ux", "uy", "uz", "vx", "vy", "vz", "cx", "cy", "cz")

    def checkpoint(self):
        """Everything needed to resume this run on another handle: the state
        fields, the step count, the surface records so far and the inputs."""
        self.sync()
        ck = {k: self.download(k) for k in self.state_fields}
        ck["steps_done"] = np.array(self.steps_done)
        ck["surface"] = self.read_surface()
        ck["ids"] = self.host_ids()
        ck["table"] = self.table
        ck["source"] = self._source if self._source is not None else np.zeros(0)
        for k, v in self._sp.items():
            ck[k] = v
        listed = isinstance(self.x_segment, tuple)
        ck["meta"] = np.array([self.dt, self.max_steps, self.record_every, self.tile_j,
                               0 if listed else self.x_segment], np.float64)
        ck["segments"] = np.array(self.x_segment if listed else [], np.int32)
        ck["modes"] = np.array([self.precision, self.surface_mode, self.bc, self.source_mode])
        return ck

    def save_checkpoint(self, path):
        np.savez(path, **self.checkpoint())

    def restore(self, ck):
        """Resume from a checkpoint of a run with the same description and source."""
        steps = int(ck["steps_done"])
        check(self._L.phono_set_steps_done(self._h, steps))  # selects the buffers the fields go to
        for k in self.state_fields:
            self.upload(k, ck[k])
        surf = np.ascontiguousarray(ck["surface"], dtype=self.dtype)
        if surf.shape[0]:
            check(self._L.phono_upload_surface(self._h, 0, surf.shape[0], surf.ctypes.data))

    @classmethod
    def from_checkpoint(cls, ck):
        """A new simulation resumed from a checkpoint (dict or .npz path)."""
        if not isinstance(ck, dict):
            with np.load(ck) as f:
                ck = {k: f[k] for k in f.files}
        dt, max_steps, record_every, tile_j, x_segment = ck["meta"]
        segs = ck.get("segments")
        if segs is not None and np.size(segs):
            x_segment = tuple(int(v) for v in segs)
        precision, surface_mode, bc, source_mode = (str(x) for x in ck["modes"])
        sp = {k: ck[k] for k in ("fdx", "fdy", "fdz", "sdx", "sdy", "sdz")}
        sim = cls(sp, ck["ids"], ck["table"], float(dt), precision=precision, surface_mode=surface_mode, bc=bc,
                  source_mode=source_mode, max_steps=int(max_steps), record_every=int(record_every),
                  tile_j=int(tile_j), x_segment=x_segment if isinstance(x_segment, tuple) else int(x_segment))
        if ck["source"].size:
            sim.set_source(ck["source"])
        sim.restore(ck)
        return sim

    def energy(self):
        out = np.zeros(2, np.float64)
        check(self._L.phono_energy(self._h, out.ctypes.data))
        return float(out[0]), float(out[1])

    def close(self):
        if getattr(self, "_h", None):
            self._L.phono_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
