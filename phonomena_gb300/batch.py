"""Many simulations stepped together (phono_batch_* of include/phono.h).

A ``Batch`` holds up to ``capacity`` device simulations of one arithmetic
scheme.  Two launch schemes:

* persistent (``streams=0``, the default): every instance at the batch's
  tile height; each time step is one persistent tile launch in which the
  CTAs pull (instance, tile) work items, costliest instances first, plus one
  face launch for all instances;
* streams (``streams=W``): every instance runs its own step kernels, with
  its own tile height and x segments, on one of W worker streams, so that
  the instances' launches run side by side on the GPU; each instance
  replays its own 12-step graph (captured when it joins) and does not wait
  for the others between chunks.

Chunks of 12 steps are replayed from captured CUDA graphs.  Instances
keep their own step counters and budgets, so a batch can hold simulations of
different sizes at different points of their runs, and instances can join
and leave between calls.  Results are those of stepping each alone.
"""
from __future__ import annotations

import ctypes

from . import _lib
from ._lib import check


class Batch:
    def __init__(self, capacity, precision="f32k", tile_j=8, streams=0):
        L = _lib.load()
        self._L = L
        self.precision = precision
        self.tile_j = int(tile_j)
        self.streams = int(streams)
        b = ctypes.c_void_p()
        check(L.phono_batch_create(int(capacity), _lib.PRECISIONS[precision], self.tile_j, ctypes.byref(b)))
        self._b = b
        if self.streams:
            try:
                check(L.phono_batch_set_mode(b, _lib.BATCH_STREAMS, self.streams))
            except Exception:
                L.phono_batch_destroy(b)
                self._b = None
                raise
        self._members = {}  # slot -> DeviceSimulation (kept alive while in the batch)

    def add(self, sim, nsteps):
        """Attach a DeviceSimulation for nsteps more steps; returns its slot."""
        if sim.precision != self.precision:
            raise ValueError("simulation precision differs from the batch")
        rc = self._L.phono_batch_add(self._b, sim._h, int(nsteps))
        if rc < 0:
            check(rc)
        self._members[rc] = sim
        return rc

    def remove(self, slot):
        check(self._L.phono_batch_remove(self._b, int(slot)))
        return self._members.pop(slot)

    def remaining(self, slot):
        rc = self._L.phono_batch_remaining(self._b, int(slot))
        if rc < 0:
            check(rc)
        return rc

    def step(self, nsteps):
        check(self._L.phono_batch_step(self._b, int(nsteps)))

    def sync(self):
        check(self._L.phono_batch_sync(self._b))

    def last_step_ms(self):
        ms = ctypes.c_float()
        check(self._L.phono_batch_last_step_ms(self._b, ctypes.byref(ms)))
        return float(ms.value)

    @property
    def members(self):
        return dict(self._members)

    def close(self):
        if getattr(self, "_b", None):
            self._L.phono_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
