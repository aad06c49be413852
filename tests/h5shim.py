"""A minimal stand-in for h5py over NumPy .npz archives (test infrastructure).

h5py and libhdf5 are absent here and on the GPU machine.  The reference's
writer (simulation/base_solver.py:105-160) and reader
(simulation/analysis.py:44-96) use only a small part of h5py: ``File(path,
mode)`` as a context manager or with ``close()``, ``create_dataset(name,
shape=..., chunks=..., dtype=..., data=...)``, item assignment into a
dataset (``ux[:, :, :, tt] = g.ux``), ``get(name)``, ``attrs`` and
``type(f) == h5py.File``.  This module provides exactly that, storing a file
as an .npz archive at the given path (attributes as JSON under
``__attrs__``, lists turned back into arrays on reading), the same format
phonomena_gb300.output writes when h5py is missing.  Install it with
``sys.modules["h5py"] = h5shim`` before the reference modules are imported.
"""
from __future__ import annotations

import json
import os

import numpy as np


def _load(path):
    with np.load(path, allow_pickle=False) as z:
        attrs = json.loads(str(z["__attrs__"])) if "__attrs__" in z.files else {}
        data = {k: np.array(z[k]) for k in z.files if k != "__attrs__"}
    attrs = {k: (np.asarray(v) if isinstance(v, list) else v) for k, v in attrs.items()}
    return data, attrs


class Dataset:
    """An array behind h5py's Dataset interface: indexing reads or writes the
    array; the object itself compares by identity (``u != None`` holds, as
    analysis.spectrum asserts)."""

    def __init__(self, arr):
        self._a = arr

    shape = property(lambda self: self._a.shape)
    dtype = property(lambda self: self._a.dtype)

    def __getitem__(self, idx):
        return self._a[idx]

    def __setitem__(self, idx, value):
        self._a[idx] = value

    def __array__(self, dtype=None, copy=None):
        return self._a if dtype is None else self._a.astype(dtype)


class File:
    def __init__(self, path, mode="r"):
        self.path = os.fspath(path)
        self.mode = mode
        if mode in ("r", "r+", "a") and os.path.exists(self.path):
            self._data, self.attrs = _load(self.path)
        elif mode == "r":
            raise FileNotFoundError(self.path)
        else:
            self._data, self.attrs = {}, {}

    def create_dataset(self, name, shape=None, chunks=None, dtype=None, data=None):
        arr = np.array(data, dtype=dtype) if data is not None else np.zeros(shape, dtype=dtype or np.float64)
        self._data[name] = arr
        return Dataset(arr)

    def get(self, name):
        return Dataset(self._data[name]) if name in self._data else None

    def __getitem__(self, name):
        return Dataset(self._data[name])

    def keys(self):
        return self._data.keys()

    def close(self):
        if self.mode != "r":
            js = {k: (v.tolist() if isinstance(v, np.ndarray) else (v.item() if isinstance(v, np.generic) else v))
                  for k, v in self.attrs.items()}
            with open(self.path, "wb") as f:
                np.savez(f, __attrs__=np.array(json.dumps(js)), **self._data)
        self.mode = "r"

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
