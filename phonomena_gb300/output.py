"""Result file in the reference writer's schema (simulation/base_solver.py:105-133).

Datasets keep the reference names.  The surface-sampled output stores
``uz`` as a 4-D (nx, ny, 1, records) array, so ``analysis.spectrum(file,
'uz', z_index=0, ...)`` (simulation/analysis.py:44-96) reads it the way it
reads a full-volume file; ``ux``, ``uy``, ``uz_final`` hold the last state.
Attributes: x, y, z, sdx..fdz (reference shapes), steps, dt, prim_material,
sec_material, solver_cfg, plus record_every and dt_record = dt*record_every
(the time step of the ``uz`` axis 3).

HDF5 is written with h5py when it is importable; otherwise the same names go
into a NumPy ``.npz`` archive (attributes as a JSON string under
``__attrs__``) and the returned path ends in ``.npz``.
"""
from __future__ import annotations

import json

import numpy as np


def _attrs(solver):
    g, m = solver.g, solver.m
    a = {"x": np.asarray(g.x), "y": np.asarray(g.y), "z": np.asarray(g.z)}
    for k in ("sdx", "sdy", "sdz", "fdx", "fdy", "fdz"):
        a[k] = np.asarray(getattr(g, k))
    a["steps"] = int(solver.t)
    a["dt"] = float(m.dt)
    a["prim_material"] = str(m.primary["name"]) if m.primary else ""
    a["sec_material"] = str(m.secondary["name"]) if m.secondary else ""
    a["solver_cfg"] = json.dumps(solver.cfg)
    a["record_every"] = int(solver.record_every)
    a["dt_record"] = float(m.dt) * max(int(solver.record_every), 1)
    return a


def write_results(path, solver):
    surf = solver.surface if solver.surface is not None else np.zeros((0, solver.g.x.size, solver.g.y.size))
    uz_rec = np.ascontiguousarray(np.transpose(surf, (1, 2, 0))[:, :, None, :])
    data = {"uz": uz_rec, "ux": solver.g.ux, "uy": solver.g.uy, "uz_final": solver.g.uz}
    attrs = _attrs(solver)
    try:
        import h5py  # type: ignore
    except ImportError:
        h5py = None
    if h5py is not None:
        with h5py.File(path, mode="w") as hdf:
            for k, v in data.items():
                hdf.create_dataset(k, data=v)
            for k, v in attrs.items():
                hdf.attrs[k] = v
        return str(path)
    out = str(path) if str(path).endswith(".npz") else str(path) + ".npz"
    js = {k: (v.tolist() if isinstance(v, np.ndarray) else v) for k, v in attrs.items()}
    np.savez(out, __attrs__=np.array(json.dumps(js)), **data)
    return out


def read_results(path):
    """(datasets dict, attrs dict) from a file written by write_results."""
    if str(path).endswith(".npz"):
        z = np.load(path, allow_pickle=False)
        attrs = json.loads(str(z["__attrs__"]))
        return {k: z[k] for k in z.files if k != "__attrs__"}, attrs
    import h5py  # type: ignore
    with h5py.File(path, "r") as hdf:
        return {k: hdf[k][...] for k in hdf.keys()}, dict(hdf.attrs)
