"""Result file in the reference writer's schema (simulation/base_solver.py:105-133).

The reference writes the full volume after every step: datasets ``ux``
(nx-1, ny, nz, T), ``uy`` (nx, ny-1, nz, T), ``uz`` (nx, ny, nz-1, T), and
attributes x, y, z, sdx..fdz (in the Grid's 3-D shapes), steps, dt,
prim_material, sec_material, solver_cfg.  Its reader ``analysis.spectrum``
(simulation/analysis.py:44-96) takes the time step of axis 3 from
``attrs["dt"]`` and the number of samples from ``u.shape[3]``.

Two layouts, both with a time axis of ``records`` samples spaced
``attrs["dt"] = dt_step * record_every`` (so that spectrum's frequency axis
is right for sampled output):

* ``volume``: ``ux``, ``uy``, ``uz`` exactly as the reference lays them out,
  one record after every ``record_every``-th step (record_every = 1 gives the
  reference's own file);
* ``surface``: only ``uz`` at the top surface, as a 4-D (nx, ny, 1, records)
  array (read it with ``z_index=0``); the final state is kept in
  ``ux_final``, ``uy_final``, ``uz_final``.

Both also hold ``density`` (nx, ny, nz), ``material_ids`` and
``material_table`` (the solver keeps materials as a uint8 id per node and
one table row per id instead of the per-node 6x6 ``elasticity``), and the
attributes ``dt_step`` (the solver's time step), ``record_every``,
``records``, ``solver_steps``, ``layout``.  ``steps`` is the length of the
time axis, as in the reference.

HDF5 is written with h5py when it is importable; otherwise the same names go
into a NumPy ``.npz`` archive (attributes as a JSON string under
``__attrs__``) and the returned path ends in ``.npz``.
"""
from __future__ import annotations

import json

import numpy as np


def _attrs(solver, records, layout):
    g, m = solver.g, solver.m
    a = {"x": np.asarray(g.x), "y": np.asarray(g.y), "z": np.asarray(g.z)}
    for k in ("sdx", "sdy", "sdz", "fdx", "fdy", "fdz"):
        a[k] = np.asarray(getattr(g, k))
    k_rec = max(int(solver.record_every), 1)
    a["steps"] = int(records)
    a["dt"] = float(m.dt) * k_rec
    a["dt_step"] = float(m.dt)
    a["record_every"] = k_rec
    a["records"] = int(records)
    a["solver_steps"] = int(solver.t)
    a["layout"] = layout
    a["prim_material"] = str(m.primary["name"]) if getattr(m, "primary", None) else ""
    a["sec_material"] = str(m.secondary["name"]) if getattr(m, "secondary", None) else ""
    a["solver_cfg"] = json.dumps(solver.cfg)
    return a


def result_datasets(solver):
    """(datasets, layout) of a finished GB300 solver run."""
    ids, table = solver.material_ids(), solver.material_table()
    common = {"density": table[ids, 12], "material_ids": ids, "material_table": table}
    vol = getattr(solver, "volume", None)
    if vol is not None:
        return {"ux": vol["ux"], "uy": vol["uy"], "uz": vol["uz"], **common}, "volume"
    g = solver.g
    surf = solver.surface if solver.surface is not None else np.zeros((0, g.x.size, g.y.size))
    uz_rec = np.ascontiguousarray(np.transpose(surf, (1, 2, 0))[:, :, None, :])
    return {"uz": uz_rec, "ux_final": g.ux, "uy_final": g.uy, "uz_final": g.uz, **common}, "surface"


def write_results(path, solver):
    data, layout = result_datasets(solver)
    attrs = _attrs(solver, data["uz"].shape[3], layout)
    try:
        import h5py  # type: ignore
    except ImportError:
        h5py = None
    if h5py is not None and hasattr(h5py, "File"):
        with h5py.File(path, mode="w") as hdf:
            for k, v in data.items():
                hdf.create_dataset(k, data=v)
            for k, v in attrs.items():
                hdf.attrs[k] = v
        return str(path)
    out = str(path) if str(path).endswith(".npz") else str(path) + ".npz"
    js = {k: (v.tolist() if isinstance(v, np.ndarray) else v) for k, v in attrs.items()}
    with open(out, "wb") as f:
        np.savez(f, __attrs__=np.array(json.dumps(js)), **data)
    return out


def read_results(path):
    """(datasets dict, attrs dict) from a file written by write_results."""
    if str(path).endswith(".npz"):
        z = np.load(path, allow_pickle=False)
        attrs = json.loads(str(z["__attrs__"]))
        attrs = {k: (np.asarray(v) if isinstance(v, list) else v) for k, v in attrs.items()}
        return {k: z[k] for k in z.files if k != "__attrs__"}, attrs
    import h5py  # type: ignore
    with h5py.File(path, "r") as hdf:
        return {k: hdf[k][...] for k in hdf.keys()}, dict(hdf.attrs)
