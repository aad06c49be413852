"""Mesh and material inputs: a host-side mirror of phonomena's Grid/Material.

The GPU solver reads only what the reference's solver reads from these
objects: node coordinates and SI conversion (-> full and staggered spacing
arrays, simulation/grid.py:112-128), the time step
(simulation/material.py:80-93) and per-node material constants.  Material
constants are held compactly as a uint8 id per node plus one table row per
id instead of the reference's (nx, ny, nz, 6, 6) C and (nx, ny, nz) P arrays
(simulation/material.py:49-63); at 288 bytes per node the reference layout
does not fit host memory for the large crystals.

``Grid`` and ``Material`` keep the reference attribute and method names
(init, buildMesh, update, addInclusion, inclusionIndices, setPrimary,
setSecondary, setTimeStep, setConstants, c_max, dt, SI_conversion, ...), so
settings code written for the reference drives them unchanged.
"""
from __future__ import annotations

import copy

import numpy as np

TABLE_COLS = 13
_SEL = [(0, 0), (0, 1), (0, 2), (1, 0), (1, 1), (1, 2), (2, 0), (2, 1), (2, 2), (3, 3), (4, 4), (5, 5)]


def spacing_from_coords(x, y, z, SI):
    """fd = diff(coord * SI); sd = mean of neighbouring fd (simulation/grid.py:112-128)."""
    out = {}
    for ax, c in (("x", x), ("y", y), ("z", z)):
        cs = np.asarray(c, dtype=np.float64) * SI
        fd = cs[1:] - cs[:-1]
        out["fd" + ax] = fd
        out["sd" + ax] = (fd[1:] + fd[:-1]) / 2.0
    return out


def table_row(C, rho):
    """Table row from a 6x6 stiffness matrix (Pa) and a density (kg/m^3)."""
    C = np.asarray(C, dtype=np.float64)
    return np.array([C[a, b] for a, b in _SEL] + [float(rho)], dtype=np.float64)


def ids_from_CP(C, P):
    """Compress per-node (nx, ny, nz, 6, 6) C and (nx, ny, nz) P into ids + table."""
    rows = np.stack([C[..., a, b] for a, b in _SEL] + [P], axis=-1).reshape(-1, TABLE_COLS)
    table, inv = np.unique(rows, axis=0, return_inverse=True)
    if table.shape[0] > 256:
        raise ValueError("more than 256 distinct materials")
    return inv.reshape(P.shape).astype(np.uint8), table


def _append_sorted(arr, values):
    values = np.setdiff1d(values, arr)
    arr = np.append(arr, values)
    arr.sort()
    return arr


class Grid:
    """Rectilinear mesh (mirror of simulation/grid.py:29-303).

    Uniform meshes are built here; a non-uniform mesh is given by assigning
    ``x``, ``y``, ``z`` node coordinates directly (e.g. copied from a
    reference Grid) before ``update()``.
    """

    def __init__(self):
        self.max_dx = 1
        self.max_dy = 1
        self.max_dz = 1
        self.min_d = 1
        self.slope = 1
        self.SI_conversion = 1
        self.x = np.array((), dtype=np.float64)
        self.y = np.array((), dtype=np.float64)
        self.z = np.array((), dtype=np.float64)
        self.targets = []  # (x, y, z, r) cylinders from z=0 down to z
        self.ux = self.uy = self.uz = None
        self._fixed_coords = False

    def init(self, size_x, size_y, size_z, fn="linear"):
        self.size_x, self.size_y, self.size_z = int(size_x), int(size_y), int(size_z)
        self.buildMesh()
        self.update()

    def set_coordinates(self, x, y, z):
        """Use explicit node coordinates (non-uniform meshes)."""
        self.x = np.asarray(x, dtype=np.float64).copy()
        self.y = np.asarray(y, dtype=np.float64).copy()
        self.z = np.asarray(z, dtype=np.float64).copy()
        self._fixed_coords = True

    def buildMesh(self, *args, **kwargs):
        """Uniform mesh as the reference builds it without inclusions
        (end points plus closestFit's linspace, simulation/grid.py:245-301)."""
        if self._fixed_coords:
            return
        if self.targets and (self.min_d != self.max_dx or self.min_d != self.max_dy):
            raise NotImplementedError("inclusion-refined meshes: pass coordinates with set_coordinates()")
        for ax, size, md in (("x", self.size_x, self.max_dx), ("y", self.size_y, self.max_dy)):
            mesh = _append_sorted(np.array((), dtype=np.float64), 0)
            mesh = _append_sorted(mesh, size)
            n = int(abs(size - 0) / md)
            if n > 0:
                mesh = _append_sorted(mesh, np.linspace(0, size, n + 1, dtype=float))
            setattr(self, ax, mesh)
        n = int(self.size_z / self.max_dz)
        self.z = np.linspace(0, self.size_z, n + 1, dtype=float)

    def update(self):
        sp = spacing_from_coords(self.x, self.y, self.z, self.SI_conversion)
        nx, ny, nz = self.x.size, self.y.size, self.z.size
        self.fdx = sp["fdx"].reshape(nx - 1, 1, 1)
        self.fdy = sp["fdy"].reshape(1, ny - 1, 1)
        self.fdz = sp["fdz"].reshape(1, 1, nz - 1)
        self.sdx = sp["sdx"].reshape(nx - 2, 1, 1)
        self.sdy = sp["sdy"].reshape(1, ny - 2, 1)
        self.sdz = sp["sdz"].reshape(1, 1, nz - 2)

    def spacing(self):
        return {k: np.ravel(getattr(self, k)).copy() for k in ("fdx", "fdy", "fdz", "sdx", "sdy", "sdz")}

    @property
    def shape(self):
        return (self.x.size, self.y.size, self.z.size)

    def addInclusion(self, x, y, r, z=None):
        x, y, r = float(x), float(y), float(r)
        if z is None:
            z = self.size_z
        self.targets.append((x, y, float(z), r))

    def clearInclusions(self):
        self.targets = []

    def inclusionIndices(self):
        """(yx, z) index pairs of nodes inside each cylinder (simulation/grid.py:158-175).

        The reference's loop assigns its z selection to the name that held
        the node coordinates (grid.py:174), so only the first inclusion
        compares coordinates with its depth; each later one compares the
        previous selection's positions.  Kept as is: results must match."""
        out = []
        X, Y = np.meshgrid(self.x, self.y)
        zsel = self.z
        for tx, ty, tz, tr in self.targets:
            R = np.sqrt(np.square(X - np.float32(tx)) + np.square(Y - np.float32(ty)))
            yx = np.array(np.where(R < np.float32(tr))).transpose()
            zsel = np.array(np.where(zsel <= np.float32(tz))).flatten()
            out.append((yx, zsel))
        return out

    def freezeData(self):
        return copy.copy(self)


class Material:
    """Material constants (mirror of simulation/material.py:22-93) held as ids + table."""

    def __init__(self):
        self.primary = None
        self.primary_key = None
        self.secondary = None
        self.secondary_key = None
        self.c_max = 0.5
        self.dt = 0
        self.ids = None
        self.table = None
        self._custom = None

    def init(self, grid, properties):
        self.grid = grid
        self.properties = dict(copy.deepcopy(properties))
        for val in self.properties.values():
            val["c"] = np.array(val["c"]) * 1e10
        keys = list(self.properties.keys())
        self.setPrimary(keys[0])
        self.setSecondary(keys[0])

    def setPrimary(self, m):
        if m not in self.properties:
            raise KeyError(m)
        self.primary, self.primary_key = self.properties[m], m

    def setSecondary(self, m):
        if m not in self.properties:
            raise KeyError(m)
        self.secondary, self.secondary_key = self.properties[m], m

    def set_ids(self, ids, names):
        """Assign materials per node: ids (nx, ny, nz) index ``names`` (property keys)."""
        self._custom = (np.asarray(ids, dtype=np.uint8), list(names))

    def update(self):
        self.setTimeStep()
        self.setConstants()

    def setTimeStep(self):
        """CFL step over primary and secondary (simulation/material.py:80-93),
        including its second multiplication by SI_conversion."""
        g = self.grid
        fds = [np.ravel(getattr(g, k)) for k in ("fdx", "fdy", "fdz")]

        def calc(c, p):
            vl = np.sqrt(c[0][0] / p)
            vt = np.sqrt(c[3][3] / p)
            vmax = max((vl, vt))
            dxmin = min((np.amin(fds[0]), np.amin(fds[1]), np.amin(fds[2]))) * g.SI_conversion
            return self.c_max * dxmin / vmax

        self.dt = min((calc(self.primary["c"], self.primary["p"]), calc(self.secondary["c"], self.secondary["p"])))

    def setConstants(self):
        g = self.grid
        shape = (g.x.size, g.y.size, g.z.size)
        if self._custom is not None:
            ids, names = self._custom
            if ids.shape != shape:
                raise ValueError(f"material ids {ids.shape} do not match the mesh {shape}")
            self.ids = ids
            self.table = np.stack([table_row(self.properties[n]["c"], self.properties[n]["p"]) for n in names])
            return
        ids = np.zeros(shape, dtype=np.uint8)
        for yx, zi in g.inclusionIndices():
            for yy, xx in yx:
                ids[xx, yy, zi] = 1
        self.ids = ids
        self.table = np.stack([table_row(self.primary["c"], self.primary["p"]),
                               table_row(self.secondary["c"], self.secondary["p"])])


def solver_inputs(grid, material):
    """(spacing dict, ids, table, dt) from either this module's Grid/Material
    or the reference's (which carry the per-node C and P arrays)."""
    spacing = {k: np.ravel(np.asarray(getattr(grid, k), dtype=np.float64)).copy()
               for k in ("fdx", "fdy", "fdz", "sdx", "sdy", "sdz")}
    if getattr(material, "ids", None) is not None and getattr(material, "table", None) is not None:
        ids, table = material.ids, material.table
    else:
        ids, table = ids_from_CP(np.asarray(material.C), np.asarray(material.P))
    return spacing, ids, table, float(material.dt)


def inclusion_inputs(grid, material):
    """(spacing dict, table, dt, targets) for building the material ids on the
    device (phono_set_inclusions) from a Grid with inclusions and a
    two-material Material, this module's or the reference's: table row 0 is
    the primary material (host), row 1 the secondary (inclusions).  Only the
    time step is computed on the host (Material.setTimeStep,
    simulation/material.py:80-93); the per-node constants of
    Material.setConstants (material.py:55-63) are not built.  None when the
    material does not follow that model (ids assigned per node)."""
    if getattr(material, "_custom", None) is not None:
        return None
    if getattr(material, "primary", None) is None or getattr(material, "secondary", None) is None:
        return None
    if not hasattr(grid, "targets"):
        return None
    material.setTimeStep()
    spacing = {k: np.ravel(np.asarray(getattr(grid, k), dtype=np.float64)).copy()
               for k in ("fdx", "fdy", "fdz", "sdx", "sdy", "sdz")}
    table = np.stack([table_row(material.primary["c"], material.primary["p"]),
                      table_row(material.secondary["c"], material.secondary["p"])])
    return spacing, table, float(material.dt), grid.targets
