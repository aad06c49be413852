"""Seeded synthetic phononic crystals (the benchmark and test inputs).

A crystal is a uniform mesh (spacing ``dx`` metres, ``SI_conversion = dx``)
of a Si-like host with a square lattice (pitch ``a`` cells) of vertical
cylindrical holes running from the surface z=0 down through ``depth`` cells.
Holes are voids (stiffness 0, host density, which keeps the scheme stable)
or tungsten-like inclusions.  Radii and the tungsten choice are drawn from
``numpy.random.default_rng(seed)``.

Material constants (isotropic, C11 = lam + 2 mu, C12 = lam, C44 = mu):
  host      rho 2330 kg/m^3, lam 64 GPa,  mu 80 GPa
  tungsten  rho 19300 kg/m^3, lam 200 GPa, mu 160 GPa
  void      rho 2330 kg/m^3, C = 0
The time step is 0.5 x CFL through the reference's own formula
(simulation/material.py:80-93): ``c_max = courant / SI_conversion`` undoes its
second SI multiplication.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .model import Grid, Material


def isotropic_c(lam_gpa, mu_gpa):
    """6x6 stiffness in units of 1e10 Pa (the reference's JSON convention)."""
    c = np.zeros((6, 6))
    l, m = lam_gpa / 10.0, mu_gpa / 10.0
    c[:3, :3] = l
    for q in range(3):
        c[q, q] = l + 2 * m
        c[q + 3, q + 3] = m
    return c


HOST = {"name": "host", "c": isotropic_c(64.0, 80.0).tolist(), "p": 2330}
TUNGSTEN = {"name": "tungsten", "c": isotropic_c(200.0, 160.0).tolist(), "p": 19300}
VOID = {"name": "void", "c": np.zeros((6, 6)).tolist(), "p": 2330}


@dataclass
class CrystalSpec:
    cells: tuple = (40, 40, 20)     # cells per axis (nodes = cells + 1)
    dx: float = 10e-6               # mesh spacing (m)
    lattice: int = 8                # hole pitch a (cells)
    radius: tuple = (0.3, 0.3)      # radius range as a fraction of a (uniform draw)
    depth: int = 10                 # holes run through z = 0..depth (cells)
    tungsten_frac: float = 0.0      # share of holes that are tungsten instead of void
    holes_are_tungsten: bool = False  # 2-material variant: every hole is tungsten
    seed: int = 0
    courant: float = 0.5
    freq: float = 42e6              # sinusoidal source frequency (Hz)
    steps: int = 500
    record_every: int = 10
    extra: dict = field(default_factory=dict)

    @property
    def nodes(self):
        return tuple(c + 1 for c in self.cells)

    @property
    def n_nodes(self):
        nx, ny, nz = self.nodes
        return nx * ny * nz


def lattice(spec: CrystalSpec):
    """The crystal's hole lattice: pitch, per-cell radii (cells) and material
    ids (0 host, 1 void, 2 tungsten), and the depth of the holes (nodes)."""
    rng = np.random.default_rng(spec.seed)
    a = spec.lattice
    npx, npy = -(-spec.cells[0] // a), -(-spec.cells[1] // a)
    lo, hi = spec.radius
    radii = rng.uniform(lo, hi, size=(npx, npy)) * a
    if spec.holes_are_tungsten:
        kind = np.full((npx, npy), 2, np.uint8)
    else:
        kind = np.where(rng.uniform(size=(npx, npy)) < spec.tungsten_frac, 2, 1).astype(np.uint8)
    # Lattice cells whose hole would cover a node of the two layers at an
    # absorbing face (x = N, y = 0, y = N) stay solid host.  The reference's
    # first-order absorbing faces (simulation/base_solver.py:519-554) use the
    # host's wave speeds and go unstable next to a void or an inclusion: a
    # 128x128x48 crystal with a = 12 grew to max|u| = 1.2e4 after 1500 steps,
    # 4.8 with the cut cells left solid.  The benchmark crystals with whole
    # cells and r <= 0.4a clear the faces and are unchanged by this rule.
    ccx = (np.arange(npx) + 0.5) * a
    ccy = (np.arange(npy) + 0.5) * a
    reach = (ccx[:, None] + radii > spec.cells[0] - 1) | (ccy[None, :] + radii > spec.cells[1] - 1) | \
            (ccy[None, :] - radii < 1)
    kind = np.where(reach, 0, kind).astype(np.uint8)
    return {"pitch": a, "radius": radii, "kind": kind, "depth": spec.depth, "host": 0}


def ids_from_lattice(nodes, lat):
    """(nx, ny, nz) uint8 ids of a hole lattice (the host-side twin of phono_set_lattice)."""
    nx, ny, nz = nodes
    a, radii, kind = lat["pitch"], lat["radius"], lat["kind"]
    npx, npy = radii.shape
    x = np.arange(nx, dtype=np.float64)
    y = np.arange(ny, dtype=np.float64)
    px = np.minimum((x // a).astype(int), npx - 1)
    py = np.minimum((y // a).astype(int), npy - 1)
    cx = (px + 0.5) * a
    cy = (py + 0.5) * a
    d2 = (x - cx)[:, None] ** 2 + (y - cy)[None, :] ** 2
    r = radii[px[:, None], py[None, :]]
    inside = d2 < r * r
    plane = np.where(inside, kind[px[:, None], py[None, :]], lat["host"]).astype(np.uint8)
    ids = np.full((nx, ny, nz), lat["host"], np.uint8)
    kmax = min(lat["depth"], nz - 1)
    ids[:, :, : kmax + 1] = plane[:, :, None]
    return ids


def material_ids(spec: CrystalSpec):
    """(nx, ny, nz) uint8 ids: 0 host, 1 void, 2 tungsten."""
    return ids_from_lattice(spec.nodes, lattice(spec))


def build(spec: CrystalSpec):
    """Grid + Material for a crystal (three property entries: host, void, tungsten)."""
    g = Grid()
    g.SI_conversion = spec.dx
    g.init(*spec.cells)
    m = Material()
    m.init(grid=g, properties={p["name"]: dict(p) for p in (HOST, VOID, TUNGSTEN)})
    m.c_max = spec.courant / spec.dx
    m.setPrimary("host")
    ids = material_ids(spec)
    m.setSecondary("tungsten" if (ids == 2).any() else "host")
    m.set_ids(ids, ["host", "void", "tungsten"])
    m.update()
    return g, m


def sin_source(freq, dt, steps):
    """s(tt) = sin(2 pi f tt dt), evaluated as simulation/base_solver.py:298 does."""
    dt = np.float64(dt)
    return np.array([np.sin(2 * np.pi * freq * tt * dt) for tt in range(steps)], dtype=np.float64)


def ricker_source(freq, dt, steps, source_delay=0):
    """Ricker wavelet of simulation/base_solver.py:310-311."""
    dt = np.float64(dt)
    out = np.empty(steps, np.float64)
    for tt in range(steps):
        arg = (np.pi * freq * (dt * tt - source_delay)) ** 2
        out[tt] = (1 - 2 * arg) * np.exp(-arg)
    return out


# the workloads named by the benchmark configuration
def config1(seed=0, **kw):
    """40x40x20 cells, a=8, voids r=0.3a through the top 10 cells, 42 MHz, 500 steps."""
    return CrystalSpec(cells=(40, 40, 20), lattice=8, radius=(0.3, 0.3), depth=10, seed=seed, steps=500, **kw)


def config2(seed=0, **kw):
    """256x256x128 cells, a=16, r ~ U[0.2a, 0.4a], 25% tungsten, 2000 steps."""
    return CrystalSpec(cells=(256, 256, 128), lattice=16, radius=(0.2, 0.4), depth=10, tungsten_frac=0.25,
                       seed=seed, steps=2000, **kw)


def config3(seed=0, **kw):
    """1024x1024x256 cells (about 268M nodes), as config2, 4000 steps."""
    return CrystalSpec(cells=(1024, 1024, 256), lattice=16, radius=(0.2, 0.4), depth=10, tungsten_frac=0.25,
                       seed=seed, steps=4000, **kw)


def config4_specs(n=64, seed=0, steps=1500):
    """Uneven batch: sizes from {64..192}^2 x {32..96}, a in {8,12,16}, f ~ U[20,60] MHz."""
    rng = np.random.default_rng(seed)
    specs = []
    for q in range(n):
        cx = int(rng.choice([64, 96, 128, 160, 192]))
        cy = int(rng.choice([64, 96, 128, 160, 192]))
        cz = int(rng.choice([32, 48, 64, 96]))
        a = int(rng.choice([8, 12, 16]))
        f = float(rng.uniform(20e6, 60e6))
        specs.append(CrystalSpec(cells=(cx, cy, cz), lattice=a, radius=(0.2, 0.4), depth=10, tungsten_frac=0.25,
                                 seed=int(rng.integers(1 << 31)), freq=f, steps=steps))
    return specs
