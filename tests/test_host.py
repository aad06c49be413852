"""Host-side logic on CPU: input mirror, C-ABI exports, plugin discovery."""
import importlib.util
import re
import sys
from pathlib import Path

import numpy as np
import pytest

import golden_cases as G

ROOT = Path(__file__).resolve().parents[1]


def test_testdefaults_mirror_matches_reference_inputs():
    from phonomena_gb300.base import TestDefaults

    d = G.load("testdefaults_ricker")
    g, m = TestDefaults.make()
    g.buildMesh()
    g.update()
    m.update()
    for k in ("fdx", "fdy", "fdz", "sdx", "sdy", "sdz"):
        assert np.array_equal(np.ravel(getattr(g, k)), d[k]), k
    assert m.dt == d["dt"]
    assert np.array_equal(np.unique(m.table, axis=0), d["table"])


@pytest.mark.parametrize("name,seed,tungsten", [("config1_void_corrected", 0, False),
                                                ("config1_tungsten_ref", 1, True)])
def test_crystal_mirror_matches_reference_inputs(name, seed, tungsten):
    from phonomena_gb300 import crystal

    d = G.load(name)
    spec = crystal.config1(seed=seed, holes_are_tungsten=tungsten)
    g, m = crystal.build(spec)
    for k in ("fdx", "fdy", "fdz", "sdx", "sdy", "sdz"):
        assert np.array_equal(g.spacing()[k], d[k]), k
    assert m.dt == d["dt"]
    # same per-node constants (the reference table is sorted and unused rows dropped)
    assert np.array_equal(m.table[m.ids], d["table"][d["ids"]])
    assert np.array_equal(crystal.sin_source(spec.freq, m.dt, spec.steps), d["src"])


def test_nonuniform_coordinates_give_reference_spacings():
    from phonomena_gb300.model import Grid

    d = G.load("nonuniform_json")
    g = Grid()
    g.SI_conversion = d["SI"]
    g.set_coordinates(d["x"], d["y"], d["z"])
    g.update()
    for k in ("fdx", "fdy", "fdz", "sdx", "sdy", "sdz"):
        assert np.array_equal(g.spacing()[k], d[k]), k


def test_ids_from_CP_roundtrip():
    from phonomena_gb300.model import ids_from_CP

    rng = np.random.default_rng(3)
    C = rng.normal(size=(3, 6, 6))
    P = np.array([1.0, 2.0, 3.0])
    ids = rng.integers(0, 3, size=(4, 5, 6))
    ids2, table = ids_from_CP(C[ids], P[ids])
    assert np.array_equal(table[ids2][..., 12], P[ids])
    assert np.array_equal(table[ids2][..., 9], C[ids][..., 3, 3])


def test_ricker_source_matches_reference_expression():
    from phonomena_gb300 import crystal

    d = G.load("testdefaults_ricker")
    assert np.array_equal(crystal.ricker_source(100, d["dt"], 10), d["src"])


def _declared_symbols():
    text = (ROOT / "include" / "phono.h").read_text()
    return sorted(set(re.findall(r"\b(phono_[a-z_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    """Build libphono_gpu.so (nvcc cross-compiles without a GPU), load it, check exports."""
    import ctypes

    from phonomena_gb300 import _lib, build

    lib = build.build()
    L = ctypes.CDLL(str(lib))
    declared = _declared_symbols()
    assert declared, "no declarations parsed"
    for name in declared:
        assert hasattr(L, name), f"{name} declared in include/phono.h but not exported"
    assert set(_lib.EXPORTS) >= set(declared)
    L.phono_abi_version.restype = ctypes.c_int
    assert L.phono_abi_version() == 2


def test_plugin_is_discoverable_like_common_findSolvers(tmp_path, monkeypatch):
    """Mimic phonomena/common.py:88-110: import simulation.solvers.<module>, read Solver().name."""
    pkg = tmp_path / "simulation" / "solvers"
    pkg.mkdir(parents=True)
    (tmp_path / "simulation" / "__init__.py").write_text("")
    (pkg / "__init__.py").write_text("")
    (pkg / "solver_gb300.py").write_text("from phonomena_gb300.solver_gb300 import *  # noqa\n"
                                         "from phonomena_gb300.solver_gb300 import Solver, cfg  # noqa\n")
    monkeypatch.syspath_prepend(str(tmp_path))
    for mod in [m for m in sys.modules if m == "simulation" or m.startswith("simulation.")]:
        monkeypatch.delitem(sys.modules, mod)
    mod = __import__("simulation.solvers.solver_gb300", fromlist=["Solver"])
    s = getattr(mod, "Solver")()
    assert s.name == "gb300"
    assert {"wave", "wave_args", "write_mode", "precision", "record_every"} <= set(s.cfg)
    import json
    json.dumps(s.cfg)  # cfg stays JSON-serialisable (common.py:178, json.dump of solver.cfg in saveSettings)


def test_output_npz_schema(tmp_path):
    from types import SimpleNamespace

    from phonomena_gb300.base import TestDefaults
    from phonomena_gb300.output import read_results, write_results

    g, m = TestDefaults.make()
    g.update()
    m.update()
    nx, ny, nz = g.shape
    g.ux, g.uy, g.uz = np.zeros((nx - 1, ny, nz)), np.zeros((nx, ny - 1, nz)), np.zeros((nx, ny, nz - 1))
    s = SimpleNamespace(g=g, m=m, t=10, cfg={"wave": "ricker"}, record_every=2, volume=None,
                        surface=np.arange(5 * nx * ny, dtype=np.float64).reshape(5, nx, ny),
                        material_ids=lambda: m.ids, material_table=lambda: m.table)
    path = write_results(tmp_path / "out.hdf", s)
    data, attrs = read_results(path)
    assert data["uz"].shape == (nx, ny, 1, 5)
    assert np.array_equal(data["uz"][:, :, 0, 3], s.surface[3])
    assert "ux" not in data and data["ux_final"].shape == (nx - 1, ny, nz)
    # the time step of the record axis is what analysis.spectrum reads (analysis.py:61-65)
    assert attrs["dt"] == m.dt * 2 and attrs["dt_step"] == m.dt and attrs["record_every"] == 2
    assert attrs["steps"] == 5 and attrs["solver_steps"] == 10 and attrs["layout"] == "surface"
    assert np.asarray(attrs["fdx"]).shape == (nx - 1, 1, 1)  # spectrum reads attrs["fdx"][:, 0, 0] for ux
    assert data["density"].shape == (nx, ny, nz) and data["material_ids"].shape == (nx, ny, nz)
    for k in ("x", "y", "z", "sdx", "fdz", "steps", "dt", "prim_material", "sec_material", "solver_cfg"):
        assert k in attrs
    vol = {"ux": np.ones((nx - 1, ny, nz, 3)), "uy": np.ones((nx, ny - 1, nz, 3)), "uz": np.ones((nx, ny, nz - 1, 3))}
    s.volume, s.record_every = vol, 1
    data, attrs = read_results(write_results(tmp_path / "vol.hdf", s))
    assert attrs["layout"] == "volume" and attrs["dt"] == m.dt and attrs["steps"] == 3
    for k, v in vol.items():
        assert data[k].shape == v.shape


def test_footprint_is_the_padded_layout():
    """phono_footprint (host only, no device call) against the padded layout:
    planes -1..nx, rows -1..ny, z rows of 128 bytes after an 8-float front pad."""
    from phonomena_gb300.device import footprint

    def r(b):
        return (b + 511) // 512 * 512

    nx, ny, nz, steps, rec = 30, 20, 10, 100, 10
    row = -(-(8 + nz + 1) // 32) * 32  # floats per z row
    fe = (nx + 2) * (ny + 2) * row
    want = 3 * r(fe * 4 * 3 * 2)  # u (2 buffers), v, c: three components each
    for n in (nx - 1, ny - 1, nz - 1, nx - 2, ny - 2, nz - 2):
        want += r((n + 3) * 4) + r(n * 8)  # device spacings carry 1 + 2 pad values
    want += r((nx + 2) * (ny + 2) * (-(-(8 + nz + 1) // 16) * 16))  # ids
    want += r(256 * 16 * 4) + r(256 * 13 * 8) + r(steps * 8) + r(steps // rec * nx * ny * 4)
    want += r(8) + r(16 * 1024) + r(16)
    assert footprint((nx, ny, nz), "f32k", steps, rec) == want
    assert footprint((nx, ny, nz), "f64", steps, 0) < footprint((nx, ny, nz), "f64v", steps, 0)
    with pytest.raises(Exception):
        footprint((2, 5, 5), "f32k", 10, 1)


def test_crystal_holes_clear_the_absorbing_faces():
    """No void or inclusion node in the two node layers next to x = N, y = 0, y = N."""
    from phonomena_gb300 import crystal

    for spec in crystal.config4_specs(n=24, seed=3, steps=10):
        ids = crystal.material_ids(spec)
        assert not ids[-2:].any() and not ids[:, :2].any() and not ids[:, -2:].any(), spec.cells
        assert ids.any()  # the lattice is still there


def test_listed_segment_candidates_cover_the_planes():
    """The tuner's listed x segments add up to nx - 1 planes, fit the kernel's
    64-entry table and end with their shortening tail."""
    from phonomena_gb300 import autotune

    for shape in ((257, 257, 129), (1025, 1025, 257), (65, 65, 33), (97, 161, 49), (9, 9, 9)):
        for tj, xs in autotune.candidates_for(shape):
            assert tj in autotune.TILE_J
            if isinstance(xs, tuple):
                assert sum(xs) == shape[0] - 1 and len(xs) <= 64 and min(xs) >= 1
                assert any(xs[-len(t):] == t for t in autotune.TAILS)
            elif xs < 0:  # tapered: the launch describes them by table too
                assert autotune.tapered_count(shape[0] - 1, -xs) <= 64
    # 1024 planes: -16 would take 66 segments and is left out
    assert autotune.tapered_count(1024, 16) == 66
    assert all(xs != -16 for _, xs in autotune.candidates_for((1025, 1025, 257)))
    assert autotune.tapered_count(256, 28) == 12 and autotune.tapered_count(3, 8) == 3
    assert autotune.listed_segments(256, 30, (16, 12, 8, 6, 4)) == (30,) * 7 + (16, 12, 8, 6, 4)
    assert autotune.listed_segments(40, 36, (16, 12, 8, 6, 4)) is None
