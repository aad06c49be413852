"""Generate the golden fixtures of tests/golden/ by running the reference solver.

Run from the repository root where the phonomena sources are available
(the baseline/_ref install made by oracle/install_reference.py, or
$PHONO_REFERENCE_ROOT):

    python tests/golden/make_golden.py                 # every case
    python tests/golden/make_golden.py fine_json       # named settings-file cases only

Each case runs the reference's unmodified ``solver_default`` through
``oracle/ref_harness.py`` (``write_mode='off'``) and stores its inputs (node
coordinates, SI conversion, spacings, material ids + table, dt, source
samples, modes) and outputs: the final ux, uy, uz and the uz[:, :, 0]
surface records, either in full (small cases) or as SHA-256 digests of
their little-endian float64 bytes plus norms (large cases).  For two cases
the reference ``solver_threading`` is run too and must agree bit for bit.
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import ref_harness as H  # noqa: E402
from phonomena_gb300 import crystal  # noqa: E402

OUT = Path(__file__).resolve().parent


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


def mats3():
    return [dict(crystal.HOST), dict(crystal.VOID), dict(crystal.TUNGSTEN)]


def uniform_case(cells, ids, steps, freq=42e6, dx=10e-6, **kw):
    g, m = H.make_uniform_case(cells, dx, mats3(), ids, c_max=0.5 / dx, primary=0, secondary=2)
    return H.run_reference(g, m, steps, wave="sin", wave_args={"f": freq}, **kw)


def save(name, out, meta, full=True, check_threading=None):
    rec = dict(meta)
    arrays = {k: out[k] for k in ("x", "y", "z", "fdx", "fdy", "fdz", "sdx", "sdy", "sdz", "ids", "table", "src")}
    arrays["dt"] = np.array(out["dt"])
    arrays["SI"] = np.array(out["SI"])
    assert out["dt2"] == out["dt"] * out["dt"], "dt**2 differs from dt*dt"
    if full:
        for k in ("ux", "uy", "uz", "surf"):
            arrays[k] = out[k]
    for k in ("ux", "uy", "uz", "surf"):
        rec[f"sha256_{k}"] = digest(out[k])
        rec[f"l2_{k}"] = float(np.linalg.norm(out[k]))
        rec[f"max_{k}"] = float(np.abs(out[k]).max()) if out[k].size else 0.0
    if check_threading is not None:
        for k in ("ux", "uy", "uz", "surf"):
            assert np.array_equal(out[k], check_threading[k]), f"threading solver differs in {k}"
        rec["threading_bitwise_equal"] = True
    arrays["meta"] = np.array(json.dumps(rec))
    np.savez_compressed(OUT / f"{name}.npz", **arrays)
    print(name, {k: v for k, v in rec.items() if k.startswith("max_")})


def settings_case(name, rel_path, steps):
    """A case from one of the reference's own settings files, run as
    common.loadSettings would set it up (mesh, inclusions, materials, courant)."""
    g, m, cfg = H.load_settings_case(H.REF_ROOT / rel_path)
    out = H.run_reference(g, m, steps, wave=cfg["simulation"]["cfg"]["wave"],
                          wave_args=cfg["simulation"]["cfg"]["wave_args"], record_every=5)
    save(name, out, dict(steps=steps, record_every=5, wave=cfg["simulation"]["cfg"]["wave"],
                         surface_mode="reference", bc="absorbing", source_mode="line", settings=rel_path),
         full=out["ux"].size < 20000)


def main(only=None):
    rng = np.random.default_rng(20261203)
    R = H.import_reference()
    if only:  # only the named cases from the reference's settings files
        for name, rel_path, steps in SETTINGS_CASES:
            if name in only:
                settings_case(name, rel_path, steps)
        return

    # A. the reference's own test setup (base_solver.py:28-70, test_solvers.py:18-23)
    TD = R.base_solver.TestDefaults
    out = H.run_reference(TD.g, TD.m, 10, wave="ricker", wave_args={"f": 100}, record_every=2)
    save("testdefaults_ricker", out, dict(steps=10, record_every=2, wave="ricker", surface_mode="reference",
                                         bc="absorbing", source_mode="line"))

    # B-D. small 3-material crystal, three mode combinations
    cells = (7, 5, 4)
    ids = rng.integers(0, 3, size=tuple(c + 1 for c in cells)).astype(np.uint8)
    ids[0, 0, 0] = 0
    for name, sm, bc in (("small3_ref", "reference", "reference"), ("small3_corrected", "corrected", "reference"),
                         ("small3_rigid", "reference", "rigid")):
        out = uniform_case(cells, ids, 40, surface_mode=sm, bc=bc, record_every=5)
        thr = None
        if name == "small3_ref":
            thr = H.run_reference(*H.make_uniform_case(cells, 10e-6, mats3(), ids, 0.5 / 10e-6, 0, 2), 40,
                                  wave="sin", wave_args={"f": 42e6}, record_every=5, solver="threading")
        save(name, out, dict(steps=40, record_every=5, wave="sin", surface_mode=sm,
                             bc="rigid" if bc == "rigid" else "absorbing", source_mode="line"), check_threading=thr)

    # E-F. degenerate sizes: 3 x 3 x 3 nodes, and a grid 3 nodes wide in y
    for name, cells in (("tiny", (2, 2, 2)), ("thin_y", (9, 2, 3))):
        ids = rng.integers(0, 3, size=tuple(c + 1 for c in cells)).astype(np.uint8)
        ids[0, 0, 0] = 0
        out = uniform_case(cells, ids, 25, record_every=5)
        save(name, out, dict(steps=25, record_every=5, wave="sin", surface_mode="reference", bc="absorbing",
                             source_mode="line"))

    # G-H. config-1 geometry (40 x 40 x 20 cells, 500 steps)
    spec = crystal.config1(seed=1, holes_are_tungsten=True)
    ids = crystal.material_ids(spec)
    out = uniform_case(spec.cells, ids, 500, record_every=10)
    thr = H.run_reference(*H.make_uniform_case(spec.cells, 10e-6, mats3(), ids, 0.5 / 10e-6, 0, 2), 500,
                          wave="sin", wave_args={"f": 42e6}, record_every=10, solver="threading")
    save("config1_tungsten_ref", out, dict(steps=500, record_every=10, wave="sin", surface_mode="reference",
                                           bc="absorbing", source_mode="line", crystal="config1 seed 1, tungsten"),
         full=False, check_threading=thr)
    spec = crystal.config1(seed=0)
    ids = crystal.material_ids(spec)
    out = uniform_case(spec.cells, ids, 500, surface_mode="corrected", record_every=10)
    save("config1_void_corrected", out, dict(steps=500, record_every=10, wave="sin", surface_mode="corrected",
                                             bc="absorbing", source_mode="line", crystal="config1 seed 0, voids"),
         full=False)

    # I-K. the reference's own settings files: a non-uniform mesh, a fine mesh
    # (0.3-cell spacing) and the application's default, GaAs with Au inclusions
    for name, rel_path, steps in SETTINGS_CASES:
        settings_case(name, rel_path, steps)


SETTINGS_CASES = (("nonuniform_json", "tests/data/nonuniform.json", 30),
                  ("fine_json", "tests/data/fine.json", 30),
                  ("default_json", "data/default.json", 40))

if __name__ == "__main__":
    main(only=set(sys.argv[1:]) or None)
