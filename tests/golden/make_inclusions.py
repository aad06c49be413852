"""Generate tests/golden/materials/inclusions.npz from the reference's own material fill.

Run from the repository root where the phonomena sources are available
(the baseline/_ref install made by oracle/install_reference.py, or
$PHONO_REFERENCE_ROOT):

    python tests/golden/make_inclusions.py

Each case builds a reference ``Grid`` (``init``, ``addInclusion``,
``buildMesh``, ``update``) and ``Material`` (``init``, ``setPrimary``,
``setSecondary``, ``update``) exactly as ``common.loadSettings``
(phonomena/common.py:112-156) does, and stores the node coordinates, the
inclusion list as the reference holds it (``Grid.targets``: float32 x, y, z,
r) and the node material the reference's ``Material.setConstants``
(simulation/material.py:55-63, with ``Grid.inclusionIndices``,
simulation/grid.py:158-175) assigned: 1 where a node got the secondary
material's constants, else 0.

Cases: the three settings files the reference ships (data/default.json,
tests/data/fine.json, tests/data/nonuniform.json) and two inclusion lists
whose depths differ, on a mesh refined in z, which exercise the way
``inclusionIndices`` reuses its ``z`` variable from one inclusion to the next.
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import ref_harness as H  # noqa: E402

OUT = Path(__file__).resolve().parent / "materials" / "inclusions.npz"


def _secondary_mask(m):
    sec_c = np.array(m.secondary["c"])
    sec_p = float(m.secondary["p"])
    return (np.all(m.C == sec_c, axis=(-1, -2)) & (m.P == sec_p)).astype(np.uint8)


def _case_arrays(g, m):
    t = np.asarray(g.targets)
    return dict(x=np.array(g.x, np.float64), y=np.array(g.y, np.float64), z=np.array(g.z, np.float64),
                tx=np.array(t["x"], np.float32) if t.size else np.zeros(0, np.float32),
                ty=np.array(t["y"], np.float32) if t.size else np.zeros(0, np.float32),
                tz=np.array(t["z"], np.float32) if t.size else np.zeros(0, np.float32),
                tr=np.array(t["r"], np.float32) if t.size else np.zeros(0, np.float32),
                ids=_secondary_mask(m))


def settings(rel_path):
    g, m, _ = H.load_settings_case(H.REF_ROOT / rel_path)
    return _case_arrays(g, m)


def layered(size, grid_keys, targets, props_path="data/default.json"):
    """A mesh with inclusions of different depths, built and filled by the reference."""
    R = H.import_reference()
    cfg = json.load(open(H.REF_ROOT / props_path))
    g = R.grid.Grid()
    g.init(*size)
    for k, v in grid_keys.items():
        setattr(g, k, v)
    for x, y, z, r in targets:
        g.addInclusion(x=x, y=y, z=z, r=r)
    g.buildMesh()
    g.update()
    m = R.material.Material()
    m.init(grid=g, properties=cfg["material"]["properties"])
    m.setPrimary("GaAs")
    m.setSecondary("Au")
    m.update()
    return _case_arrays(g, m)


def main():
    H.import_reference()
    cases = {
        "default_json": settings("data/default.json"),
        "fine_json": settings("tests/data/fine.json"),
        "nonuniform_json": settings("tests/data/nonuniform.json"),
        # z refined to half cells (11 z nodes over 5 cells): the first
        # inclusion's depth selects nodes by coordinate, the later ones by
        # node index below the previous selection
        "depths_dz_half": layered((20, 14, 5), dict(min_d=1.0, max_dx=1.0, max_dy=1.0, max_dz=0.5, slope=1.0),
                                  [(5.0, 4.0, 3.2, 2.0), (12.0, 9.0, 5.0, 2.5), (15.0, 5.0, 1.7, 1.5),
                                   (8.0, 8.0, 4.0, 3.0)]),
        "depths_shallow_first": layered((16, 12, 6), dict(min_d=0.5, max_dx=1.0, max_dy=1.0, max_dz=1.0,
                                                          slope=1.0),
                                        [(4.0, 4.0, 2.0, 1.5), (10.0, 7.0, 6.0, 2.0), (6.0, 8.0, 0.5, 2.5)]),
    }
    arrays = {}
    for name, c in cases.items():
        for k, v in c.items():
            arrays[f"{name}/{k}"] = v
        print(name, "nodes", c["ids"].shape, "targets", c["tx"].size, "secondary nodes", int(c["ids"].sum()))
    arrays["cases"] = np.array(json.dumps(list(cases)))
    np.savez_compressed(OUT, **arrays)


if __name__ == "__main__":
    main()
