"""The reference's inclusion fill on the CPU: the oracle's restatement and the
host mirror (phonomena_gb300.model) against the reference's own result.

tests/golden/materials/inclusions.npz holds, for five meshes, the node coordinates,
the inclusion list as Grid.targets stores it and the material the
reference's Material.setConstants gave each node (made by
tests/golden/make_inclusions.py from phonomena's own Grid / Material).
"""
import json
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden" / "materials" / "inclusions.npz"


def cases():
    z = np.load(GOLDEN, allow_pickle=False)
    names = json.loads(str(z["cases"]))
    return {n: {k: z[f"{n}/{k}"] for k in ("x", "y", "z", "tx", "ty", "tz", "tr", "ids")} for n in names}


CASES = cases()


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_inclusion_ids_equal_reference(name):
    from oracle.inclusions import inclusion_ids

    c = CASES[name]
    got = inclusion_ids(c["x"], c["y"], c["z"], c["tx"], c["ty"], c["tz"], c["tr"])
    assert np.array_equal(got, c["ids"])


@pytest.mark.parametrize("name", sorted(CASES))
def test_host_mirror_inclusion_fill_equals_reference(name):
    from phonomena_gb300.model import Grid, Material, table_row

    c = CASES[name]
    g = Grid()
    g.set_coordinates(c["x"], c["y"], c["z"])
    g.update()
    for x, y, zz, r in zip(c["tx"], c["ty"], c["tz"], c["tr"]):
        g.targets.append((float(x), float(y), float(zz), float(r)))
    m = Material()
    props = {"A": {"name": "A", "c": np.eye(6).tolist(), "p": 1.0}, "B": {"name": "B", "c": (2 * np.eye(6)).tolist(),
                                                                         "p": 2.0}}
    m.init(grid=g, properties=props)
    m.setPrimary("A")
    m.setSecondary("B")
    m.update()
    assert np.array_equal(m.ids, c["ids"])
    assert np.array_equal(m.table[1], table_row(np.array(props["B"]["c"]) * 1e10, 2.0))


def test_golden_exercises_the_depth_rebinding():
    """In depths_dz_half a later inclusion is deeper than the first one in
    coordinates but not in node positions: the reference fills fewer nodes
    than a per-inclusion coordinate test would."""
    from oracle.inclusions import inclusion_ids

    c = CASES["depths_dz_half"]
    naive = np.zeros_like(c["ids"])
    for t in range(c["tx"].size):
        one = inclusion_ids(c["x"], c["y"], c["z"], c["tx"][t:t + 1], c["ty"][t:t + 1], c["tz"][t:t + 1],
                            c["tr"][t:t + 1])
        naive |= one
    assert not np.array_equal(naive, c["ids"])
