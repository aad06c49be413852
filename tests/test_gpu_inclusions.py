"""phono_set_inclusions: the reference's inclusion fill built on the GPU.

The ids the device builds from node coordinates and the inclusion list must
equal, node for node, the material the reference's Material.setConstants
assigned (tests/golden/materials/inclusions.npz, made from phonomena's own
Grid / Material for its three settings files and two meshes with inclusions
of different depths).  And a simulation of data/default.json with
device-built ids must reproduce the reference solver's fields bit for bit
(the default_json golden fixture).
"""
import numpy as np
import pytest

import golden_cases as G
from test_inclusions import CASES

pytestmark = pytest.mark.gpu

TABLE2 = np.array([[1.188e11, 5.87e10, 5.38e10, 5.87e10, 1.188e11, 5.38e10, 5.87e10, 5.38e10, 1.188e11,
                    5.94e10, 5.94e10, 5.94e10, 5307.0],
                   [1.925e11, 1.63e11, 1.63e11, 1.63e11, 1.925e11, 1.63e11, 1.63e11, 1.63e11, 1.925e11,
                    4.24e10, 4.24e10, 4.24e10, 19300.0]])


def _sim(c, table=TABLE2, dt=1e-9, **kw):
    from phonomena_gb300.device import DeviceSimulation
    from phonomena_gb300.model import spacing_from_coords

    sp = spacing_from_coords(c["x"], c["y"], c["z"], 1e-6)
    ids0 = np.zeros((c["x"].size, c["y"].size, c["z"].size), dtype=np.uint8)
    return DeviceSimulation(sp, ids0, table, dt, precision="f64", **kw)


@pytest.mark.parametrize("name", sorted(CASES))
def test_device_inclusion_ids_equal_reference(gpu_lib, name):
    c = CASES[name]
    targets = np.stack([c["tx"], c["ty"], c["tz"], c["tr"]], axis=1)
    with _sim(c, max_steps=1) as sim:
        sim.set_inclusions(c["x"], c["y"], c["z"], targets, TABLE2, inside=1, host=0)
        got = sim.download_materials()
    assert got.shape == c["ids"].shape
    assert np.array_equal(got, c["ids"]), f"{name}: {int((got != c['ids']).sum())} nodes differ"


def test_device_inclusions_per_target_ids_last_wins(gpu_lib):
    """Each inclusion with its own id: where they overlap, the later one
    wins (the reference overwrites in list order); checked against the
    oracle's restatement."""
    from oracle.inclusions import inclusion_ids

    c = CASES["depths_dz_half"]
    ids = np.arange(1, c["tx"].size + 1, dtype=np.uint8)
    table = np.vstack([TABLE2[0]] + [TABLE2[1]] * c["tx"].size)
    want = inclusion_ids(c["x"], c["y"], c["z"], c["tx"], c["ty"], c["tz"], c["tr"], ids=ids)
    assert len(np.unique(want)) == c["tx"].size + 1
    targets = np.stack([c["tx"], c["ty"], c["tz"], c["tr"]], axis=1)
    with _sim(c, table=table, max_steps=1) as sim:
        sim.set_inclusions(c["x"], c["y"], c["z"], targets, table, host=0, ids=ids)
        assert np.array_equal(sim.download_materials(), want)


def test_device_inclusions_reject_bad_input(gpu_lib):
    from phonomena_gb300._lib import PhonoError

    c = CASES["default_json"]
    targets = np.stack([c["tx"], c["ty"], c["tz"], c["tr"]], axis=1)
    with _sim(c, max_steps=1) as sim:
        with pytest.raises(PhonoError):
            sim.set_inclusions(c["x"][::-1], c["y"], c["z"], targets, TABLE2)  # descending x
        with pytest.raises(PhonoError):
            sim.set_inclusions(c["x"], c["y"], c["z"], targets, TABLE2, inside=2)  # id past the table
        sim.set_inclusions(c["x"], c["y"], c["z"], np.zeros((0, 4)), TABLE2, host=1)  # no inclusions
        assert (sim.download_materials() == 1).all()


def test_default_json_with_device_ids_bit_exact_vs_reference(gpu_lib):
    """data/default.json (GaAs with six Au inclusions): ids built on the GPU,
    F64 leapfrog, the reference solver's final fields and surface records."""
    from phonomena_gb300.device import DeviceSimulation

    d = G.load("default_json")
    c = CASES["default_json"]
    assert np.array_equal(d["x"], c["x"]) and np.array_equal(d["y"], c["y"]) and np.array_equal(d["z"], c["z"])
    # the fixture's table is sorted by value: find the primary (GaAs) and secondary (Au) rows
    host = int(np.argmin(d["table"][:, 12]))
    m = d["meta"]
    sim = DeviceSimulation(G.spacing(d), np.full(d["ids"].shape, host, np.uint8), d["table"], d["dt"],
                           precision="f64", surface_mode=m["surface_mode"], bc=m["bc"],
                           source_mode=m["source_mode"], max_steps=len(d["src"]), record_every=m["record_every"])
    with sim:
        targets = np.stack([c["tx"], c["ty"], c["tz"], c["tr"]], axis=1)
        sim.set_inclusions(c["x"], c["y"], c["z"], targets, d["table"], inside=1 - host, host=host)
        assert np.array_equal(sim.download_materials(), d["ids"])
        sim.set_source(d["src"])
        sim.step(m["steps"])
        sim.sync()
        for key in ("ux", "uy", "uz"):
            assert G.matches(d, key, sim.download(key)), key
        assert G.matches(d, "surf", sim.read_surface())
