"""The allocation-free energy entry point, phono_energy_static.

Some callers cannot call cudaMalloc: applications whose device memory
belongs to another allocator (a framework's caching pool, a reservation made
at start-up) and latency-bound loops that must not take cudaFree's implicit
device synchronisation.  phono_energy_static serves them: it reads
the caller's own device arrays and keeps its partial sums in a static
__device__ array instead of allocating.  These tests call it through the C
ABI on dense copies of a solver state and check it against phono_energy (the
handle's reduction, which uses a cudaMalloc'd buffer), twice in a row,
because every call reuses the same static array.

This file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12  # the two reductions add the same terms in different orders


def _state(precision):
    from phonomena_gb300 import crystal
    from phonomena_gb300.device import DeviceSimulation

    spec = crystal.CrystalSpec(cells=(40, 36, 20), lattice=8, radius=(0.2, 0.4), tungsten_frac=0.25, seed=11,
                               steps=60)
    g, m = crystal.build(spec)
    sim = DeviceSimulation(g.spacing(), m.ids, m.table, m.dt, precision=precision, surface_mode="corrected",
                           max_steps=spec.steps)
    sim.set_source(crystal.sin_source(spec.freq, m.dt, spec.steps))
    sim.step(spec.steps)
    sim.sync()
    return sim, g, m


def _dense_inputs(sim, g, m, precision):
    import torch

    from phonomena_gb300 import _lib

    vel = ("ux_old", "uy_old", "uz_old") if precision == "f64" else ("vx", "vy", "vz")
    keep = {k: torch.from_numpy(np.ascontiguousarray(sim.download(k))).cuda() for k in ("ux", "uy", "uz") + vel}
    keep["mat"] = torch.from_numpy(np.ascontiguousarray(m.ids)).cuda()
    keep["table"] = torch.from_numpy(np.ascontiguousarray(m.table, dtype=np.float64)).cuda()
    for k, v in g.spacing().items():
        keep[k] = torch.from_numpy(np.ascontiguousarray(v, dtype=np.float64)).cuda()
    nx, ny, nz = m.ids.shape
    d = _lib.PhonoEnergyDense(nx, ny, nz, _lib.PRECISIONS[precision],
                              *(keep[k].data_ptr() for k in ("ux", "uy", "uz") + vel),
                              keep["mat"].data_ptr(), keep["table"].data_ptr(),
                              *(keep[k].data_ptr() for k in ("fdx", "fdy", "fdz", "sdx", "sdy", "sdz")),
                              float(m.dt), int(m.table.shape[0]))
    return d, keep


@pytest.mark.parametrize("precision", ["f64", "f32k", "f64v"])
def test_energy_static_matches_allocating_entry_point(gpu_lib, precision):
    import torch

    from phonomena_gb300._lib import check

    sim, g, m = _state(precision)
    ek, es = sim.energy()
    d, keep = _dense_inputs(sim, g, m, precision)
    out = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")
    for _ in range(2):  # the static scratch keeps the last call's partials
        out.fill_(float("nan"))
        torch.cuda.synchronize()
        check(gpu_lib.phono_energy_static(ctypes.byref(d), out.data_ptr(), None))
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert ek > 0 and es > 0
        assert abs(got[0] - ek) <= RTOL * abs(ek), (got, ek)
        assert abs(got[1] - es) <= RTOL * abs(es), (got, es)
    sim.close()


def test_energy_static_rejects_grids_beyond_the_scratch(gpu_lib):
    from phonomena_gb300 import _lib

    d = _lib.PhonoEnergyDense()
    d.nx, d.ny, d.nz, d.precision, d.dt = _lib.ENERGY_STATIC_MAX_NX + 1, 8, 8, 0, 1.0
    for name in ("ux", "uy", "uz", "vx", "vy", "vz", "mat", "table", "fdx", "fdy", "fdz", "sdx", "sdy", "sdz"):
        setattr(d, name, 16)  # never dereferenced: the size check comes first
    rc = gpu_lib.phono_energy_static(ctypes.byref(d), 16, None)
    assert rc == -1
    assert b"PHONO_ENERGY_STATIC_MAX_NX" in gpu_lib.phono_last_error()


def test_energy_static_flags_material_ids_past_the_table(gpu_lib):
    """A material id at or past nmat is not used to index the table: both
    outputs come back NaN (a table of one row, ids up to 2)."""
    import torch

    from phonomena_gb300._lib import check

    sim, g, m = _state("f64")
    d, keep = _dense_inputs(sim, g, m, "f64")
    assert int(m.ids.max()) >= 1
    d.nmat = 1
    out = torch.zeros((2,), dtype=torch.float64, device="cuda")
    check(gpu_lib.phono_energy_static(ctypes.byref(d), out.data_ptr(), None))
    torch.cuda.synchronize()
    assert np.isnan(out.cpu().numpy()).all()
    d.nmat = 0
    assert gpu_lib.phono_energy_static(ctypes.byref(d), out.data_ptr(), None) == -1
    sim.close()
