"""Served requests against the same requests run alone: each surface trace
is bit-identical (tolerance 0), whatever else was on the GPU meanwhile,
including requests that reuse a pooled simulation of an earlier one."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _requests():
    from phonomena_gb300 import serve
    from phonomena_gb300.crystal import CrystalSpec

    rng = np.random.default_rng(7)
    cells = [(24, 20, 12), (40, 36, 20), (24, 20, 12), (32, 48, 16), (40, 36, 20), (24, 20, 12), (56, 30, 18),
             (32, 48, 16)]
    out, t = [], 0.0
    for q, c in enumerate(cells):
        steps = int(rng.integers(20, 90))
        spec = CrystalSpec(cells=c, lattice=8, radius=(0.2, 0.4), tungsten_frac=0.25, seed=100 + q,
                           freq=float(rng.uniform(20e6, 60e6)), steps=steps)
        t += float(rng.exponential(0.002))
        out.append(serve.Request(q, spec, steps, t, record_every=5))
    return out


@pytest.mark.parametrize("precision,streams", [("f32k", 0), ("f64", 0), ("f32k", 2)])
def test_served_equals_alone(gpu_lib, precision, streams):
    from phonomena_gb300 import serve
    from phonomena_gb300.device import DeviceSimulation

    reqs = _requests()
    be = serve.GpuBackend(precision=precision, capacity=3, max_steps=120, streams=streams)
    budget = 3.2 * be.footprint((57, 49, 21), 120, 5)  # forces queueing and pool eviction
    srv = serve.Server(be, budget_bytes=budget, capacity=3, chunk=24)
    streamed = []
    res = srv.run(reqs, realtime=True)
    srv.close()
    assert srv.stats.peak_bytes <= budget
    assert sorted(r.rid for r in res) == list(range(len(reqs)))
    assert any(len(v) for v in be.pool.values())  # the pool was used
    be.close()
    for r in res:
        streamed.append(r.rid)
        p = serve.prepare(reqs[r.rid])
        with DeviceSimulation(p.spacing, p.ids, p.table, p.dt, precision=precision, surface_mode="corrected",
                              max_steps=p.req.steps, record_every=5) as sim:
            sim.set_source(p.source)
            sim.step(p.req.steps)
            sim.sync()
            alone = sim.read_surface()
        assert r.surface.shape == alone.shape
        assert np.array_equal(r.surface, alone), f"request {r.rid} differs from its alone run"
