"""The tile pass's bounded waits: the time-out path runs, reports and recovers.

Every mbarrier wait of the tile pass (the plane copies of the TMA ring) gives
up after a poll budget; the block then sets error bit 2 of the handle's
error word, waits for the copies it did issue and returns, and phono_sync
reports PHONO_ERR_TIMEOUT.  The test hook phono_test_wait_timeout makes that
happen without any fault: blocks arm one plane's barrier and issue no copy
for it (a barrier nothing completes), with a short budget.  Covered: the
one-row tile pass (F64, F32K at tile height 4), the two-row pass (F32K at
heights 8 and 16) and the persistent batch kernel.  After the hook is turned
off and the handle reset, a run equals a clean run bit for bit: the context
and the handle stay usable.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

POLLS = 4096  # about 0.3 ms per wait
STEPS = 24


def _case():
    from phonomena_gb300 import crystal

    spec = crystal.CrystalSpec(cells=(40, 36, 40), lattice=8, radius=(0.2, 0.4), tungsten_frac=0.25, seed=5,
                               steps=STEPS, record_every=4)
    g, m = crystal.build(spec)
    return spec, g, m, crystal.sin_source(spec.freq, m.dt, STEPS)


def _sim(spec, g, m, src, precision, tile_j):
    from phonomena_gb300.device import DeviceSimulation

    sim = DeviceSimulation(g.spacing(), m.ids, m.table, m.dt, precision=precision, surface_mode="corrected",
                           max_steps=STEPS, record_every=spec.record_every, tile_j=tile_j, x_segment=8)
    sim.set_source(src)
    return sim


@pytest.mark.parametrize("precision,tile_j", [("f64", 8), ("f32k", 4), ("f32k", 8), ("f32k", 16)])
def test_tile_pass_wait_timeout_reported_and_recovered(gpu_lib, precision, tile_j):
    from phonomena_gb300._lib import PhonoError

    spec, g, m, src = _case()
    with _sim(spec, g, m, src, precision, tile_j) as clean:
        clean.step(STEPS)
        clean.sync()
        want = [clean.download(k) for k in ("ux", "uy", "uz")]
    with _sim(spec, g, m, src, precision, tile_j) as sim:
        sim.test_wait_timeout(POLLS, 5)
        sim.step(3)
        with pytest.raises(PhonoError) as e:
            sim.sync()
        assert e.value.code == -6, e.value
        sim.test_wait_timeout(0, -1)
        sim.reset()
        sim.step(STEPS)
        sim.sync()  # the error word was cleared by the reset
        for key, w in zip(("ux", "uy", "uz"), want):
            assert np.array_equal(sim.download(key), w), key


def test_batch_kernel_wait_timeout_reported(gpu_lib):
    from phonomena_gb300._lib import PhonoError
    from phonomena_gb300.batch import Batch

    spec, g, m, src = _case()
    sims = [_sim(spec, g, m, src, "f32k", 16) for _ in range(2)]
    try:
        sims[1].test_wait_timeout(POLLS, 7)
        with Batch(4, precision="f32k", tile_j=16) as b:
            for s in sims:
                b.add(s, STEPS)
            b.step(2)
            with pytest.raises(PhonoError) as e:
                b.sync()
            assert e.value.code == -6 and "instance 1" in str(e.value), e.value
    finally:
        for s in sims:
            s.close()
