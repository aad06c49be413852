"""Results must not depend on what else the GPU runs.

Handles stepped at the same time on their own streams, and a handle stepped
while another stream saturates HBM with copies, give the same bits as each
handle stepped alone.  The tile pass refills its shared-memory ring with TMA
copies; without a proxy fence between the threads' reads of a slot and the
copy that refills it, a read still pending under heavy memory traffic saw the
next plane (these cases differed in every run before the fence)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STEPS = 120
NAMES = ("ux", "uy", "uz", "vx", "vy", "vz", "cx", "cy", "cz")


def _sim(spec, tile_j):
    from phonomena_gb300 import crystal
    from phonomena_gb300.device import DeviceSimulation

    g, m = crystal.build(spec)
    sim = DeviceSimulation(g.spacing(), m.ids, m.table, m.dt, precision="f32k", surface_mode="corrected",
                           max_steps=STEPS, record_every=1, tile_j=tile_j, x_segment=min(32, spec.nodes[0] - 1))
    sim.set_source(crystal.sin_source(spec.freq, m.dt, STEPS))
    return sim


def _state(sim):
    sim.sync()
    return [sim.download(k) for k in NAMES] + [sim.read_surface()]


def _specs(n):
    from phonomena_gb300 import crystal

    return crystal.config4_specs(n=n, seed=0, steps=STEPS)


@pytest.mark.parametrize("tile_j", [4, 16])
def test_concurrent_handles_equal_alone(gpu_lib, tile_j):
    specs = _specs(16)
    alone = []
    for spec in specs:
        s = _sim(spec, tile_j)
        s.step(STEPS)
        alone.append(_state(s))
        s.close()
    sims = [_sim(spec, tile_j) for spec in specs]
    for s in sims:  # each handle's stream: all sixteen run at once
        s.step(STEPS)
    for q, s in enumerate(sims):
        got = _state(s)
        for name, a, b in zip(NAMES + ("surface",), alone[q], got):
            assert np.array_equal(a, b), f"instance {q} ({specs[q].nodes}): {name} differs from the alone run"
        s.close()


def test_results_under_background_hbm_traffic(gpu_lib):
    import torch

    side = torch.cuda.Stream()
    src = torch.empty(1 << 28, dtype=torch.float32, device="cuda")  # 1 GiB
    dst = torch.empty_like(src)
    specs = _specs(8)
    for q, tile_j in ((7, 4), (0, 4), (2, 16), (5, 8)):
        s = _sim(specs[q], tile_j)
        s.step(STEPS)
        want = _state(s)
        s.close()
        for rep in range(2):
            s = _sim(specs[q], tile_j)
            torch.cuda.synchronize()
            for _ in range(0, STEPS, 12):
                with torch.cuda.stream(side):
                    for _ in range(100):
                        dst.copy_(src)
                s.step(12)
            got = _state(s)
            torch.cuda.synchronize()
            s.close()
            for name, a, b in zip(NAMES + ("surface",), want, got):
                assert np.array_equal(a, b), f"instance {q}, tile {tile_j}, run {rep}: {name} differs under load"
