"""Batched instances (one persistent launch for many crystals, or every
instance's own kernels on worker streams) against the same instances stepped
alone: every field and surface record must be bit-identical, whatever the
mix, the tiles, the budgets and the join/leave order."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(40, 36, 20), (33, 48, 17), (64, 40, 30), (20, 20, 12), (50, 45, 33)]
BUDGETS = [60, 37, 60, 13, 48]


def _sim(cells, seed, precision, steps, tile_j=8, x_segment=16):
    from phonomena_gb300 import crystal
    from phonomena_gb300.device import DeviceSimulation

    spec = crystal.CrystalSpec(cells=cells, lattice=8, radius=(0.2, 0.4), tungsten_frac=0.25, seed=seed,
                               freq=30e6 + 5e6 * seed, steps=steps)
    g, m = crystal.build(spec)
    sim = DeviceSimulation(g.spacing(), m.ids, m.table, m.dt, precision=precision, surface_mode="corrected",
                           max_steps=steps, record_every=5, tile_j=tile_j, x_segment=x_segment)
    sim.set_source(crystal.sin_source(spec.freq, m.dt, steps))
    return sim


def _state(sim):
    sim.sync()
    return [sim.download(k) for k in ("ux", "uy", "uz")], sim.read_surface()


@pytest.mark.parametrize("streams", [0, 3])
@pytest.mark.parametrize("precision", ["f32k", "f64", "f64v"])
def test_batch_bit_identical_to_alone(gpu_lib, precision, streams):
    from phonomena_gb300.batch import Batch

    alone = []
    for q, (cells, n) in enumerate(zip(SHAPES, BUDGETS)):
        s = _sim(cells, q, precision, 60)
        s.step(n)
        alone.append(_state(s))
        s.close()
    sims = [_sim(cells, q, precision, 60) for q, cells in enumerate(SHAPES)]
    with Batch(8, precision=precision, tile_j=8, streams=streams) as b:
        slots = [b.add(s, n) for s, n in zip(sims, BUDGETS)]
        b.step(25)
        b.step(1)
        b.step(40)  # more than any budget left: every instance stops at its own
        b.sync()
        for s, slot, n in zip(sims, slots, BUDGETS):
            assert b.remaining(slot) == 0
            assert s.steps_done == n
    for q, s in enumerate(sims):
        got = _state(s)
        for a, e in zip(got[0], alone[q][0]):
            assert np.array_equal(a, e), f"instance {q}: field differs from the alone run"
        assert np.array_equal(got[1], alone[q][1]), f"instance {q}: surface differs"
        s.close()


@pytest.mark.parametrize("streams", [0, 2])
def test_batch_join_and_leave(gpu_lib, streams):
    """Instances joining and leaving between calls (continuous batching)."""
    from phonomena_gb300.batch import Batch

    ref = []
    for q in range(3):
        s = _sim(SHAPES[q], 10 + q, "f32k", 60)
        s.step(50)
        ref.append(_state(s))
        s.close()
    sims = [_sim(SHAPES[q], 10 + q, "f32k", 60) for q in range(3)]
    with Batch(2, precision="f32k", streams=streams) as b:
        s0 = b.add(sims[0], 50)
        b.step(20)
        s1 = b.add(sims[1], 50)
        b.step(30)  # instance 0 finishes
        b.sync()
        assert b.remaining(s0) == 0
        b.remove(s0)
        s2 = b.add(sims[2], 50)  # reuses the freed slot
        b.step(12)
        b.step(40)
        b.sync()
        assert b.remaining(s1) == 0 and b.remaining(s2) == 0
    for q, s in enumerate(sims):
        got = _state(s)
        for a, e in zip(got[0], ref[q][0]):
            assert np.array_equal(a, e)
        assert np.array_equal(got[1], ref[q][1])
        s.close()


@pytest.mark.parametrize("precision", ["f32k", "f64"])
def test_streams_scheme_mixed_tiles(gpu_lib, precision):
    """Streams scheme: each instance keeps its own tile height and x segments."""
    from phonomena_gb300.batch import Batch

    tiles = [(4, 16), (16, [20, 10, 3]), (8, -12), (4, 8), (16, 24)]
    alone = []
    for q, ((cells, n), (tj, xs)) in enumerate(zip(zip(SHAPES, BUDGETS), tiles)):
        s = _sim(cells, q, precision, 60, tile_j=tj, x_segment=xs)
        s.step(n)
        alone.append(_state(s))
        s.close()
    sims = [_sim(cells, q, precision, 60, tile_j=tj, x_segment=xs) for q, (cells, (tj, xs)) in enumerate(zip(SHAPES, tiles))]
    with Batch(len(sims), precision=precision, streams=2) as b:
        for s, n in zip(sims, BUDGETS):
            b.add(s, n)
        b.step(7)
        b.step(60)
        b.sync()
    for q, s in enumerate(sims):
        got = _state(s)
        for a, e in zip(got[0], alone[q][0]):
            assert np.array_equal(a, e), f"instance {q}: field differs from the alone run"
        assert np.array_equal(got[1], alone[q][1]), f"instance {q}: surface differs"
        s.close()


def test_set_mode_guards(gpu_lib):
    from phonomena_gb300 import _lib
    from phonomena_gb300._lib import PhonoError, check
    from phonomena_gb300.batch import Batch

    with pytest.raises(PhonoError, match="streams"):
        Batch(2, precision="f32k", streams=257)
    with Batch(2, precision="f32k") as b:
        with pytest.raises(PhonoError, match="mode"):
            check(gpu_lib.phono_batch_set_mode(b._b, 7, 4))
        s = _sim(SHAPES[0], 0, "f32k", 10)
        slot = b.add(s, 10)
        with pytest.raises(PhonoError, match="empty"):
            check(gpu_lib.phono_batch_set_mode(b._b, _lib.BATCH_STREAMS, 4))
        b.remove(slot)
        check(gpu_lib.phono_batch_set_mode(b._b, _lib.BATCH_STREAMS, 4))
        s16 = _sim(SHAPES[0], 0, "f32k", 10, tile_j=16)  # any tile height in the streams scheme
        b.add(s16, 10)
        b.step(10)
        b.sync()
        s.close()
        s16.close()


def test_batch_rejects_mismatched_instances(gpu_lib):
    from phonomena_gb300._lib import PhonoError
    from phonomena_gb300.batch import Batch

    with Batch(2, precision="f32k", tile_j=8) as b:
        s64 = _sim(SHAPES[0], 0, "f64", 10)
        with pytest.raises(ValueError):
            b.add(s64, 10)
        s16 = _sim(SHAPES[0], 0, "f32k", 10, tile_j=16)
        with pytest.raises(PhonoError, match="tile_j"):
            b.add(s16, 10)
        s = _sim(SHAPES[0], 0, "f32k", 10)
        with pytest.raises(PhonoError, match="source"):
            b.add(s, 11)
        for x in (s64, s16, s):
            x.close()


def test_set_tiling_keeps_results(gpu_lib):
    """Changing the tile shape mid-run changes nothing in the results."""
    ref = _sim(SHAPES[2], 3, "f32k", 60)
    ref.step(60)
    want = _state(ref)
    ref.close()
    s = _sim(SHAPES[2], 3, "f32k", 60)
    s.step(17)
    s.set_tiling(16, 24)
    s.step(25)
    s.set_tiling(4, 0)
    s.step(18)
    got = _state(s)
    for a, e in zip(got[0], want[0]):
        assert np.array_equal(a, e)
    assert np.array_equal(got[1], want[1])
    s.close()


def test_listed_segments_keep_results(gpu_lib):
    """Explicit x segment lists (phono_set_segments) change nothing in the
    results, alone and in a batch; bad lists are refused."""
    from phonomena_gb300._lib import PhonoError
    from phonomena_gb300.batch import Batch

    cells = SHAPES[2]  # 65 x planes: segments add up to 64
    ref = _sim(cells, 3, "f32k", 60)
    ref.step(60)
    want = _state(ref)
    ref.close()

    s = _sim(cells, 3, "f32k", 60, tile_j=4, x_segment=[20, 20, 10, 8, 4, 1, 1])
    assert s.x_segment == (20, 20, 10, 8, 4, 1, 1)
    s.step(23)
    s.set_tiling(16, [1, 1, 1, 1, 60])
    s.step(20)
    s.set_tiling(8, 0)  # keeps the list
    assert s.x_segment == (1, 1, 1, 1, 60)
    s.step(17)
    got = _state(s)
    for a, e in zip(got[0], want[0]):
        assert np.array_equal(a, e)
    assert np.array_equal(got[1], want[1])
    for bad in ([63], [65], [0, 64], [1] * 65, [-1, 65]):
        with pytest.raises(PhonoError):
            s.set_tiling(4, bad)
    s.close()

    s = _sim(cells, 3, "f32k", 60, tile_j=16, x_segment=[30, 20, 10, 4])
    with Batch(1, precision="f32k", tile_j=16) as b:
        b.add(s, 60)
        b.step(60)
        b.sync()
    got = _state(s)
    for a, e in zip(got[0], want[0]):
        assert np.array_equal(a, e)
    assert np.array_equal(got[1], want[1])
    s.close()


def test_handle_in_batch_is_guarded(gpu_lib):
    from phonomena_gb300._lib import PhonoError
    from phonomena_gb300.batch import Batch

    s = _sim(SHAPES[0], 0, "f32k", 24)
    b = Batch(2, precision="f32k")
    slot = b.add(s, 24)
    for call in (lambda: s.step(1), s.reset, lambda: s.set_tiling(4, 16), lambda: b.add(s, 1)):
        with pytest.raises(PhonoError):
            call()
    b.step(24)
    b.sync()
    b.remove(slot)
    s.reset()  # allowed again once out of the batch
    slot = b.add(s, 24)
    s.close()  # a handle destroyed while in the batch leaves it
    b.step(12)
    b.sync()
    b.close()


def test_footprint_matches_device_allocation(gpu_lib):
    import torch

    from phonomena_gb300.device import footprint

    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    s = _sim((120, 100, 60), 1, "f32k", 200)
    free1 = torch.cuda.mem_get_info()[0]
    want = footprint((121, 101, 61), "f32k", 200, 5)
    used = free0 - free1
    # cudaMalloc reserves whole pages: allow 2 MiB per allocation
    assert want <= used + (1 << 20) and used - want < 24 * (2 << 20), (used, want)
    s.close()
