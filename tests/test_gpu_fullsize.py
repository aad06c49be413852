"""The benchmarked configuration itself, against the oracle at full size.

The 256 x 256 x 128-cell crystal of the headline benchmark (8,520,321 nodes:
lattice a = 16, radii U[0.2a, 0.4a], 25% tungsten, holes 10 cells deep,
42 MHz line source, corrected z = 0 row, absorbing walls), with the tile
shapes the benchmark runs: FP64 at the autotuner's choice for the plain
FP64 path and the benchmark's tuned FP32K segment list (seven segments of 30
planes, then 16, 12, 8, 6, 4).  At this size the tile counts, the x
segments, the face work lists and the divisor table's hash all differ from
the small grids of the other tests.  200 time steps of the plain FP64 path
must equal the oracle's restatement of the reference (oracle/cpu_ref.c,
itself pinned bit for bit to phonomena's solver) bit for bit, surface
records included; 200 FP32K steps must equal the oracle's FP32 restatement
bit for bit.  About 10 s of host time on 16 cores for each oracle run.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STEPS = 200
CELLS = (256, 256, 128)
F32K_SEGMENTS = [30] * 7 + [16, 12, 8, 6, 4]  # adds up to nx - 1 = 256


def _crystal():
    from phonomena_gb300 import crystal

    spec = crystal.CrystalSpec(cells=CELLS, lattice=16, radius=(0.2, 0.4), depth=10, tungsten_frac=0.25, seed=0,
                               steps=STEPS)
    g, m = crystal.build(spec)
    return spec, g, m, crystal.sin_source(spec.freq, m.dt, STEPS)


@pytest.fixture(scope="module")
def case(oracle):
    spec, g, m, src = _crystal()
    prob = oracle.OracleProblem(g.spacing(), m.ids, m.table, m.dt, src, surface_mode=1)
    return spec, g, m, src, prob


@pytest.mark.parametrize("tile_j,x_segment", [(8, 24), (16, 32)])
def test_config2_f64_bit_exact_vs_oracle(gpu_lib, oracle, case, tile_j, x_segment):
    from phonomena_gb300.device import DeviceSimulation

    spec, g, m, src, prob = case
    assert sum(F32K_SEGMENTS) == g.x.size - 1
    st, surf = oracle.run_f64(prob, record_every=10)
    with DeviceSimulation(g.spacing(), m.ids, m.table, m.dt, precision="f64", surface_mode="corrected",
                          max_steps=STEPS, record_every=10, tile_j=tile_j, x_segment=x_segment) as sim:
        sim.set_source(src)
        sim.step(STEPS)
        sim.sync()
        for key, ref in zip(("ux", "uy", "uz"), st.u):
            got = sim.download(key)
            assert np.array_equal(got, ref), f"{key}: {int((got != ref).sum())} values differ"
        assert np.array_equal(sim.read_surface(), surf)
        assert np.abs(st.u[2]).max() > 0  # the wave has entered the crystal


def test_config2_f32k_bit_exact_vs_oracle(gpu_lib, oracle, case):
    from phonomena_gb300.device import DeviceSimulation

    spec, g, m, src, prob = case
    st, surf = oracle.run_f32k(prob, record_every=10)
    with DeviceSimulation(g.spacing(), m.ids, m.table, m.dt, precision="f32k", surface_mode="corrected",
                          max_steps=STEPS, record_every=10, tile_j=4, x_segment=F32K_SEGMENTS) as sim:
        sim.set_source(src)
        sim.step(STEPS)
        sim.sync()
        for key, ref in zip(("ux", "uy", "uz"), st.u):
            assert np.array_equal(sim.download(key), ref), key
        for key, ref in zip(("vx", "vy", "vz"), st.v):
            assert np.array_equal(sim.download(key), ref), key
        assert np.array_equal(sim.read_surface(), surf)
