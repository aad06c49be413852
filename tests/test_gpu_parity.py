"""GPU parity: the fused sm_103a kernels against the reference and the oracle.

F64 must reproduce the reference solver's outputs bit for bit (golden
fixtures, produced by phonomena's own solver_default); F32K must reproduce the
oracle's FP32 restatement bit for bit and stay within 1e-5 relative L2 of
FP64.  All calls go through the C ABI (libphono_gpu.so via ctypes).
"""
import numpy as np
import pytest

import golden_cases as G

pytestmark = pytest.mark.gpu

SURF = {"reference": 0, "corrected": 1}
BC = {"absorbing": 0, "rigid": 1}


def device_sim(d, precision="f64", steps=None, record_every=None, **kw):
    from phonomena_gb300.device import DeviceSimulation

    m = d["meta"]
    steps = steps or m["steps"]
    sim = DeviceSimulation(G.spacing(d), d["ids"], d["table"], d["dt"], precision=precision,
                           surface_mode=m["surface_mode"], bc=m["bc"], source_mode=m["source_mode"],
                           max_steps=len(d["src"]), record_every=m["record_every"] if record_every is None
                           else record_every, **kw)
    sim.set_source(d["src"])
    return sim


@pytest.mark.parametrize("name", G.CASES)
def test_f64_bit_exact_vs_reference(gpu_lib, name):
    d = G.load(name)
    with device_sim(d) as sim:
        sim.step(d["meta"]["steps"])
        sim.sync()
        for key in ("ux", "uy", "uz"):
            assert G.matches(d, key, sim.download(key)), f"{name}: {key} differs from the reference"
        assert G.matches(d, "surf", sim.read_surface()), f"{name}: surface differs from the reference"


@pytest.mark.parametrize("tile_j,x_segment", [(4, 5), (8, 64), (16, 3), (8, 1), (4, -8), (8, -3)])
@pytest.mark.parametrize("name", ["small3_ref", "config1_void_corrected", "nonuniform_json"])
def test_f64_tile_shapes_bit_exact(gpu_lib, name, tile_j, x_segment):
    d = G.load(name)
    with device_sim(d, tile_j=tile_j, x_segment=x_segment) as sim:
        sim.step(d["meta"]["steps"])
        sim.sync()
        for key in ("ux", "uy", "uz"):
            assert G.matches(d, key, sim.download(key)), f"{name} tj={tile_j} xs={x_segment}: {key}"


def test_f64_split_calls_equal_one_run(gpu_lib):
    """Graph replays (12-step chunks) and single launches interleave correctly."""
    d = G.load("config1_void_corrected")
    with device_sim(d) as sim:
        for n in (5, 12, 1, 30, 24, 7, 421):
            sim.step(n)
        sim.sync()
        assert sim.steps_done == 500
        for key in ("ux", "uy", "uz"):
            assert G.matches(d, key, sim.download(key))
        assert G.matches(d, "surf", sim.read_surface())


def _oracle_prob(oracle, d):
    m = d["meta"]
    return oracle.OracleProblem(G.spacing(d), d["ids"], d["table"], d["dt"], d["src"],
                                surface_mode=SURF[m["surface_mode"]], bc=BC[m["bc"]])


@pytest.mark.parametrize("precision", ["f32k", "f64v"])
@pytest.mark.parametrize("name", G.CASES)
def test_velocity_form_bit_exact_vs_oracle(gpu_lib, oracle, name, precision):
    d = G.load(name)
    m = d["meta"]
    run = oracle.run_f32k if precision == "f32k" else oracle.run_f64v
    st, surf = run(_oracle_prob(oracle, d), record_every=m["record_every"])
    with device_sim(d, precision=precision) as sim:
        sim.step(m["steps"])
        sim.sync()
        for key, ref in zip(("ux", "uy", "uz"), st.u):
            got = sim.download(key)
            assert np.array_equal(got, ref), f"{name}: {key} max diff {np.abs(got - ref).max()}"
        for key, ref in zip(("vx", "vy", "vz"), st.v):
            assert np.array_equal(sim.download(key), ref), f"{name}: {key}"
        for key, ref in zip(("cx", "cy", "cz"), st.c):
            assert np.array_equal(sim.download(key), ref), f"{name}: {key}"
        assert np.array_equal(sim.read_surface(), surf)


def _crystal_case(cells, steps, seed, surface_mode="corrected"):
    from phonomena_gb300 import crystal

    spec = crystal.CrystalSpec(cells=cells, lattice=16, radius=(0.2, 0.4), depth=10, tungsten_frac=0.25,
                               seed=seed, steps=steps)
    g, m = crystal.build(spec)
    src = crystal.sin_source(spec.freq, m.dt, steps)
    d = dict(fdx=g.spacing()["fdx"], fdy=g.spacing()["fdy"], fdz=g.spacing()["fdz"], sdx=g.spacing()["sdx"],
             sdy=g.spacing()["sdy"], sdz=g.spacing()["sdz"], ids=m.ids, table=m.table, dt=m.dt, src=src,
             meta=dict(steps=steps, record_every=10, surface_mode=surface_mode, bc="absorbing", source_mode="line"))
    return d


@pytest.mark.parametrize("cells,tile_j", [((70, 45, 37), 8), ((33, 64, 65), 16), ((40, 40, 20), 4)])
def test_f64_and_f32k_vs_oracle_multi_tile(gpu_lib, oracle, cells, tile_j):
    """Grids with ragged tiles in y and z and several x segments."""
    d = _crystal_case(cells, 60, seed=sum(cells))
    prob = _oracle_prob(oracle, d)
    s64, surf64 = oracle.run_f64(prob, record_every=10)
    s32, surf32 = oracle.run_f32k(prob, record_every=10)
    with device_sim(d, tile_j=tile_j, x_segment=16) as sim:
        sim.step(60)
        sim.sync()
        for key, ref in zip(("ux", "uy", "uz"), s64.u):
            assert np.array_equal(sim.download(key), ref), key
        assert np.array_equal(sim.read_surface(), surf64)
    with device_sim(d, precision="f32k", tile_j=tile_j, x_segment=16) as sim:
        sim.step(60)
        sim.sync()
        for key, ref in zip(("ux", "uy", "uz"), s32.u):
            assert np.array_equal(sim.download(key), ref), key
        assert np.array_equal(sim.read_surface(), surf32)


def test_f64_without_divisor_table_vs_oracle(gpu_lib, oracle):
    """A mesh with more distinct spacings than the divisor table takes (random
    non-uniform x spacings) divides with IEEE division everywhere; the result
    is the oracle's bit for bit."""
    d = _crystal_case((640, 6, 5), 30, seed=5)
    rng = np.random.default_rng(5)
    fdx = d["fdx"] * rng.uniform(0.95, 1.25, d["fdx"].shape)
    d["fdx"], d["sdx"] = fdx, (fdx[1:] + fdx[:-1]) / 2.0
    assert len(np.unique(np.concatenate([d[k] for k in ("fdx", "sdx")]))) > 1024
    s64, surf64 = oracle.run_f64(_oracle_prob(oracle, d), record_every=10)
    with device_sim(d) as sim:
        sim.step(30)
        sim.sync()
        for key, ref in zip(("ux", "uy", "uz"), s64.u):
            assert np.array_equal(sim.download(key), ref), key
        assert np.array_equal(sim.read_surface(), surf64)


def test_f64_corrected_divisors_vs_oracle(gpu_lib, oracle):
    """Spacings whose two-operation quotient is not exact for every operand
    (the remainder-corrected path of the divisor table) mixed with exact
    ones; the result is the oracle's (IEEE division) bit for bit."""
    from test_division import INEXACT

    d = _crystal_case((48, 40, 24), 60, seed=11)
    fdx = np.array([INEXACT[q % len(INEXACT)] if q % 3 else d["fdx"][q] for q in range(len(d["fdx"]))])
    fdy = np.array([INEXACT[(q + 2) % len(INEXACT)] if q % 4 == 1 else d["fdy"][q] for q in range(len(d["fdy"]))])
    d["fdx"], d["sdx"] = fdx, (fdx[1:] + fdx[:-1]) / 2.0
    d["fdy"], d["sdy"] = fdy, (fdy[1:] + fdy[:-1]) / 2.0
    s64, surf64 = oracle.run_f64(_oracle_prob(oracle, d), record_every=10)
    with device_sim(d, tile_j=8, x_segment=16) as sim:
        sim.step(60)
        sim.sync()
        for key, ref in zip(("ux", "uy", "uz"), s64.u):
            assert np.array_equal(sim.download(key), ref), key
        assert np.array_equal(sim.read_surface(), surf64)


def test_f64v_matches_reference_arithmetic(gpu_lib):
    """The FP64 velocity form (the fast FP64 error reference) agrees with the
    reference-arithmetic FP64 path to 1e-12 relative L2 over 500 steps."""
    d = G.load("config1_void_corrected")
    out = {}
    for precision in ("f64", "f64v"):
        with device_sim(d, precision=precision) as sim:
            sim.step(d["meta"]["steps"])
            sim.sync()
            out[precision] = ([sim.download(k) for k in ("ux", "uy", "uz")], sim.read_surface())
    num = sum(np.linalg.norm(a - b) ** 2 for a, b in zip(out["f64"][0], out["f64v"][0])) ** 0.5
    den = sum(np.linalg.norm(a) ** 2 for a in out["f64"][0]) ** 0.5
    assert num / den < 1e-12, num / den
    assert np.linalg.norm(out["f64"][1] - out["f64v"][1]) / np.linalg.norm(out["f64"][1]) < 1e-12


def test_wall_source_matches_oracle(gpu_lib, oracle):
    d = G.load("small3_corrected")
    m = d["meta"]
    prob = oracle.OracleProblem(G.spacing(d), d["ids"], d["table"], d["dt"], d["src"], surface_mode=1, source_mode=1)
    st, surf = oracle.run_f64(prob, record_every=m["record_every"])
    from phonomena_gb300.device import DeviceSimulation

    with DeviceSimulation(G.spacing(d), d["ids"], d["table"], d["dt"], surface_mode="corrected",
                          source_mode="wall", max_steps=m["steps"], record_every=m["record_every"]) as sim:
        sim.set_source(d["src"])
        sim.step(m["steps"])
        sim.sync()
        for key, ref in zip(("ux", "uy", "uz"), st.u):
            assert np.array_equal(sim.download(key), ref)
        assert np.array_equal(sim.read_surface(), surf)


def test_upload_download_resume(gpu_lib):
    """Checkpoint/resume: download state mid-run, upload into a fresh handle, continue."""
    d = G.load("config1_void_corrected")
    with device_sim(d) as a:
        a.step(200)
        a.sync()
        snap = {k: a.download(k) for k in ("ux", "uy", "uz", "ux_old", "uy_old", "uz_old")}
    with device_sim(d) as b:
        # advance the step counter of b to 200 without touching its fields
        b.step(200)
        b.sync()
        for k, v in snap.items():
            b.upload(k, v)
        b.step(300)
        b.sync()
        for key in ("ux", "uy", "uz"):
            assert G.matches(d, key, b.download(key))


def _energy_numpy(d, u, vel):
    """Kinetic and strain energy restated in numpy: 1/2 rho v^2 over the
    interior displacement points, 1/2 T . e over the reference's normal-stress
    nodes and shear edges (base_solver.py:329-372)."""
    ux, uy, uz = u
    ids, tab = d["ids"], d["table"]
    nx, ny, nz = ids.shape
    rho = tab[ids, 12]
    vx, vy, vz = vel
    ek = 0.5 * (np.sum(rho[1:-1, 1:-1, :-1] * vx[:-1, 1:-1, :-1] ** 2)
                + np.sum(rho[1:-1, 2:-1, :-1] * vy[1:-1, 1:-1, :-1] ** 2)
                + np.sum(rho[1:-1, 1:-1, 1:-1] * vz[1:-1, 1:-1, :-1] ** 2))
    fdx, fdy, fdz = d["fdx"], d["fdy"], d["fdz"]
    sdx, sdy, sdz = d["sdx"], d["sdy"], d["sdz"]
    I, J, K = slice(1, nx - 1), slice(1, ny - 1), slice(1, nz - 1)
    e1 = (ux[1:nx - 1, J, K] - ux[0:nx - 2, J, K]) / sdx[:, None, None]
    e2 = (uy[I, 1:ny - 1, K] - uy[I, 0:ny - 2, K]) / sdy[None, :, None]
    e3 = (uz[I, J, 1:nz - 1] - uz[I, J, 0:nz - 2]) / sdz[None, None, :]
    c = tab[ids[I, J, K]]
    t1 = c[..., 0] * e1 + c[..., 1] * e2 + c[..., 2] * e3
    t2 = c[..., 3] * e1 + c[..., 4] * e2 + c[..., 5] * e3
    t3 = c[..., 6] * e1 + c[..., 7] * e2 + c[..., 8] * e3
    es = 0.5 * np.sum(t1 * e1 + t2 * e2 + t3 * e3)
    g4 = ((uy[I, 0:ny - 1, 2:nz] - uy[I, 0:ny - 1, 1:nz - 1]) / fdz[None, None, 1:]
          + (uz[I, 1:ny, 1:nz - 1] - uz[I, 0:ny - 1, 1:nz - 1]) / fdy[None, :, None])
    g5 = ((ux[0:nx - 1, J, 2:nz] - ux[0:nx - 1, J, 1:nz - 1]) / fdz[None, None, 1:]
          + (uz[1:nx, J, 1:nz - 1] - uz[0:nx - 1, J, 1:nz - 1]) / fdx[:, None, None])
    g6 = ((ux[0:nx - 1, 1:ny, K] - ux[0:nx - 1, 0:ny - 1, K]) / fdy[None, :, None]
          + (uy[1:nx, 0:ny - 1, K] - uy[0:nx - 1, 0:ny - 1, K]) / fdx[:, None, None])
    es += 0.5 * (np.sum(tab[ids[I, 1:ny, 2:nz], 9] * g4 ** 2) + np.sum(tab[ids[1:nx, J, 2:nz], 10] * g5 ** 2)
                 + np.sum(tab[ids[1:nx, 1:ny, K], 11] * g6 ** 2))
    return ek, es


@pytest.mark.parametrize("precision", ["f64", "f32k"])
def test_energy_matches_numpy(gpu_lib, precision):
    d = G.load("small3_corrected")
    with device_sim(d, precision=precision) as sim:
        sim.step(d["meta"]["steps"])
        sim.sync()
        ek, es = sim.energy()
        u = [sim.download(k).astype(np.float64) for k in ("ux", "uy", "uz")]
        if precision == "f64":
            old = [sim.download(k) for k in ("ux_old", "uy_old", "uz_old")]
            vel = [(a - b) / d["dt"] for a, b in zip(u, old)]
        else:
            vel = [sim.download(k).astype(np.float64) for k in ("vx", "vy", "vz")]
    ek_ref, es_ref = _energy_numpy(d, u, vel)
    assert ek_ref > 0 and es_ref > 0
    assert abs(ek - ek_ref) <= 1e-9 * abs(ek_ref), (ek, ek_ref)
    assert abs(es - es_ref) <= 1e-9 * abs(es_ref), (es, es_ref)


def test_numeric_guard_reports_nonfinite(gpu_lib):
    from phonomena_gb300._lib import PhonoError

    d = G.load("small3_ref")
    with device_sim(d) as sim:
        bad = np.zeros(sim.download("uz").shape)
        bad[2, 2, 0] = np.inf
        sim.upload("uz", bad)
        sim.step(3)
        with pytest.raises(PhonoError, match="PHONO_ERR_NUMERIC"):
            sim.sync()


def test_invalid_arguments_rejected(gpu_lib):
    from phonomena_gb300._lib import PhonoError

    d = G.load("small3_ref")
    with pytest.raises(PhonoError, match="PHONO_ERR_ARG"):
        device_sim(d, tile_j=5)
    bad = dict(d)
    bad["ids"] = d["ids"].copy()
    bad["ids"][1, 1, 1] = 7
    with pytest.raises(PhonoError, match="material id"):
        device_sim(bad)
    with device_sim(d) as sim:
        with pytest.raises(PhonoError, match="source"):
            sim.step(len(d["src"]) + 1)


def test_plugin_solver_test_defaults(gpu_lib):
    """Solver().test() runs the reference's TestDefaults; the result equals the golden."""
    from phonomena_gb300.solver_gb300 import Solver

    d = G.load("testdefaults_ricker")
    s = Solver()
    s.cfg["write_mode"] = "off"
    s.cfg["record_every"] = 2
    s.test()
    for key in ("ux", "uy", "uz"):
        assert G.matches(d, key, getattr(s.g, key))
    assert G.matches(d, "surf", s.surface)
    s.release()


@pytest.mark.parametrize("precision", ["f64", "f32k"])
def test_checkpoint_resume_bit_exact(gpu_lib, tmp_path, precision):
    """A run stopped at step 130, saved to a file and resumed in a new handle
    ends bit-identical to the run that never stopped (fields and records)."""
    from phonomena_gb300 import crystal
    from phonomena_gb300.device import DeviceSimulation

    spec = crystal.CrystalSpec(cells=(40, 36, 24), lattice=8, radius=(0.2, 0.4), tungsten_frac=0.3, seed=5,
                               steps=300)
    g, m = crystal.build(spec)
    src = crystal.sin_source(spec.freq, m.dt, 300)

    def make():
        s = DeviceSimulation(g.spacing(), m.ids, m.table, m.dt, precision=precision, surface_mode="corrected",
                             max_steps=300, record_every=10, tile_j=8, x_segment=16)
        s.set_source(src)
        return s

    with make() as ref:
        ref.step(300)
        ref.sync()
        want = {k: ref.download(k) for k in ref.state_fields}
        want_surf = ref.read_surface()
    with make() as a:
        a.step(130)
        a.save_checkpoint(tmp_path / "ck.npz")
    with DeviceSimulation.from_checkpoint(tmp_path / "ck.npz") as b:
        assert b.steps_done == 130
        b.step(170)
        b.sync()
        for k, v in want.items():
            assert np.array_equal(b.download(k), v), k
        assert np.array_equal(b.read_surface(), want_surf)


@pytest.mark.parametrize("cells,a,seed", [((40, 36, 24), 8, 1), ((64, 50, 20), 12, 2), ((33, 47, 30), 16, 3)])
def test_device_lattice_ids_equal_host_ids(gpu_lib, cells, a, seed):
    """Material ids built by the lattice kernel give the same run, bit for bit,
    as the host-built ids (FP32K: any id difference shows in the fields)."""
    from phonomena_gb300 import crystal
    from phonomena_gb300.device import DeviceSimulation

    spec = crystal.CrystalSpec(cells=cells, lattice=a, radius=(0.2, 0.45), tungsten_frac=0.4, seed=seed, depth=7,
                               steps=40)
    g, m = crystal.build(spec)
    lat = crystal.lattice(spec)
    src = crystal.sin_source(spec.freq, m.dt, 40)
    out = []
    for mode in ("host", "device"):
        with DeviceSimulation(g.spacing(), np.zeros_like(m.ids), m.table, m.dt, precision="f32k",
                              surface_mode="corrected", max_steps=40, record_every=5) as sim:
            if mode == "host":
                sim.set_materials(crystal.ids_from_lattice(spec.nodes, lat), m.table)
            else:
                sim.set_lattice(lat, m.table)
            sim.set_source(src)
            sim.step(40)
            sim.sync()
            out.append([sim.download(k) for k in ("ux", "uy", "uz")] + [sim.read_surface()])
    assert np.array_equal(crystal.ids_from_lattice(spec.nodes, lat), m.ids)
    for x, y in zip(*out):
        assert np.array_equal(x, y)


def test_time_kernels_equals_step(gpu_lib):
    """phono_time_kernels (each step launch between its own CUDA events, no
    graph) advances the state exactly as phono_step does."""
    d = G.load("config1_void_corrected")
    with device_sim(d) as a, device_sim(d) as b:
        a.step(37)
        tile_ms, face_ms = b.time_kernels(37)
        a.sync()
        b.sync()
        assert tile_ms > 0 and face_ms >= 0 and b.steps_done == 37
        for key in ("ux", "uy", "uz"):
            assert np.array_equal(a.download(key), b.download(key)), key
        assert np.array_equal(a.read_surface(), b.read_surface())
