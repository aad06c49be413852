"""The C oracle against the reference solver's own outputs (bit-exact).

Pins the oracle: every golden fixture was produced by running phonomena's
unmodified ``solver_default`` (tests/golden/make_golden.py); the oracle must
reproduce ux, uy, uz and the surface records bit for bit from the same
inputs.  CPU only.
"""
import numpy as np
import pytest

import golden_cases as G

SURF = {"reference": 0, "corrected": 1}
BC = {"absorbing": 0, "rigid": 1}


def oracle_problem(oracle, d):
    m = d["meta"]
    return oracle.OracleProblem(G.spacing(d), d["ids"], d["table"], d["dt"], d["src"],
                                surface_mode=SURF[m["surface_mode"]], bc=BC[m["bc"]])


@pytest.mark.parametrize("name", G.CASES)
def test_oracle_matches_reference(oracle, name):
    d = G.load(name)
    m = d["meta"]
    prob = oracle_problem(oracle, d)
    st, surf = oracle.run_f64(prob, record_every=m["record_every"])
    for key, arr in zip(("ux", "uy", "uz"), st.u):
        assert G.matches(d, key, arr), f"{name}: {key} differs from the reference"
    assert G.matches(d, "surf", surf), f"{name}: surface records differ from the reference"


@pytest.mark.parametrize("name", ["small3_ref", "small3_corrected", "tiny"])
def test_oracle_split_runs_equal_one_run(oracle, name):
    """Stepping in two calls (checkpoint-style restart) gives the same bits."""
    d = G.load(name)
    m = d["meta"]
    prob = oracle_problem(oracle, d)
    n = m["steps"]
    st, s1 = oracle.run_f64(prob, t0=0, nsteps=n // 2 + 1, record_every=m["record_every"])
    st, s2 = oracle.run_f64(prob, state=st, t0=n // 2 + 1, nsteps=n - n // 2 - 1, record_every=m["record_every"])
    surf = np.concatenate([s1, s2])
    for key, arr in zip(("ux", "uy", "uz"), st.u):
        assert G.matches(d, key, arr)
    assert G.matches(d, "surf", surf)


def test_oracle_thread_count_does_not_change_bits(oracle):
    d = G.load("config1_void_corrected")
    prob = oracle_problem(oracle, d)
    a, _ = oracle.run_f64(prob, nsteps=60, nthreads=1)
    b, _ = oracle.run_f64(prob, nsteps=60, nthreads=4)
    for x, y in zip(a.u, b.u):
        assert np.array_equal(x, y)


def test_f32k_restatement_tracks_f64(oracle):
    """The FP32 Kahan velocity form stays within 1e-5 relative L2 of FP64
    (corrected surface) on the config-1 crystal over its 500 steps."""
    d = G.load("config1_void_corrected")
    prob = oracle_problem(oracle, d)
    a, sa = oracle.run_f64(prob, record_every=10)
    b, sb = oracle.run_f32k(prob, record_every=10)
    num = sum(np.linalg.norm(x - y.astype(np.float64)) ** 2 for x, y in zip(a.u, b.u)) ** 0.5
    den = sum(np.linalg.norm(x) ** 2 for x in a.u) ** 0.5
    assert num / den < 1e-5, num / den
    rel_s = np.linalg.norm(sa - sb) / np.linalg.norm(sa)
    assert rel_s < 1e-5, rel_s
