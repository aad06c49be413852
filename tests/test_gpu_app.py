"""The GB300 plugin inside the reference phonomena application, on the GPU.

tests/reference_app.py (mode ``gpu``) copies the reference application,
adds solver_gb300.py to its solvers directory and runs the application's own
registry and settings code: ``common.findSolvers()`` discovers the plugin,
``common.loadSettings(data/default.json with "solver": "gb300")`` selects it
and hands it the reference's own Grid (non-uniform mesh around six Au
inclusions) and Material objects; ``init`` / ``run(signals=...)`` then run
on the GPU, the material ids built on the device from the inclusion list.

Checked: the plugin's class subclasses the reference's BaseSolver; progress
is emitted as integers ending at 100; the final ux, uy, uz and the surface
records equal the reference solver's (the default_json golden fixture) bit
for bit; the device-built materials equal the reference's
Material.setConstants; and the reference's analysis.spectrum gives the same
axes and spectrum on the plugin's result files (surface records every 5
steps; the full volume every step) as on the reference's own file.
"""
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

import golden_cases as G
from test_output_spectrum import compare_spectra

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def app_result(gpu_lib, tmp_path_factory):
    from oracle import ref_harness as H

    if not H.available():
        pytest.skip(f"reference application not installed under {H.REF_ROOT} (oracle/install_reference.py)")
    tmp = tmp_path_factory.mktemp("app")
    r = subprocess.run([sys.executable, str(ROOT / "tests" / "reference_app.py"), "gpu", str(tmp)],
                       capture_output=True, text=True, timeout=900, cwd=str(tmp))
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    return dict(np.load(tmp / "result.npz", allow_pickle=False))


def test_plugin_found_selected_and_subclasses_reference(app_result):
    res = app_result
    assert "gb300" in res["found"] and "default" in res["found"]
    assert str(res["selected"]) == "gb300"
    assert bool(res["subclass"])
    p = res["progress"]
    assert p.dtype.kind == "i" and p[0] == 0 and p[-1] == 100 and np.all(np.diff(p) >= 0)


def test_plugin_in_application_bit_exact_vs_reference(app_result):
    res = app_result
    d = G.load("default_json")
    for key in ("ux", "uy", "uz"):
        assert G.matches(d, key, res[key]), key
        assert np.array_equal(res[key], res[f"ref_{key}"]), key
    assert G.matches(d, "surf", res["surf"])
    assert np.array_equal(res["ids"].astype(bool), res["ref_secondary"])


def test_plugin_files_give_reference_spectrum(app_result):
    compare_spectra(app_result, "gb", "ref", 2)
    compare_spectra(app_result, "gbvol", "refvol", 3)
