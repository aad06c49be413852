"""The result file's schema answers the reference's own reader (CPU, no GPU).

tests/reference_app.py (mode ``schema``) runs the reference application's
default solver with its own Writer, then writes the plugin's file format
(phonomena_gb300.output) from those same results: surface records every 5
steps, and the full volume every step.  The reference's unmodified
``analysis.spectrum`` must then give the same position axis, frequency axis
and spectrum on the plugin's files as on the reference's own file (sampled
at the same steps for the surface layout): the time step of the record axis
is attrs["dt"].  Needs the reference install (oracle/install_reference.py).
"""
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def _run(mode, tmp_path):
    from oracle import ref_harness as H

    if not H.available():
        pytest.skip(f"reference application not installed under {H.REF_ROOT} (oracle/install_reference.py)")
    r = subprocess.run([sys.executable, str(ROOT / "tests" / "reference_app.py"), mode, str(tmp_path)],
                       capture_output=True, text=True, timeout=900, cwd=str(tmp_path))
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    return dict(np.load(tmp_path / "result.npz", allow_pickle=False))


def compare_spectra(res, mine, ref, n):
    for q in range(n):
        for part in ("x", "f", "dft"):
            a, b = res[f"{mine}_s{q}_{part}"], res[f"{ref}_s{q}_{part}"]
            assert a.shape == b.shape and np.array_equal(a, b), (mine, q, part)


def test_plugin_file_schema_gives_reference_spectrum(tmp_path):
    res = _run("schema", tmp_path)
    assert "gb300" in res["found"] and str(res["selected"]) == "gb300"
    compare_spectra(res, "gb", "ref", 2)
    compare_spectra(res, "gbvol", "refvol", 3)
    # the frequency axis of the sampled records: spacing 1 / (records * dt * k)
    f = res["gb_s0_f"]
    assert f.size == (40 // 5) // 2 and f[1] > 0
