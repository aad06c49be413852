"""The FP64 leapfrog's division on isotropic meshes equals IEEE division.

On a mesh whose spacings are all one value h, the FP64 path divides by h with
a double-word reciprocal and one Markstein correction (div_iso in
phonomena_gb300/csrc/fdtd_step.cu) instead of a general division; the
reference's results stay bit-identical only if that quotient is the IEEE one
for every operand.  tests/div_check.c restates the method on the host and
compares it with x / h bit for bit: random operands over the whole fast
range, quotients built to lie within about 2^-107 of a rounding midpoint (the
hard cases), exact multiples, signed zeros and the values that take the
fallback division.
"""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

HERE = Path(__file__).resolve().parent


@pytest.fixture(scope="module")
def div_check(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    exe = tmp_path_factory.mktemp("div") / "div_check"
    subprocess.run([cc, "-O2", "-ffp-contract=off", "-o", str(exe), str(HERE / "div_check.c"), "-lm"], check=True)
    return exe


@pytest.mark.parametrize("seed", [1, 2])
def test_isotropic_division_is_ieee(div_check, seed):
    out = subprocess.run([str(div_check), "2000000", str(seed)], capture_output=True, text=True)
    cases, bad = (int(v) for v in out.stdout.split()[-2:])
    assert cases > 10_000_000
    assert bad == 0 and out.returncode == 0, out.stdout


def test_check_detects_an_uncorrected_quotient(div_check, tmp_path):
    """Without the remainder correction the near-midpoint cases catch errors,
    so the check above is not passing vacuously."""
    src = (HERE / "div_check.c").read_text()
    weak = src.replace("return fma(r, d->yh, q0);", "return q0;")
    assert weak != src
    f = tmp_path / "weak.c"
    f.write_text(weak)
    exe = tmp_path / "weak"
    subprocess.run([shutil.which("gcc") or "cc", "-O2", "-ffp-contract=off", "-o", str(exe), str(f), "-lm"], check=True)
    out = subprocess.run([str(exe), "2000000", "1"], capture_output=True, text=True)
    assert int(out.stdout.split()[-1]) > 0
