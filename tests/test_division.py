"""The FP64 leapfrog's divisor-table division equals IEEE division.

The FP64 path divides by the mesh's spacings through a table of double-word
reciprocals (div_tab in phonomena_gb300/csrc/div_table.cuh): two operations for
a divisor the host has proven exact (two_op_exact, same file), one
Markstein correction more for the others.  The reference's results stay
bit-identical only if that quotient is the IEEE one for every operand.
tests/div_check.c restates the method and the exactness check on the host and
compares the quotient with x / h bit for bit for 256 divisors: random operands
over the whole fast range, quotients built to lie within |c| * 2^-107 of a
rounding midpoint for |c| up to 3000 (the hard cases; the check itself looks
at |c| <= 8), exact multiples, signed zeros and the values that take the
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
def test_table_division_is_ieee(div_check, seed):
    out = subprocess.run([str(div_check), "2000000", str(seed)], capture_output=True, text=True)
    cases, bad = (int(v) for v in out.stdout.split()[-2:])
    assert cases > 10_000_000
    assert bad == 0 and out.returncode == 0, out.stdout


@pytest.mark.parametrize("weaken", [
    ("return fma(r, d->yh, q0);", "return q0;"),         # no correction for the inexact divisors
    ("for (int c = -8; c <= 8; c++) {", "for (int c = 0; c <= 0; c++) {"),  # every divisor taken as exact
])
def test_check_detects_a_weakened_method(div_check, tmp_path, weaken):
    """A weakened method (no remainder correction, or an exactness check that
    looks at no candidate) gives wrong quotients that the near-midpoint cases
    catch, so the check above is not passing vacuously."""
    src = (HERE / "div_check.c").read_text()
    weak = src.replace(*weaken)
    assert weak != src
    f = tmp_path / "weak.c"
    f.write_text(weak)
    exe = tmp_path / "weak"
    subprocess.run([shutil.which("gcc") or "cc", "-O2", "-ffp-contract=off", "-o", str(exe), str(f), "-lm"], check=True)
    out = subprocess.run([str(exe), "2000000", "1"], capture_output=True, text=True)
    assert int(out.stdout.split()[-1]) > 0


# spacing values near 10 um whose two-operation quotient is not exact for
# every x (found with the check; the FP64 path corrects them), and values of
# the benchmark meshes, whose quotient is
INEXACT = [float.fromhex(h) for h in ("0x1.734124667319bp-17", "0x1.67e041ec7f1c3p-17", "0x1.7d89477b95583p-17",
                                      "0x1.6d2f31fa6e7f3p-17", "0x1.6452afa20d79bp-17", "0x1.8c5e7d6c6587bp-17")]
EXACT = [float.fromhex(h) for h in ("0x1.4f8b588e368e0p-17", "0x1.4f8b588e368f0p-17", "0x1.4f8b588e368f1p-17",
                                    "0x1.4f8b588e368f2p-17", "0x1.4f8b588e368f4p-17")] + [1e-5, 1.0, 1.1]


def _two_op_failures(b):
    """x whose RN(x*yh + RN(x*yl)) differs from x / b, over the near-midpoint
    candidates of the host check, in exact rational arithmetic (Fraction
    converts to float with round-to-nearest-even)."""
    import math
    from fractions import Fraction as Q

    yh = 1.0 / b
    yl = float(Q(1) - Q(b) * Q(yh)) / b  # the remainder is exact; IEEE division
    m, e = math.frexp(b)
    H, eh = int(m * 2 ** 53), e - 53
    while H % 2 == 0:
        H //= 2
        eh += 1
    inv = pow(H, -1, 2 ** 64)
    bad = []
    for D in range(50, 55):
        for c in range(-8, 9):
            if c == 0:
                continue
            M = (c * inv) % (2 ** D)
            while M < 2 ** 54:
                if M >= 2 ** 53 and M % 2 == 1 and (H * M - c) % (2 ** D) == 0:
                    X = (H * M - c) >> D
                    if 0 < X < 2 ** 53:
                        x = math.ldexp(float(X), D + eh)
                        q = float(Q(x) * Q(yh) + Q(float(Q(x) * Q(yl))))
                        if q != x / b:
                            bad.append(x)
                if D == 54:
                    break
                M += 2 ** D
    return bad


def test_exactness_check_restated_in_rational_arithmetic():
    for b in INEXACT:
        assert _two_op_failures(b), b.hex()
    for b in EXACT:
        assert not _two_op_failures(b), b.hex()


def test_divisor_table_host_code():
    """build_div_table (the host code phono_create runs, through the test
    library): every divisor sits at its hash slot with yh = 1/b, yl the
    rounded remainder term and the exact flag of the rational-arithmetic
    check; values outside [2^-40, 2^40] get no entry."""
    import ctypes
    import math
    from fractions import Fraction as Q

    import numpy as np

    from conftest import build_divcheck

    lib = ctypes.CDLL(str(build_divcheck()))
    lib.div_table_host.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                   ctypes.POINTER(ctypes.c_uint), ctypes.POINTER(ctypes.c_int)]
    rng = np.random.default_rng(3)
    values = EXACT + INEXACT + [float(v) for v in rng.uniform(0.9e-5, 1.3e-5, 40)] + [math.ldexp(1.0, 41), 0.0]
    v = np.ascontiguousarray(values, dtype=np.float64)
    cap = 4 * 4096
    out = np.empty(cap, dtype=np.float64)
    mult, shift = ctypes.c_uint(), ctypes.c_int()
    slots = lib.div_table_host(v.ctypes.data, len(v), out.ctypes.data, cap, ctypes.byref(mult), ctypes.byref(shift))
    assert slots > 0 and slots & (slots - 1) == 0
    tab = out[:4 * slots].reshape(slots, 4)
    bits = tab[:, 0].view(np.uint64)
    filled = bits != np.uint64(0xFFFFFFFFFFFFFFFF)
    inside = sorted({b for b in values if 2.0 ** -40 <= b <= 2.0 ** 40})
    assert filled.sum() == len(inside)
    for b in inside:
        u = int(np.float64(b).view(np.uint64))
        slot = ((((u & 0xFFFFFFFF) ^ (u >> 32)) * mult.value) & 0xFFFFFFFF) >> shift.value
        e = tab[slot]
        assert e[0] == b and e[1] == 1.0 / b
        assert e[2] == float((Q(1) - Q(b) * Q(e[1])) / Q(b))
        assert (e[3] == 1.0) == (not _two_op_failures(b)), b.hex()
    assert any(tab[filled, 3] == 0.0) and any(tab[filled, 3] == 1.0)
