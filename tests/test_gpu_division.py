"""The FP64 leapfrog's divisor-table division on the GPU equals __ddiv_rn.

div_tab (phonomena_gb300/csrc/div_table.cuh), the device code the FP64 step
kernels divide with, runs over operand pairs chosen here, with a table built
by the same host code as phono_create's, and every quotient is compared with
the GPU's IEEE division bit for bit (tests/div_gpu.cu).  The operands: for
each divisor every x whose quotient lies within |c| * 2^-107 (relative) of a
rounding midpoint for |c| <= 64 (the hard cases, in several binades and both
signs), random x over the fast range, and the values that take the fallback
division (zeros, subnormals, the range edges, huge values, inf, nan).  The
divisors: the benchmark meshes' spacings, 1.0, six spacings whose
two-operation quotient is not exact (the corrected path) and random ones.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np
import pytest

from conftest import build_divcheck
from test_division import EXACT, INEXACT

pytestmark = pytest.mark.gpu


def _near_midpoint_x(b, cmax=64, exps=(-500, -250, 0, 250, 500)):
    """x with x / b within |c| * 2^-107 of a rounding midpoint (see
    two_op_exact): H * M = X * 2^D + c with H the odd part of b's
    significand and M an odd 54-bit midpoint significand."""
    m, e = math.frexp(b)
    H, eh = int(m * 2 ** 53), e - 53
    while H % 2 == 0:
        H //= 2
        eh += 1
    inv = pow(H, -1, 2 ** 64)
    out = []
    for D in (52, 53, 54):
        for c in range(-cmax, cmax + 1):
            if c == 0:
                continue
            M = (c * inv) % (2 ** D)
            while M < 2 ** 54:
                if M >= 2 ** 53 and M % 2 == 1 and (H * M - c) % (2 ** D) == 0:
                    X = (H * M - c) >> D
                    if 0 < X < 2 ** 53:
                        for s in exps:
                            x = math.ldexp(float(X), D + eh + s)
                            out += [x, -x]
                if D == 54:
                    break
                M += 2 ** D
    return out


@pytest.fixture(scope="module")
def divcheck():
    lib = ctypes.CDLL(str(build_divcheck()))
    lib.div_check_gpu.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_longlong,
                                  ctypes.POINTER(ctypes.c_ulonglong)]
    lib.div_check_gpu.restype = ctypes.c_int
    return lib


def test_table_division_equals_ieee_on_the_gpu(gpu_lib, divcheck):
    rng = np.random.default_rng(17)
    randoms = [abs(math.ldexp(float(rng.uniform(1.0, 2.0)), int(rng.integers(-40, 40)))) for _ in range(100)]
    divisors = EXACT + INEXACT + randoms
    specials = [0.0, -0.0, 5e-324, -5e-324, 2.2250738585072014e-308, math.ldexp(1.0, -801), math.ldexp(1.0, -800),
                math.ldexp(1.0, 800), math.ldexp(1.999, 800), math.ldexp(1.0, 801), 1e300, math.inf, -math.inf,
                math.nan, 1.0, -1.0]
    xs, bs = [], []
    for b in divisors:
        hard = _near_midpoint_x(b)
        rand = list(rng.uniform(1.0, 2.0, 400) * np.exp2(rng.integers(-790, 790, 400)) *
                    np.where(rng.random(400) < 0.5, -1.0, 1.0))
        sub = list(rng.uniform(1.0, 2.0, 50) * np.exp2(rng.integers(-1070, -800, 50)))
        for x in hard + rand + sub + specials:
            xs.append(x)
            bs.append(b)
    x = np.ascontiguousarray(xs, dtype=np.float64)
    b = np.ascontiguousarray(bs, dtype=np.float64)
    out = (ctypes.c_ulonglong * 4)()
    rc = divcheck.div_check_gpu(x.ctypes.data, b.ctypes.data, len(x), out)
    assert rc == 0, rc
    mismatches, entries, exact = out[0], out[1], out[2]
    first = np.frombuffer(np.uint64(out[3]).tobytes(), np.float64)[0]
    assert entries == len(set(divisors)), entries
    assert 0 < exact < entries  # both the two-operation and the corrected path are exercised
    assert mismatches == 0, f"{mismatches} of {len(x)} quotients differ from __ddiv_rn (first x = {first!r})"
    assert len(x) > 200_000
