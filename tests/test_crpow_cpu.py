"""The correctly rounded pow(x, 0.2) of the FP64 tracker, compiled for the
host, against a 300-bit mpmath evaluation (CPU only)."""
import ctypes
import math
import os
import subprocess
import tempfile
from fractions import Fraction

import numpy as np
import pytest

from conftest import ROOT

SRC = r'''
#include "crpow.cuh"
extern "C" void crpow_batch(const double* x, double* y, long n) {
    for (long i = 0; i < n; ++i) y[i] = oneka::cr_pow_fifth(x[i]);
}
'''


@pytest.fixture(scope="module")
def crpow():
    td = tempfile.mkdtemp()
    src = os.path.join(td, "crpow.cpp")
    so = os.path.join(td, "libcrpow.so")
    open(src, "w").write(SRC)
    subprocess.run(["g++", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-I",
                    os.path.join(ROOT, "onekapy_gb300", "csrc"), "-o", so, src], check=True)
    lib = ctypes.CDLL(so)

    def f(x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty_like(x)
        lib.crpow_batch(x.ctypes.data_as(ctypes.c_void_p), y.ctypes.data_as(ctypes.c_void_p),
                        ctypes.c_long(x.size))
        return y
    return f


def _cr(x):
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 300
    e = mpmath.power(mpmath.mpf(float(x)), mpmath.mpf(0.2))
    m, ex = mpmath.frexp(e)
    return float(Fraction(int(m * 2**300)) * Fraction(2) ** (int(ex) - 300))


def test_correctly_rounded_on_random_and_edge_inputs(crpow):
    rng = np.random.default_rng(11)
    x = np.concatenate([10 ** rng.uniform(-12, 16, size=20000),
                        [1.0, 2.0, 0.5, 3.0, 1e-300, 5e-324, 1e308, 4.5e15, 1 + 2**-52, 1 - 2**-53]])
    y = crpow(x)
    bad = [(v, w) for v, w in zip(x, y) if w != _cr(v)]
    assert not bad, bad[:5]


def test_special_values(crpow):
    y = crpow(np.array([0.0, np.inf, np.nan, -1.0]))
    assert y[0] == 0.0 and y[1] == np.inf and np.isnan(y[2]) and np.isnan(y[3])


def test_agrees_with_libm_except_its_misroundings(crpow):
    rng = np.random.default_rng(12)
    x = 10 ** rng.uniform(-8, 15, size=20000)
    y = crpow(x)
    libm = np.array([math.pow(v, 0.2) for v in x])
    assert (y == libm).mean() > 0.995
