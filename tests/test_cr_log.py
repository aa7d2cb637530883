"""The correctly rounded logarithm of the device noise stream (csrc/cr_log.cuh),
compiled for the host from the same source: equal to the correctly rounded
natural log (mpmath at 200 bits, rounded to nearest) on every value of the
polar transform's argument distribution and on edge values; the C library's
log (the reference's, utilities.cpp:304-336) is not correctly rounded on a
small fraction of them, which is why the device stream equals a host stream
set to BD_LOG_CR bit for bit, and the reference's only where glibc rounds
correctly."""
import ctypes as C
import math
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "brownian_dynamics_cuda_gb300", "csrc")


@pytest.fixture(scope="module")
def crlog(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("crlog") / "crlog.so")
    subprocess.check_call(["g++", "-O2", "-fPIC", "-shared", "-std=c++17", "-ffp-contract=off", "-I", CSRC,
                           os.path.join(ROOT, "tests", "cr_log_check.cpp"), "-o", so])
    lib = C.CDLL(so)
    lib.cr_log_many.argtypes = [C.c_void_p, C.c_void_p, C.c_int]

    def f(x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty_like(x)
        lib.cr_log_many(x.ctypes.data, y.ctypes.data, x.size)
        return y
    return f


def _cr_ref(xs):
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 200
    return np.array([float(mpmath.log(mpmath.mpf(float(x)))) for x in xs])


def _polar_q(n, seed):
    # the polar transform's argument: x, y = 2 u - 1 with u = k / (2^32 - 1)
    rng = np.random.default_rng(seed)
    k = rng.integers(0, 2**32, size=(2, 2 * n), dtype=np.uint64).astype(np.float64)
    x = 2.0 * (k[0] * (1.0 / 4294967295.0)) - 1.0
    y = 2.0 * (k[1] * (1.0 / 4294967295.0)) - 1.0
    q = x * x + y * y
    return q[(q > 0.0) & (q <= 1.0)][:n]


def test_correctly_rounded_on_polar_arguments(crlog):
    q = _polar_q(40000, 7)
    ref = _cr_ref(q)
    got = crlog(q)
    assert np.array_equal(got, ref), int(np.sum(got != ref))
    libm = np.array([math.log(v) for v in q])
    miss = int(np.sum(libm != ref))
    # glibc's log is within one ulp but not correctly rounded everywhere
    assert np.all(np.abs(libm - ref) <= np.spacing(np.abs(ref)))
    assert miss < 0.01 * q.size


def test_edge_values(crlog):
    xs = [1.0, np.nextafter(1.0, 0.0), np.nextafter(1.0, 2.0), 0.5, 2.0, 0.25, 1e-300, 5e-324, 2.2250738585072014e-308,
          math.sqrt(2.0), np.nextafter(math.sqrt(2.0), 0.0), np.nextafter(math.sqrt(2.0), 2.0), 1.0 / math.sqrt(2.0),
          0.7071067811865475, 0.7071067811865476, 1e300, 1.7976931348623157e308, math.e, 10.0, 1e-20, 3.0e-10]
    rng = np.random.default_rng(11)
    xs += list(np.exp(rng.uniform(-700, 700, size=3000)))
    xs += list(1.0 + rng.uniform(-1e-6, 1e-6, size=1000))
    xs = np.array(xs, dtype=np.float64)
    assert np.array_equal(crlog(xs), _cr_ref(xs))
    assert crlog(np.array([1.0]))[0] == 0.0
    special = crlog(np.array([0.0, -1.0, np.inf, np.nan]))
    assert special[0] == -np.inf and np.isnan(special[1]) and special[2] == np.inf and np.isnan(special[3])


def test_host_stream_log_modes():
    """A host stream set to LOG_CR differs from the reference's (LOG_LIBM)
    only where glibc's log rounds differently: in the last bit, on a small
    fraction of the deviates; the uniform words are the same."""
    pytest.importorskip("mpmath")
    from brownian_dynamics_cuda_gb300 import LOG_CR, Noise
    a, b = Noise(42), Noise(42, log_mode=LOG_CR)
    r_var = np.full(300, 0.5)
    diff = total = 0
    for step in range(20):
        ra, pa = a.step(step, r_var, 3000)
        rb, pb = b.step(step, r_var, 3000)
        for x, y in ((ra, rb), (pa, pb)):
            assert np.all(np.abs(x - y) <= 4 * np.spacing(np.abs(x)))
            diff += int(np.sum(x != y))
            total += x.size
    assert 0 < diff < 0.01 * total
    assert np.array_equal(a.u32(1000), b.u32(1000))


def test_log_mode_argument_checked():
    from brownian_dynamics_cuda_gb300 import LOG_CR, LOG_LIBM, BDError, Noise
    g = Noise(1)
    g.set_log(LOG_CR)
    g.set_log(LOG_LIBM)
    with pytest.raises(BDError):
        g.set_log(7)
