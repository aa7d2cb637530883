"""The oracle at the benchmark sizes, on the CPU.

* oracle/ref_loader.py (the reference readers and main() set-up restated in
  numpy) loads every benchmark fiber exactly as the library's loader does,
  so the CPU baseline and the reference arm of bench.py need no product
  library.
* orc_cholesky on many threads (column-blocked, register-tiled) gives the
  reference's single-threaded factor bit for bit.
* The large fixtures (made by the reference's own code) are reproduced by
  the oracle: forces at every fixture bit for bit; the complete step of the
  headline fiber (3N = 11,700) to 1e-12 relative (bit for bit expected).
"""
import os
import sys
import tempfile

import numpy as np
import pytest

from conftest import ROOT

sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
import largefix as lf  # noqa: E402

LARGE = os.path.join(ROOT, "tests", "golden", "large")


def _specs():
    from brownian_dynamics_cuda_gb300.fiber_gen import FiberSpec, config
    return [config(0), config(1), config(2, replica=3), config(3), config(4),
            FiberSpec(4, [26, 44, 30, 26], lh=True, seed=7, n_sites=120, tail_len=3, lh_charge_range=(0.0, 1.0),
                      cs=0.1)]


@pytest.mark.parametrize("k", range(6))
def test_ref_loader_matches_library_loader(k):
    from brownian_dynamics_cuda_gb300 import Fiber
    from brownian_dynamics_cuda_gb300.fiber_gen import write_fiber
    from oracle import ref_loader
    spec = _specs()[k]
    d = tempfile.mkdtemp()
    files = write_fiber(spec, d)
    a, b = Fiber.load(d, **files), ref_loader.load(d, **files)
    assert a.sizes == b.sizes
    assert a.scalars == b.scalars
    assert np.array_equal(a.setup, b.setup)
    for grp in ("arrays", "state"):
        for key, v in getattr(a, grp).items():
            w = getattr(b, grp)[key]
            assert v.dtype == w.dtype and np.array_equal(v, w), (grp, key)
    assert np.array_equal(lf.fiber_digest(a), lf.fiber_digest(b))


@pytest.mark.parametrize("m", [1, 2, 5, 7, 64, 501, 1003])
def test_blocked_cholesky_is_the_reference_row_loop(m):
    from oracle.pyoracle import cholesky
    rng = np.random.default_rng(m)
    A = rng.standard_normal((m, 24))
    D = A @ A.T / 24 + 0.5 * np.eye(m)
    if m > 4:
        D[3, 3] = -0.1  # a negative pivot: counted and flipped in both forms
    L1, n1 = cholesky(D, 1)
    L4, n4 = cholesky(D, 4)
    assert np.array_equal(L1, L4) and n1 == n4


def _large():
    return sorted(f[:-4] for f in os.listdir(LARGE) if f.endswith(".npz")) if os.path.isdir(LARGE) else []


@pytest.fixture(scope="module", params=_large())
def large(request):
    from brownian_dynamics_cuda_gb300.fiber_gen import config, write_fiber
    from oracle import ref_loader
    from oracle.pyoracle import OracleNoise
    z = dict(np.load(os.path.join(LARGE, request.param + ".npz")))
    spec = config(int(z["cfg"]), seed=int(z["seed"]), replica=int(z["replica"]))
    d = tempfile.mkdtemp()
    fib = ref_loader.load(d, **write_fiber(spec, d))
    assert np.array_equal(lf.fiber_digest(fib), z["fiber_digest"])
    rr, p = OracleNoise(int(z["noise_seed"])).step(0, fib.arrays["r_var"], fib.m)
    assert np.array_equal(lf.digest_arrays(rr, p), z["noise_digest"])
    return request.param, fib, z, rr, p


def test_oracle_forces_match_large_fixtures(large):
    from oracle.pyoracle import Oracle
    name, fib, z, rr, p = large
    f = Oracle(fib).forces()
    for k in ("force", "torque", "t_force", "LH_force"):
        if lf.has(z, "f0_" + k) and f[k].size:
            assert lf.rel_err_packed(f[k], z, "f0_" + k) == 0.0, (name, k)
    assert f["energy"] == float(z["f0_energy"])


def test_oracle_step_matches_reference_at_3n_11700(large):
    from oracle.pyoracle import Oracle, set_threads
    name, fib, z, rr, p = large
    if int(z["cfg"]) != 1:
        pytest.skip("the complete step is checked on the headline fiber only (seconds on the CPU)")
    set_threads(os.cpu_count() or 1)
    try:
        o = Oracle(fib)
        e = o.step(rr, p)
    finally:
        set_threads(1)
    assert abs(e - float(z["step0_energy"])) <= 1e-12 * abs(e)
    for k in ("rd", "r", "a", "b", "c", "r_t", "r_lh"):
        assert lf.rel_err_packed(o.get(k), z, "step0_" + k) <= 1e-12, k
