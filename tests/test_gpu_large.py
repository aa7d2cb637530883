"""Parity at the benchmark sizes, through the C ABI, against fixtures made by
the reference's own CPU code (tests/golden/make_large_golden.py):

  config 1  the headline fiber, 50 nucleosomes, 44-bp linkers, LH
            (3N = 11,700): forces and one step by the reference, whole arrays;
  config 4  the large fiber, 200 nucleosomes, LH (3N = 46,200): forces by the
            reference, one step by the CPU oracle; packed arrays;
  config 2  four replicas of the uneven batch (smallest, largest, each salt):
            forces and one step by the reference; packed arrays.

Tolerances.  FP64 path: 1e-10 relative (max |x - ref| / max |ref| per array;
packed arrays: per stored entry and per projection) for forces, torques,
energy, the noise displacement rd, positions and frames, as for the small
fixtures.  Mixed path: the step's displacement and rd to 1e-6 relative (the
bound the mixed step is specified to meet); its start-state forces to 1e-7
relative (FP32 pair sums with Kahan-compensated accumulation; measured
<= 2.6e-8 on every fixture).
"""
import os
import sys
import tempfile

import numpy as np
import pytest

from conftest import ROOT

sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
import largefix as lf  # noqa: E402

pytestmark = pytest.mark.gpu
LARGE = os.path.join(ROOT, "tests", "golden", "large")
TOL64 = 1e-10
TOL_DISP = 1e-6
TOL_FORCE_MIXED = 1e-7
STATE = ("rd", "r", "a", "b", "c", "r_t", "r_lh")
FORCES = ("force", "torque", "t_force", "LH_force")


def _names():
    return sorted(f[:-4] for f in os.listdir(LARGE) if f.endswith(".npz")) if os.path.isdir(LARGE) else []


@pytest.fixture(scope="module", params=_names())
def case(request):
    from brownian_dynamics_cuda_gb300 import Fiber
    from brownian_dynamics_cuda_gb300.fiber_gen import config, write_fiber
    from oracle.pyoracle import OracleNoise
    z = dict(np.load(os.path.join(LARGE, request.param + ".npz")))
    spec = config(int(z["cfg"]), seed=int(z["seed"]), replica=int(z["replica"]))
    d = tempfile.mkdtemp(prefix="bdlarge_")
    fib = Fiber.load(d, **write_fiber(spec, d))
    assert np.array_equal(lf.fiber_digest(fib), z["fiber_digest"]), \
        "the fiber generator wrote a different fiber on this host than the fixture's"
    rr, p = OracleNoise(int(z["noise_seed"])).step(0, fib.arrays["r_var"], fib.m)
    assert np.array_equal(lf.digest_arrays(rr, p), z["noise_digest"])
    return request.param, fib, z, rr, p


def _disp_err(ctx, fib, z) -> float:
    worst = 0.0
    for k in ("r", "r_t", "r_lh"):
        x0 = fib.state[k]
        if x0.size == 0:
            continue
        d = ctx.get(k) - x0
        if "step0_d" + k in z or "step0_d" + k + "__n" in z:
            worst = max(worst, lf.rel_err_packed(d, z, "step0_d" + k))
        else:
            ref = z["step0_" + k] - x0
            worst = max(worst, float(np.abs(d - ref).max() / np.abs(ref).max()))
    return worst


def test_fp64_forces_large(case):
    from brownian_dynamics_cuda_gb300 import PREC_FP64, Context
    name, fib, z, rr, p = case
    c = Context(fib, precision=PREC_FP64)
    f = c.forces()
    for k in FORCES:
        if lf.has(z, "f0_" + k) and f[k].size:
            assert lf.rel_err_packed(f[k], z, "f0_" + k) <= TOL64, (name, k)
    e0 = float(z["f0_energy"])
    assert abs(f["energy"] - e0) <= TOL64 * abs(e0)
    c.close()


def test_fp64_step_large(case):
    from brownian_dynamics_cuda_gb300 import PREC_FP64, Context
    name, fib, z, rr, p = case
    c = Context(fib, precision=PREC_FP64)
    e = c.step(rr, p)
    e0 = float(z["step0_energy"])
    assert abs(e - e0) <= TOL64 * abs(e0)
    for k in STATE:
        if lf.has(z, "step0_" + k):
            x = c.get(k)
            if x.size:
                assert lf.rel_err_packed(x, z, "step0_" + k) <= TOL64, (name, k)
    assert c.negative_pivots() == 0
    c.close()


def test_mixed_step_large(case):
    from brownian_dynamics_cuda_gb300 import PREC_MIXED, Context
    name, fib, z, rr, p = case
    c = Context(fib, precision=PREC_MIXED)
    f = c.forces()
    ferr = {k: lf.rel_err_packed(f[k], z, "f0_" + k) for k in FORCES if lf.has(z, "f0_" + k) and f[k].size}
    c.step(rr, p)
    derr = _disp_err(c, fib, z)
    rderr = lf.rel_err_packed(c.get("rd"), z, "step0_rd")
    print(f"{name}: mixed displacement {derr:.2e}, rd {rderr:.2e}, forces",
          {k: f"{v:.1e}" for k, v in ferr.items()})
    assert derr <= TOL_DISP, name
    assert rderr <= TOL_DISP, name
    assert max(ferr.values()) <= TOL_FORCE_MIXED, ferr
    assert c.negative_pivots() == 0
    c.close()
