"""Failures injected on the host, none of which faults the GPU.

* An indefinite diffusion tensor (one bead given a negative radius, so its
  3x3 diagonal block of D is negative): the reference's Cholesky counts the
  non-positive pivot, writes "wrong D here." and continues with |f|
  (func.cpp:827-833; cuSOLVER's potrf in func_cuda.cu:3526-3529 would stop).
  The library counts the same pivots (bd_negative_pivots), keeps the
  reference's |f| rule in both precisions, and the FP64 factor and step
  still equal the oracle's to 1e-10.
* A NaN or Inf in the host noise: bd_step returns BD_ERR_NONFINITE before it
  launches anything, and the context's state is untouched.
* A NaN in the state (set through bd_set): the next step's energy is not
  finite, and bd_step returns BD_ERR_NONFINITE.
"""
import copy

import numpy as np
import pytest

from conftest import load_golden, rel_err

pytestmark = pytest.mark.gpu


def _indefinite(fib):
    f = copy.deepcopy(fib)
    f.arrays["rad"] = f.arrays["rad"].copy()
    dna = int(np.nonzero(f.arrays["type"] == 0)[0][1])
    f.arrays["rad"][dna] = -1.5
    return f


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_indefinite_tensor_counts_pivots(prec):
    from brownian_dynamics_cuda_gb300 import PREC_FP64, PREC_MIXED, Context
    from oracle.pyoracle import Oracle, cholesky
    fib, z = load_golden("syn_4nuc_lh")
    bad = _indefinite(fib)
    o = Oracle(bad)
    D, L_ref = o.tensor()
    _, neg_ref = cholesky(D, 1)
    assert neg_ref > 0
    c = Context(bad, precision=PREC_FP64 if prec == "fp64" else PREC_MIXED)
    L = c.cholesky()
    assert c.negative_pivots() > 0
    assert np.all(np.isfinite(L))
    if prec == "fp64":
        assert c.negative_pivots() == neg_ref
        assert rel_err(L, L_ref) <= 1e-10
        rr, p = z["noise0_rr"], z["noise0_p"]
        e = c.step(rr, p)
        assert abs(e - o.step(rr, p)) <= 1e-10 * abs(e)
        for k in ("r", "r_t", "r_lh"):
            assert rel_err(c.get(k), o.get(k)) <= 1e-10, k


@pytest.mark.parametrize("which,val", [("rr", np.nan), ("p", np.inf), ("p", np.nan)])
def test_nonfinite_noise_is_refused(which, val):
    from brownian_dynamics_cuda_gb300 import BDError, Context
    fib, z = load_golden("syn_4nuc_lh")
    c = Context(fib)
    rr, p = z["noise0_rr"].copy(), z["noise0_p"].copy()
    (rr if which == "rr" else p)[7] = val
    r0 = c.get("r")
    with pytest.raises(BDError) as ei:
        c.step(rr, p)
    assert ei.value.code == 5 and "non-finite" in str(ei.value)
    assert np.array_equal(c.get("r"), r0)
    c.step(z["noise0_rr"], z["noise0_p"])        # the context is still usable
    assert np.all(np.isfinite(c.get("r")))


def test_nonfinite_state_is_reported():
    from brownian_dynamics_cuda_gb300 import BDError, Context
    fib, z = load_golden("syn_4nuc_lh")
    c = Context(fib)
    r = c.get("r")
    r[4] = np.nan
    c.set("r", r)
    with pytest.raises(BDError) as ei:
        c.step(z["noise0_rr"], z["noise0_p"])
    assert ei.value.code == 5
