"""The CPU oracle against the golden fixtures made by the reference's own
CPU code (tests/golden/make_golden.py).  The oracle restates the reference
expression by expression and is built without FMA contraction, so the
comparison is bitwise except for transcendental-function differences
between C libraries (tolerance 1e-12 relative)."""
import numpy as np
import pytest

from conftest import golden_names, load_golden, rel_err
from oracle.pyoracle import Oracle

TOL = 1e-12


@pytest.mark.parametrize("name", golden_names())
def test_oracle_start_state(name):
    fib, z = load_golden(name)
    o = Oracle(fib)
    for k in ("a", "b", "c", "alpha", "beta", "gamma", "length", "a_dna", "b_dna", "c_dna", "beta_p", "beta_t",
              "beta_lh"):
        if z["s0_" + k].size:
            assert rel_err(o.get(k), z["s0_" + k]) <= TOL, k
    f = o.forces()
    for k in ("force", "torque", "t_force", "LH_force"):
        if z["f0_" + k].size:
            assert rel_err(f[k], z["f0_" + k]) <= TOL, k
    assert abs(f["energy"] - float(z["f0_energy"])) <= TOL * abs(float(z["f0_energy"]))


@pytest.mark.parametrize("name", golden_names())
def test_oracle_tensor_checksums(name):
    fib, z = load_golden(name)
    if fib.m > 2000:
        pytest.skip("naive CPU Cholesky of this size is covered by the step test")
    D, L = Oracle(fib).tensor()
    assert rel_err(D.sum(axis=1), z["D_rowsum"]) <= TOL
    assert rel_err(np.diag(D), z["D_diag"]) <= TOL
    assert rel_err(np.diag(L), z["L_diag"]) <= TOL
    assert rel_err(L[:, 0], z["L_col0"]) <= TOL


@pytest.mark.parametrize("name", golden_names())
def test_oracle_steps(name):
    fib, z = load_golden(name)
    o = Oracle(fib)
    for s in range(int(z["steps"])):
        e = o.step(z[f"noise{s}_rr"], z[f"noise{s}_p"])
        assert abs(e - float(z[f"step{s}_energy"])) <= TOL * max(1.0, abs(float(z[f"step{s}_energy"])))
        for k in ("r", "a", "b", "c", "r_t", "r_lh", "rd", "force", "torque"):
            ref = z[f"step{s}_{k}"]
            if ref.size:
                assert rel_err(o.get(k), ref) <= TOL, (s, k)


@pytest.mark.parametrize("name", golden_names())
def test_oracle_em_update_composes_the_step(name):
    """orc_em_update (the reference for bd_em_update) composed as main_cuda
    does - predictor with the forces at the state, forces at the predicted
    state, corrector from the state with the averaged forces - reproduces
    the reference's golden step."""
    fib, z = load_golden(name)
    rr, rd = z["noise0_rr"], z["step0_rd"]
    keys = ("force", "torque", "t_force", "LH_force")
    o = Oracle(fib)
    f0 = o.forces()
    o.em_update(*[f0[k] for k in keys], rr, rd)
    f1 = o.forces()
    avg = [0.5 * (f0[k] + f1[k]) for k in keys]
    c = Oracle(fib)
    c.em_update(*avg, rr, rd)
    for k in ("r", "a", "b", "c", "r_t", "r_lh"):
        ref = z[f"step0_{k}"]
        if ref.size:
            assert rel_err(c.get(k), ref) <= TOL, k
