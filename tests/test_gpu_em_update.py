"""bd_em_update (one Ermak-McCammon move with caller forces and noise, then
the frame refresh) against the oracle's orc_em_update, which composed as
main_cuda does reproduces the reference's golden steps (test_oracle_golden):
FP64 context to 1e-10 relative, mixed-precision context to 1e-6 (positions)."""
import numpy as np
import pytest

from conftest import golden_names, load_golden, rel_err

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", golden_names())
@pytest.mark.parametrize("prec", [0, 1])
def test_em_update_matches_oracle(name, prec):
    from brownian_dynamics_cuda_gb300 import Context
    from oracle.pyoracle import Oracle
    fib, z = load_golden(name)
    rr, rd = z["noise0_rr"], z["step0_rd"]
    o = Oracle(fib)
    f = o.forces()
    args = [f[k] for k in ("force", "torque", "t_force", "LH_force")] + [rr, rd]
    ctx = Context(fib, precision=prec)
    ctx.em_update(*args)
    o.em_update(*args)
    tol = 1e-10 if prec == 0 else 1e-6
    for k in ("r", "r_t", "r_lh") + (("a", "b", "c") if prec == 0 else ()):
        ref = o.get(k)
        if ref.size:
            assert rel_err(ctx.get(k), ref) <= tol, k
