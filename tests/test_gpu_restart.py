"""A run resumed from a binary restart (state, frames, internal coordinates
and the noise generator's state) continues bit for bit like the run that
was never interrupted (the reference's text restart re-seeds the generator
and re-derives the frames, so its runs do not)."""
import dataclasses

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ANGLES = ("alpha", "beta", "gamma", "length", "a_dna", "b_dna", "c_dna", "alpha_p", "beta_p", "gamma_p")


@pytest.mark.parametrize("prec", [0, 1])
def test_resume_is_bitwise(tmp_path, prec):
    from brownian_dynamics_cuda_gb300 import Context, Noise
    from brownian_dynamics_cuda_gb300.capi import restart_read, restart_write
    from brownian_dynamics_cuda_gb300.fiber_gen import FiberSpec, make_fiber
    fib = make_fiber(FiberSpec(3, [30] * 3, lh=True, seed=4), str(tmp_path / "fib"))
    r_var = fib.arrays["r_var"]
    a, g = Context(fib, precision=prec), Noise(9)
    for s in range(3):
        a.step(*g.step(s, r_var, a.m))
    path = str(tmp_path / "run.rst")
    restart_write(path, 3, a.restart_state(), fib.arrays["nc_lh_flag"], g)
    h = Noise(1)
    step, arr, flags, has = restart_read(path, h)
    assert step == 3 and has
    state = {k: arr[k] for k in ("r", "a", "b", "c", "r_t", "r_lh")}
    fib2 = dataclasses.replace(fib, state=state, arrays=dict(fib.arrays, nc_lh_flag=flags))
    b = Context(fib2, precision=prec, refresh=False, angles={k: arr[k] for k in ANGLES})
    for s in range(3, 6):
        ea = a.step(*g.step(s, r_var, a.m))
        eb = b.step(*h.step(s, r_var, b.m))
        assert ea == eb
        for k in ("r", "a", "b", "c", "r_t", "r_lh"):
            assert np.array_equal(a.get(k), b.get(k)), (s, k)
