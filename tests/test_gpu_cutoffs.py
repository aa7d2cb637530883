"""The force cut-offs of the mixed path decided as the FP64 path decides them.

The Debye-Hueckel (7 nm) and Lennard-Jones (4 nm) terms are truncated
without a shift (func.cpp:278-345), so a pair's force jumps at the cut-off.
An FP32 distance is uncertain by ~1e-6 nm there; within a guard band the
FP32 pair terms decide from the FP64 distance.  Here a tail bead is placed at
7 nm +- 2e-7 .. 1e-6 from another tail bead (and 4 nm +- the same from a
linker bead): the mixed forces on both must equal the FP64 ones to the
mixed path's FP32 class (1e-7 of the largest tail force), which a pair
dropped or kept on the wrong side of the cut-off would break (the DH force
at 7 nm is ~1e-5 of it here).
"""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("cut,delta", [(7.0, 2e-7), (7.0, -2e-7), (7.0, 6e-7), (7.0, -6e-7), (4.0, 3e-7), (4.0, -3e-7)])
def test_mixed_cutoff_decisions_match_fp64(cut, delta):
    from brownian_dynamics_cuda_gb300 import PREC_FP64, PREC_MIXED, Context
    fib, _ = load_golden("syn_4nuc_lh")
    rt = fib.state["r_t"].reshape(-1, 3).copy()
    r = fib.state["r"].reshape(-1, 3)
    grp = fib.arrays["t_grp"]
    t0 = 0
    if cut == 7.0:  # a tail bead of another tail group, moved to 7 nm - delta along x
        u = int(np.nonzero(grp != grp[t0])[0][-1])
        rt[u] = rt[t0] + np.array([cut - delta, 0.0, 0.0])
        watch = [("t_force", t0), ("t_force", u)]
    else:  # tail bead t0 moved to 4 nm - delta from a linker bead
        j = int(np.nonzero(fib.arrays["type"] == 0)[0][0])
        rt[t0] = r[j] + np.array([0.0, cut - delta, 0.0])
        watch = [("t_force", t0), ("force", j)]
    out = {}
    for prec in (PREC_FP64, PREC_MIXED):
        c = Context(fib, precision=prec)
        c.set("r_t", rt.ravel())
        out[prec] = c.forces()
        c.close()
    scale = np.abs(out[PREC_FP64]["t_force"]).max()
    for key, b in watch:
        f64 = out[PREC_FP64][key].reshape(-1, 3)[b]
        fmx = out[PREC_MIXED][key].reshape(-1, 3)[b]
        assert np.abs(fmx - f64).max() <= 1e-7 * scale, (key, b, f64, fmx)
