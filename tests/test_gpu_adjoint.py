"""Rollout gradients (bd_adjoint) against central finite differences.

The observable is the mean over the final `window` states of the squared
end-to-end distance plus the radius of gyration of the chain; the gradient
is with respect to the stretch, bend and twist moduli and the Debye length.
Finite differences: the FP64 forward path (bd_rollout_loss on an FP64
context, whose steps match the oracle to 1e-10), central, with steps of
1e-4 relative.  The same noise drives every rollout.

Tolerances: FP64 adjoint 1e-6 relative; FP32-forward (mixed-precision
context) adjoint 1e-4 relative, both per component against the largest
component.
"""
import tempfile

import numpy as np
import pytest

from brownian_dynamics_cuda_gb300 import Context, Noise, PREC_FP64, PREC_MIXED
from brownian_dynamics_cuda_gb300.fiber_gen import FiberSpec, config, make_fiber

pytestmark = pytest.mark.gpu


def noise_rows(fib, steps, seed):
    nz = Noise(seed)
    rr, p = [], []
    for s in range(steps):
        a, b = nz.step(s, fib.arrays["r_var"], fib.m)
        rr.append(a)
        p.append(b)
    return np.array(rr), np.array(p)


def theta(fib):
    sc = fib.scalars
    return np.array([sc["h"], sc["g"], sc["s"], 1.0 / sc["debye"]])


def fd_grad(fib, rr, p, window, rel=1e-4):
    ctx = Context(fib, precision=PREC_FP64)
    th = theta(fib)
    g = np.zeros(4)
    for k in range(4):
        d = rel * th[k]
        tp, tm = th.copy(), th.copy()
        tp[k] += d
        tm[k] -= d
        ctx.set_moduli(*tp)
        lp = ctx.rollout_loss(rr, p, window)
        ctx.set_moduli(*tm)
        lm = ctx.rollout_loss(rr, p, window)
        g[k] = (lp - lm) / (2 * d)
    ctx.set_moduli(*th)
    loss = ctx.rollout_loss(rr, p, window)
    ctx.close()
    return loss, g


def rel_vec(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.fixture(scope="module")
def small():
    fib = make_fiber(FiberSpec(3, [30] * 3, lh=False, seed=5), tempfile.mkdtemp())
    rr, p = noise_rows(fib, 6, 11)
    loss, g = fd_grad(fib, rr, p, 3)
    return fib, rr, p, loss, g


def test_adjoint_fp64_small(small):
    fib, rr, p, loss_fd, g_fd = small
    ctx = Context(fib, precision=PREC_FP64)
    r0 = ctx.get("r")
    loss, g = ctx.adjoint(rr, p, window=3, checkpoint_every=4)
    assert abs(loss - loss_fd) <= 1e-12 * abs(loss_fd)
    assert rel_vec(g, g_fd) <= 1e-6, (g, g_fd)
    assert np.array_equal(ctx.get("r"), r0)  # the context's state is left as it was
    assert ctx.adjoint_launches() > 0


def test_adjoint_mixed_small(small):
    fib, rr, p, loss_fd, g_fd = small
    ctx = Context(fib, precision=PREC_MIXED)
    loss, g = ctx.adjoint(rr, p, window=3, checkpoint_every=4)
    assert abs(loss - loss_fd) <= 1e-5 * abs(loss_fd)
    assert rel_vec(g, g_fd) <= 1e-4, (g, g_fd)


def test_adjoint_checkpoint_independent(small):
    fib, rr, p, _, _ = small
    ctx = Context(fib, precision=PREC_FP64)
    _, g1 = ctx.adjoint(rr, p, window=3, checkpoint_every=1)
    _, g6 = ctx.adjoint(rr, p, window=3, checkpoint_every=6)
    assert rel_vec(g1, g6) <= 1e-12


def test_adjoint_config3():
    """24 nucleosomes, 30-bp linkers, no linker histone; 200-step rollout,
    observable over the final 50 states, checkpoints every 20 steps; FP32
    forward (mixed-precision context) against FP64 central differences."""
    fib = make_fiber(config(3), tempfile.mkdtemp())
    rr, p = noise_rows(fib, 200, 1)
    loss_fd, g_fd = fd_grad(fib, rr, p, 50)
    ctx = Context(fib, precision=PREC_MIXED)
    loss, g = ctx.adjoint(rr, p, window=50, checkpoint_every=20)
    assert abs(loss - loss_fd) <= 1e-5 * abs(loss_fd)
    assert rel_vec(g, g_fd) <= 1e-4, (g, g_fd)


def test_adjoint_matches_oracle_reference_gradient():
    """bd_adjoint against the FP64 reference gradient that the CPU oracle
    (bit for bit the reference's step) gives by Richardson-extrapolated
    central differences (tests/golden/adjoint/ref_3nuc.npz)."""
    import os
    from brownian_dynamics_cuda_gb300 import Fiber
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    z = dict(np.load(os.path.join(root, "tests", "golden", "adjoint", "ref_3nuc.npz")))
    fib = Fiber.from_arrays({k[6:]: v for k, v in z.items() if k.startswith("fiber_")})
    w = int(z["window"])
    c64 = Context(fib, precision=PREC_FP64)
    loss, g = c64.adjoint(z["rr"], z["p"], window=w, checkpoint_every=4)
    assert abs(loss - float(z["loss"])) <= 1e-12 * abs(float(z["loss"]))
    assert rel_vec(g, z["grad"]) <= 1e-6, (g, z["grad"])
    cmx = Context(fib, precision=PREC_MIXED)
    _, gm = cmx.adjoint(z["rr"], z["p"], window=w, checkpoint_every=4)
    assert rel_vec(gm, z["grad"]) <= 1e-4, (gm, z["grad"])
