"""Krylov noise mode (bd_set_noise_mode, BD_NOISE_KRYLOV): rd = s2dt D^{1/2} p
by Lanczos, checked against the symmetric square root from a dense FP64
eigendecomposition of the same tensor (numpy).  Tolerances: FP64 contexts
with tol = 1e-9, 1e-7 relative (max |x - ref| / max |ref|); mixed contexts
(FP32-rounded tensor products) with tol = 1e-6, 1e-5.  The Krylov step is
deterministic (fixed-order reductions) and switching back to the Cholesky
noise gives the reference's step again."""
import numpy as np
import pytest

from conftest import load_golden, rel_err

pytestmark = pytest.mark.gpu


def _exact_sqrt_rd(D, p, s2dt):
    lam, Q = np.linalg.eigh(D)
    return s2dt * (Q @ (np.sqrt(np.clip(lam, 0, None)) * (Q.T @ p)))


@pytest.mark.parametrize("name", ["syn_4nuc_lh", "cfg0_12nuc"])
@pytest.mark.parametrize("prec,tol,bound", [(0, 1e-9, 1e-7), (1, 1e-6, 1e-5)])
def test_krylov_matches_dense_square_root(name, prec, tol, bound):
    from brownian_dynamics_cuda_gb300 import NOISE_KRYLOV, PREC_FP64, Context
    fib, _ = load_golden(name)
    D = Context(fib, precision=PREC_FP64).diffusion_tensor()
    p = np.random.default_rng(4).normal(size=fib.m)
    ref = _exact_sqrt_rd(D, p, fib.scalars["s2dt"])
    c = Context(fib, precision=prec)
    c.set_noise_mode(NOISE_KRYLOV, tol, 200)
    rd = c.noise_displacement(p)
    it, ch = c.krylov_stats()
    assert 2 <= it < 200 and ch <= tol, (it, ch)
    assert rel_err(rd, ref) <= bound, (rel_err(rd, ref), it)


def test_krylov_step_deterministic_and_switch_back():
    from brownian_dynamics_cuda_gb300 import NOISE_CHOLESKY, NOISE_KRYLOV, PREC_MIXED, Context
    fib, z = load_golden("syn_4nuc_lh")
    rr, p = z["noise0_rr"], z["noise0_p"]
    a, b = Context(fib, precision=PREC_MIXED, use_graph=True), Context(fib, precision=PREC_MIXED)
    for c in (a, b):
        c.set_noise_mode(NOISE_KRYLOV, 1e-6, 64)
    ea, eb = a.step(rr, p), b.step(rr, p)
    assert ea == eb and np.all(np.isfinite(a.get("r")))
    for k in ("r", "r_t", "r_lh", "a"):
        assert np.array_equal(a.get(k), b.get(k)), k
    # back to the reference's noise: L p again (a fresh context's factor at the
    # same positions), and the graph and eager contexts still agree
    for c in (a, b):
        c.set_noise_mode(NOISE_CHOLESKY, 0.0, 0)
    ref = Context(fib, precision=PREC_MIXED)
    for k in ("r", "a", "b", "c", "r_t", "r_lh"):
        ref.set(k, a.get(k))
    assert np.array_equal(a.noise_displacement(p), ref.noise_displacement(p))
    assert a.step(rr, p) == b.step(rr, p)
    assert np.array_equal(a.get("r"), b.get("r"))


def test_krylov_mode_with_frequency_rp():
    """D rebuilt every third step; between rebuilds the Krylov steps reuse it."""
    from brownian_dynamics_cuda_gb300 import NOISE_KRYLOV, PREC_FP64, Context, Noise
    fib, _ = load_golden("cfg0_12nuc")
    c = Context(fib, precision=PREC_FP64, frequency_RP=3)
    c.set_noise_mode(NOISE_KRYLOV, 1e-8, 100)
    g = Noise(5)
    for s in range(4):
        rr, p = g.step(s, fib.arrays["r_var"], fib.m)
        assert np.isfinite(c.step(rr, p))
    assert np.all(np.isfinite(c.get("r")))
    with pytest.raises(Exception):
        c.set_noise_mode(7, 1e-6, 64)
