"""Mixed-precision path (BD_PREC_MIXED): double-float (FP32 pair) tensor
storage, FP32 diagonal blocks and tensor-core (tcgen05, BF16 three-way
split) trailing updates.

Accuracy is stated against the FP64 oracle: the factor to 1e-5 relative
(FP32 class, |L_mixed - L| / |L|), the noise displacement rd and the step's
displacement to 1e-6 relative (max |x - ref| / max |ref|), the bound the
mixed step is specified to meet."""
import numpy as np
import pytest

from conftest import golden_names, load_golden, rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=golden_names())
def case(request):
    fib, z = load_golden(request.param)
    return request.param, fib, z


def test_mixed_tensor_fp32(case):
    """The mixed path assembles the RPY tensor in FP32 (separations formed in
    FP64): every entry within a few FP32 ulps of the FP64 tensor."""
    from brownian_dynamics_cuda_gb300 import PREC_FP64, PREC_MIXED, Context
    name, fib, z = case
    D64 = Context(fib, precision=PREC_FP64).diffusion_tensor()
    Dm = Context(fib, precision=PREC_MIXED).diffusion_tensor()
    assert np.abs(Dm - D64).max() <= 5e-7 * np.abs(D64).max()
    big = np.abs(D64) > 1e-3 * np.abs(D64).max()
    assert (np.abs(Dm - D64)[big] / np.abs(D64)[big]).max() <= 2e-6


def test_mixed_factor_matches_fp64(case):
    from brownian_dynamics_cuda_gb300 import PREC_FP64, PREC_MIXED, Context
    name, fib, z = case
    L64 = Context(fib, precision=PREC_FP64).cholesky()
    cm = Context(fib, precision=PREC_MIXED)
    Lm = cm.cholesky()
    assert cm.negative_pivots() == 0
    assert np.all(np.triu(Lm, 1) == 0.0)
    assert rel_err(Lm, L64) <= 1e-5
    p = np.random.default_rng(5).normal(size=fib.m)
    rd64 = Context(fib, precision=PREC_FP64).noise_displacement(p)
    assert rel_err(cm.noise_displacement(p), rd64) <= 1e-6


def test_mixed_step_displacement(case):
    from brownian_dynamics_cuda_gb300 import PREC_MIXED, Context
    from oracle.pyoracle import Oracle
    name, fib, z = case
    o = Oracle(fib)
    c = Context(fib, precision=PREC_MIXED)
    r0 = {k: fib.state[k] for k in ("r", "r_t", "r_lh")}
    for s in range(int(z["steps"])):
        rr, p = z[f"noise{s}_rr"], z[f"noise{s}_p"]
        o.step(rr, p)
        c.step(rr, p)
        for k in ("r", "r_t", "r_lh"):
            ref = o.get(k)
            if ref.size:
                assert rel_err(c.get(k) - r0[k], ref - r0[k]) <= 1e-6, (s, k)
        r0 = {k: o.get(k) for k in ("r", "r_t", "r_lh")}
        # continue both from the oracle's state so errors do not compound
        for k in ("r", "a", "b", "c", "r_t", "r_lh"):
            c.set(k, o.get(k))


def test_mixed_graph_matches_eager(case):
    from brownian_dynamics_cuda_gb300 import PREC_MIXED, Context
    name, fib, z = case
    a, b = Context(fib, precision=PREC_MIXED, use_graph=True), Context(fib, precision=PREC_MIXED)
    rr, p = z["noise0_rr"], z["noise0_p"]
    assert a.step(rr, p) == b.step(rr, p)
    assert np.array_equal(a.get("r"), b.get("r")) and np.array_equal(a.get("r_t"), b.get("r_t"))


def test_mixed_passes_setting():
    """bd_set_mixed_passes: at most one panel per trailing pass makes the
    factor more accurate on the config-2 replica where the default schedule
    is least accurate (3N = 7,977, 50 mM; noise displacement 1.07e-6 from the
    FP64 one with three panels per pass, 4.2e-7 with one), and a graph-captured
    context picks the new schedule up at its next step (bitwise equal to an
    eager context switched the same way)."""
    import tempfile
    from brownian_dynamics_cuda_gb300 import BDError, PREC_FP64, PREC_MIXED, Context, Noise
    from brownian_dynamics_cuda_gb300.fiber_gen import config, make_fiber
    fib = make_fiber(config(2, seed=1, replica=132), tempfile.mkdtemp())
    p = np.random.default_rng(3).normal(size=fib.m)
    rd64 = Context(fib, precision=PREC_FP64).noise_displacement(p)
    errs = {}
    for passes in (3, 1):
        c = Context(fib, precision=PREC_MIXED)
        c.set_mixed_passes(passes)
        errs[passes] = rel_err(c.noise_displacement(p), rd64)
        c.close()
    assert errs[1] <= 6e-7 and errs[1] < errs[3], errs
    g = Noise(9)
    n0 = g.step(0, fib.arrays["r_var"], fib.m)
    n1 = g.step(1, fib.arrays["r_var"], fib.m)
    a, b = Context(fib, precision=PREC_MIXED, use_graph=True), Context(fib, precision=PREC_MIXED)
    a.step(*n0)
    b.step(*n0)
    a.set_mixed_passes(1)
    b.set_mixed_passes(1)
    assert a.step(*n1) == b.step(*n1)
    for k in ("r", "r_t", "a"):
        assert np.array_equal(a.get(k), b.get(k)), k
    with pytest.raises(BDError):
        a.set_mixed_passes(4)
