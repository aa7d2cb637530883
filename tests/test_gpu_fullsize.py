"""Size-independent properties at the benchmark sizes (too large for the
CPU oracle to finish in seconds): the factor reproduces D, the step is
finite, deterministic, and its noise displacement has the statistics of
sqrt(2 dt) L p."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cfg1(tmp_path_factory):
    from brownian_dynamics_cuda_gb300.fiber_gen import config, make_fiber
    return make_fiber(config(1), str(tmp_path_factory.mktemp("cfg1")))


def test_cfg1_factor_reproduces_tensor(cfg1):
    from brownian_dynamics_cuda_gb300 import Context
    c = Context(cfg1)
    D = c.diffusion_tensor()
    L = c.cholesky()
    assert c.negative_pivots() == 0
    rng = np.random.default_rng(0)
    cols = rng.choice(c.m, 48, replace=False)
    R = L @ L[cols].T - D[:, cols]               # sampled columns of L L^T - D
    assert np.abs(R).max() <= 1e-11 * np.abs(D).max()


def test_cfg1_step_finite_and_deterministic(cfg1):
    from brownian_dynamics_cuda_gb300 import Context, Noise
    noise = Noise(2024)
    rr, p = noise.step(0, cfg1.arrays["r_var"], cfg1.m)
    a, b = Context(cfg1, use_graph=True), Context(cfg1)
    ea, eb = a.step(rr, p), b.step(rr, p)
    assert np.isfinite(ea) and ea == eb
    for k in ("r", "r_t", "r_lh", "a"):
        x = a.get(k)
        assert np.all(np.isfinite(x)) and np.array_equal(x, b.get(k))
    d = a.get("r") - cfg1.state["r"]
    assert 0 < np.abs(d).max() < 1.0   # nm per ps step


def test_cfg1_mixed_vs_fp64_displacement(cfg1):
    """At the benchmark size the mixed step's displacement stays within
    1e-6 (relative, max norm) of the FP64 step's."""
    from brownian_dynamics_cuda_gb300 import PREC_FP64, PREC_MIXED, Context, Noise
    rr, p = Noise(77).step(0, cfg1.arrays["r_var"], cfg1.m)
    a, b = Context(cfg1, precision=PREC_FP64), Context(cfg1, precision=PREC_MIXED)
    a.step(rr, p)
    b.step(rr, p)
    assert b.negative_pivots() == 0
    for k in ("r", "r_t", "r_lh"):
        d64 = a.get(k) - cfg1.state[k]
        dm = b.get(k) - cfg1.state[k]
        assert np.abs(dm - d64).max() <= 1e-6 * np.abs(d64).max(), k


def test_cfg1_mixed_factor_matches_fp64(cfg1):
    """The tensor-core factor of the 3N = 11,700 tensor agrees with the FP64
    factor tile by tile (FP32-class: within 2e-6 of max |L|), twice in a row
    on one context (the second factorisation reuses the panel buffers)."""
    from brownian_dynamics_cuda_gb300 import PREC_FP64, PREC_MIXED, Context
    L64 = Context(cfg1, precision=PREC_FP64).cholesky()
    cm = Context(cfg1, precision=PREC_MIXED)
    scale = np.abs(L64).max()
    for _ in range(2):
        Lm = cm.cholesky()
        assert cm.negative_pivots() == 0
        assert np.isfinite(Lm).all()
        assert np.abs(Lm - L64).max() <= 2e-6 * scale


def test_mixed_factor_more_panels_than_sms(tmp_path):
    """3N = 25,410 (199 panels): panel launches have more CTAs than the GPU
    has SMs, so some panel CTAs start after others have finished; the mixed
    noise displacement still matches the FP64 one."""
    from brownian_dynamics_cuda_gb300 import PREC_FP64, PREC_MIXED, Context
    from brownian_dynamics_cuda_gb300.fiber_gen import FiberSpec, make_fiber
    spec = FiberSpec(110, [26 if k % 2 == 0 else 44 for k in range(110)], lh=True, seed=1,
                     lh_charge_range=(0.0, 1.0), steps=10, name="n110")
    fib = make_fiber(spec, str(tmp_path))
    assert fib.m > 152 * 128
    p = np.random.default_rng(0).normal(size=fib.m)
    cm = Context(fib, precision=PREC_MIXED)
    rm = cm.noise_displacement(p)
    assert cm.negative_pivots() == 0
    r64 = Context(fib, precision=PREC_FP64).noise_displacement(p)
    assert np.abs(rm - r64).max() <= 1e-6 * np.abs(r64).max()


def test_concurrent_mixed_steps_on_two_streams(cfg1):
    """Two contexts' mixed steps (each a CUDA graph with the 92-launch
    tensor-core factorisation) replayed on two streams at once, so that
    k_chol_step launches of the two run side by side on the GPU: every
    state equals that of the same steps run one context after the other,
    bit for bit, eight steps each."""
    import torch
    from brownian_dynamics_cuda_gb300 import PREC_MIXED, Context, Noise
    from brownian_dynamics_cuda_gb300.fiber_gen import config, make_fiber
    import tempfile
    fibs = [cfg1, make_fiber(config(1, seed=2), tempfile.mkdtemp())]
    steps = 8
    noise = []
    for i, f in enumerate(fibs):
        g = Noise(300 + i)
        rows = [g.step(s, f.arrays["r_var"], f.m) for s in range(steps)]
        noise.append(([torch.tensor(r[0], device="cuda") for r in rows],
                      [torch.tensor(r[1], device="cuda") for r in rows]))
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]

    def run(concurrent):
        ctx = [Context(f, precision=PREC_MIXED, use_graph=True, stream=s.cuda_stream) for f, s in zip(fibs, streams)]
        torch.cuda.synchronize()
        if concurrent:
            for s in range(steps):
                for c, (rr, p) in zip(ctx, noise):
                    c.step_device(rr[s].data_ptr(), p[s].data_ptr())
        else:
            for c, (rr, p), st in zip(ctx, noise, streams):
                for s in range(steps):
                    c.step_device(rr[s].data_ptr(), p[s].data_ptr())
                st.synchronize()
        torch.cuda.synchronize()
        out = [{k: c.get(k) for k in ("r", "a", "r_t", "r_lh")} for c in ctx]
        assert all(c.negative_pivots() == 0 for c in ctx)
        for c in ctx:
            c.close()
        return out

    seq, conc = run(False), run(True)
    for i in range(2):
        for k in seq[i]:
            assert np.array_equal(seq[i][k], conc[i][k]), (i, k)
