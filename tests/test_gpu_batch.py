"""Batched replicas (bd_batch_*): replicas of uneven size and salt advanced
in one graph per batch step give, bit for bit, what each fiber's own
context gives with the same noise; bd_batch_run draws each replica's noise
from its own MT19937 stream (seed_base + i)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def replicas(tmp_path_factory):
    from brownian_dynamics_cuda_gb300.fiber_gen import config, make_fiber
    out = []
    for i in range(3):
        spec = config(2, seed=7, replica=i)
        out.append(make_fiber(spec, str(tmp_path_factory.mktemp(f"rep{i}"))))
    return out


@pytest.mark.parametrize("prec", [0, 1])
def test_batch_matches_single_contexts(replicas, prec):
    from brownian_dynamics_cuda_gb300 import Batch, Context, Noise
    b = Batch(replicas, precision=prec, use_graph=True)
    singles = [Context(f, precision=prec) for f in replicas]
    for step in range(2):
        noise = [Noise(100 + i).step(step, f.arrays["r_var"], f.m) for i, f in enumerate(replicas)]
        e = b.step([x[0] for x in noise], [x[1] for x in noise])
        for i, c in enumerate(singles):
            assert c.step(*noise[i]) == e[i]
            for k in ("r", "a", "r_t"):
                assert np.array_equal(c.get(k), b.contexts[i].get(k)), (i, k)


def test_batch_run_uses_per_replica_streams(replicas):
    from brownian_dynamics_cuda_gb300 import Batch, Context, Noise
    b = Batch(replicas, precision=1, use_graph=True)
    e = b.run(2, 500)
    for i, f in enumerate(replicas):
        c = Context(f, precision=1)
        g = Noise(500 + i)
        for step in range(2):
            ei = c.step(*g.step(step, f.arrays["r_var"], f.m))
        assert ei == e[i]
        assert np.array_equal(c.get("r"), b.contexts[i].get("r"))


def test_batch_run_device_noise(replicas):
    """bd_batch_run_device: each replica's noise generated on the device,
    one launch for all, no host wait between steps - equal bit for bit to
    the host-noise run with every stream set to the correctly rounded log,
    and to single contexts driven by such host streams."""
    from brownian_dynamics_cuda_gb300 import LOG_CR, Batch, Context, Noise
    bd = Batch(replicas, precision=1, use_graph=True)
    e = bd.run_device(3, 900)
    for i, f in enumerate(replicas):
        c = Context(f, precision=1)
        g = Noise(900 + i, log_mode=LOG_CR)
        for step in range(3):
            ei = c.step(*g.step(step, f.arrays["r_var"], f.m))
        assert ei == e[i], i
        for k in ("r", "a", "r_t"):
            assert np.array_equal(c.get(k), bd.contexts[i].get(k)), (i, k)
    # continues from where it stopped, with the generators' state kept
    e2 = bd.run_device(1, 900)
    assert np.all(np.isfinite(e2))
