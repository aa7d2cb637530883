"""Synthetic fibers have the sizes of the benchmark configurations and the
stated charge model; files round-trip through the library's readers."""
import numpy as np
import pytest

from brownian_dynamics_cuda_gb300.fiber_gen import config, linker_beads, make_fiber

# n, n_tail, n_LH per configuration (12/50/24/200 nucleosomes)
SIZES = {0: (48, 600, 0), 1: (300, 2500, 1100), 3: (96, 1200, 0), 4: (1000, 10000, 4400)}


def test_linker_beads():
    assert [linker_beads(b) for b in (20, 26, 30, 44, 60)] == [2, 3, 3, 5, 7]


@pytest.mark.parametrize("idx", [0, 1, 3, 4])
def test_config_sizes(idx, tmp_path):
    fib = make_fiber(config(idx), str(tmp_path))
    n, nt, nl = SIZES[idx]
    assert (fib.sizes["n"], fib.sizes["n_tail"], fib.sizes["n_LH"]) == (n, nt, nl)
    q = fib.arrays["core_q"]
    assert q.size == 300 and abs(q.sum() + 100.0) < 1e-5 and q.min() >= -1 - 1e-12 and q.max() <= 1 + 1e-12
    r = fib.state["r"].reshape(-1, 3)
    assert np.all(np.isfinite(r))
    typ = fib.arrays["type"]
    assert typ[0] == 1 and typ[-1] == 0


def test_config2_replicas_are_uneven():
    specs = [config(2, replica=k) for k in range(16)]
    sizes = {s.n_nuc for s in specs}
    assert len(sizes) > 4 and min(sizes) >= 12 and max(sizes) <= 48
    assert {s.cs for s in specs} <= {0.05, 0.1, 0.15}
    assert all(2 <= linker_beads(b) <= 7 for s in specs for b in s.linker_bp)


def test_generator_is_deterministic(tmp_path):
    a = make_fiber(config(0, seed=3), str(tmp_path / "a"))
    b = make_fiber(config(0, seed=3), str(tmp_path / "b"))
    assert np.array_equal(a.state["r"], b.state["r"]) and np.array_equal(a.arrays["core_q"], b.arrays["core_q"])
