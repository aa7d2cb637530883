"""Pins the CPU oracle bit for bit to the reference's own CPU functions
(func.cpp, readfile.cpp, mt.cpp, utilities.cpp compiled from the reference
sources into oracle/_ref).  Runs only where the reference tree is present."""
import os
import shutil

import numpy as np
import pytest

from conftest import REF_TESTDATA, have_ref

pytestmark = pytest.mark.skipif(not have_ref(), reason="reference sources not present")


@pytest.fixture(scope="module")
def testdata(tmp_path_factory):
    d = str(tmp_path_factory.mktemp("refdata"))
    for f in os.listdir(REF_TESTDATA):
        shutil.copy(os.path.join(REF_TESTDATA, f), d)
    return d


FILES = dict(core_file="core_data.reg.150mM", tail_file="tail_data.mod.200mM", lh_file="LH_N0G6C22.in")


def test_loader_matches_reference_readers(testdata):
    from brownian_dynamics_cuda_gb300 import Fiber
    from oracle.pyoracle import Reference
    fib = Fiber.load(testdata, **FILES)
    ref = Reference(testdata, FILES["core_file"], FILES["tail_file"], FILES["lh_file"], seed=1)
    for k in ("rad", "phi_o", "r_var", "core_pos", "core_q", "tail_pos", "h_t", "g_t", "lo_t", "beta_o_t", "t_q",
              "t_rad", "t_grp", "t_fix", "LH_g_pos", "LH_q", "LH_vdw_hh", "LH_vdw_hc", "LH_vdw_hl", "LH_vdw_ht",
              "LH_kstr", "LH_kben", "LH_streq", "LH_betaeq", "lh_rad", "LH_conn", "nc_lh_flag", "type"):
        assert np.array_equal(fib.arrays[k].astype(np.float64), ref.get(k)), k
    for k in ("r_t", "r_lh"):
        assert np.array_equal(fib.state[k], ref.get(k)), k
    for k in ("h", "g", "s", "debye", "debyell", "q_l", "k_e", "k_ex", "a1", "a2", "del_", "s2dt"):
        assert fib.scalars[k] == ref.scalars[k], k


def test_oracle_bitwise_two_steps(testdata):
    from brownian_dynamics_cuda_gb300 import Fiber
    from oracle.pyoracle import Oracle, Reference
    fib = Fiber.load(testdata, **FILES)
    ref = Reference(testdata, FILES["core_file"], FILES["tail_file"], FILES["lh_file"], seed=31)
    o = Oracle(fib)
    f, fr = o.forces(), ref.forces()
    for k in ("force", "torque", "t_force", "LH_force"):
        assert np.array_equal(f[k], fr[k]), k
    D, L = o.tensor()
    Dr, Lr = ref.tensor()
    assert np.array_equal(D, Dr) and np.array_equal(L, Lr)
    for s in range(2):
        rr, p = ref.noise(s)
        assert o.step(rr, p) == ref.step(rr, p)
        for k in ("r", "a", "b", "c", "r_t", "r_lh", "rd", "force", "torque", "t_force", "LH_force"):
            assert np.array_equal(o.get(k), ref.get(k)), (s, k)


def test_noise_streams_bitwise(testdata):
    from brownian_dynamics_cuda_gb300 import Fiber, Noise
    from oracle.pyoracle import OracleNoise, Reference
    fib = Fiber.load(testdata, **FILES)
    ref = Reference(testdata, FILES["core_file"], FILES["tail_file"], FILES["lh_file"], seed=12345)
    assert np.array_equal(ref.mt_raw(5489, 3000), Noise(5489).u32(3000))
    ref = Reference(testdata, FILES["core_file"], FILES["tail_file"], FILES["lh_file"], seed=12345)
    pn, on = Noise(12345), OracleNoise(12345)
    for s in (0, 1, 2):
        rr, p = ref.noise(s)
        rr2, p2 = pn.step(s, fib.arrays["r_var"], 3 * fib.n_D)
        rr3, p3 = on.step(s, fib.arrays["r_var"], 3 * fib.n_D)
        assert np.array_equal(rr, rr2) and np.array_equal(p, p2)
        assert np.array_equal(rr, rr3) and np.array_equal(p, p3)


def test_oracle_parallel_cholesky_bitwise(testdata):
    from brownian_dynamics_cuda_gb300 import Fiber
    from oracle.pyoracle import Oracle, cholesky
    fib = Fiber.load(testdata, **FILES)
    D, L = Oracle(fib).tensor()
    L4, neg = cholesky(D, nthreads=4)
    assert neg == 0 and np.array_equal(np.tril(L4), L)


def test_text_restart_matches_reference_readers(tmp_path):
    """restart = 1 in setup.txt: the loader takes the start structure, tails
    and LH beads from restart_*.txt exactly as the reference's own readers
    (Read_restart_ini / _tail / _LH, readfile.cpp) do in main.cpp."""
    import re
    from brownian_dynamics_cuda_gb300 import Fiber
    from brownian_dynamics_cuda_gb300.fiber_gen import FiberSpec, write_fiber
    from oracle.pyoracle import Oracle, Reference
    d = str(tmp_path)
    files = write_fiber(FiberSpec(3, [30] * 3, lh=True, seed=8), d)
    f0 = Fiber.load(d, **files)
    rng = np.random.default_rng(2)
    for k, fn in (("r", "restart_r.txt"), ("a", "restart_a.txt"), ("b", "restart_b.txt"), ("c", "restart_c.txt"),
                  ("r_t", "restart_tail.txt"), ("r_lh", "restart_lh.txt")):
        v = f0.state[k] + rng.normal(scale=0.1, size=f0.state[k].size)
        with open(os.path.join(d, fn), "w") as f:
            f.write("".join(f"{x:.15f}\n" for x in v))
    with open(os.path.join(d, "restart_Er.txt"), "w") as f:
        f.write("0.000000000000000\n" * f0.state["r"].size)
    setup = open(os.path.join(d, "setup.txt")).read()
    open(os.path.join(d, "setup.txt"), "w").write(re.sub(r"^(restart\s+)0$", r"\g<1>1", setup, flags=re.M))
    fib = Fiber.load(d, **files)
    ref = Reference(d, files["core_file"], files["tail_file"], files["lh_file"], seed=1)
    for k in ("r", "r_t", "r_lh"):
        assert np.array_equal(fib.state[k], ref.get(k)), k
    o = Oracle(fib)  # frames refreshed as main.cpp:164 does after the restart read
    for k in ("a", "b", "c", "beta_t", "beta_lh"):
        assert np.array_equal(o.get(k), ref.get(k)), k
