"""bd_set_lh_flags: a context resized in place for a new linker-histone
binding (main.cpp:386-465 releases or binds one core's linker histone every
100 steps) continues exactly as a context created from scratch with the same
state and binding: same sizes, and bit-for-bit the same steps."""
import dataclasses

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ANGLES = ("alpha", "beta", "gamma", "length", "a_dna", "b_dna", "c_dna", "alpha_p", "beta_p", "gamma_p")


@pytest.mark.parametrize("prec", [0, 1])
def test_release_one_linker_histone(tmp_path, prec):
    from brownian_dynamics_cuda_gb300 import Context, Noise
    from brownian_dynamics_cuda_gb300.fiber_gen import FiberSpec, make_fiber
    fib = make_fiber(FiberSpec(4, [30] * 4, lh=True, seed=2), str(tmp_path))
    nlh = fib.sizes["n_lh_n"] + fib.sizes["n_lh_c"]
    a = Context(fib, precision=prec)
    nz = Noise(5)
    for s in range(2):
        a.step(*nz.step(s, fib.arrays["r_var"], a.m))
    flags = fib.arrays["nc_lh_flag"].copy()
    assert flags.sum() == fib.sizes["n_c"]
    flags[1] = 0  # core 1 releases its linker histone
    keep = np.ones(fib.sizes["n_LH"], bool)
    keep[nlh:2 * nlh] = False
    r_lh = a.get("r_lh").reshape(-1, 3)[keep].ravel()
    lh_rad = fib.arrays["lh_rad"][keep]
    state = {k: a.get(k) for k in ("r", "a", "b", "c", "r_t")}
    angles = {k: a.get(k) for k in ANGLES}
    a.set_lh_flags(flags, r_lh, lh_rad)
    n_lh = int(flags.sum()) * nlh
    assert a.n_LH == n_lh and a.m == 3 * (fib.sizes["n"] + fib.sizes["n_tail"] + n_lh)
    sizes = dict(fib.sizes, n_LH=n_lh)
    arrays = dict(fib.arrays, nc_lh_flag=flags, lh_rad=lh_rad)
    fib2 = dataclasses.replace(fib, sizes=sizes, arrays=arrays, state=dict(state, r_lh=r_lh))
    b = Context(fib2, precision=prec, refresh=False, angles=angles)
    for k in ("r", "a", "b", "c", "r_t", "r_lh", "beta", "length", "a_dna", "beta_p", "beta_lh"):
        assert np.array_equal(a.get(k), b.get(k)), k
    for s in range(2, 4):
        rr, p = nz.step(s, fib.arrays["r_var"], a.m)
        assert a.step(rr, p) == b.step(rr, p)
        for k in ("r", "a", "r_t", "r_lh"):
            assert np.array_equal(a.get(k), b.get(k)), (s, k)


@pytest.mark.parametrize("prec", [0, 1])
def test_bind_one_linker_histone_in_place(tmp_path, prec):
    """Growth: a context created with core 1's linker histone released binds
    it again; the resize stays inside the buffers bd_create sized for every
    core bound (the device's free memory is unchanged), and the context
    continues exactly as one created from scratch with the new binding."""
    import torch
    from brownian_dynamics_cuda_gb300 import Context, Noise
    from brownian_dynamics_cuda_gb300.fiber_gen import FiberSpec, make_fiber
    full = make_fiber(FiberSpec(4, [30] * 4, lh=True, seed=3), str(tmp_path))
    nlh = full.sizes["n_lh_n"] + full.sizes["n_lh_c"]
    flags = full.arrays["nc_lh_flag"].copy()
    flags[1] = 0
    keep = np.ones(full.sizes["n_LH"], bool)
    keep[nlh:2 * nlh] = False
    part = dataclasses.replace(full, sizes=dict(full.sizes, n_LH=int(flags.sum()) * nlh),
                               arrays=dict(full.arrays, nc_lh_flag=flags, lh_rad=full.arrays["lh_rad"][keep]),
                               state=dict(full.state, r_lh=full.state["r_lh"].reshape(-1, 3)[keep].ravel()))
    a = Context(part, precision=prec)
    nz = Noise(8)
    for s in range(2):
        a.step(*nz.step(s, full.arrays["r_var"], a.m))
    r_lh_now = a.get("r_lh").reshape(-1, 3)
    r_lh_new = np.concatenate([r_lh_now[:nlh], full.state["r_lh"].reshape(-1, 3)[nlh:2 * nlh], r_lh_now[nlh:]]).ravel()
    state = {k: a.get(k) for k in ("r", "a", "b", "c", "r_t")}
    angles = {k: a.get(k) for k in ANGLES}
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    a.set_lh_flags(full.arrays["nc_lh_flag"], r_lh_new, full.arrays["lh_rad"])
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert a.n_LH == full.sizes["n_LH"] and a.m == full.m
    b = Context(dataclasses.replace(full, state=dict(state, r_lh=r_lh_new)), precision=prec, refresh=False,
                angles=angles)
    for k in ("r", "a", "b", "c", "r_t", "r_lh", "beta", "length", "a_dna", "beta_p", "beta_lh"):
        assert np.array_equal(a.get(k), b.get(k)), k
    for s in range(2, 4):
        rr, p = nz.step(s, full.arrays["r_var"], a.m)
        assert a.step(rr, p) == b.step(rr, p)
        for k in ("r", "a", "r_t", "r_lh"):
            assert np.array_equal(a.get(k), b.get(k)), (s, k)


@pytest.mark.parametrize("prec", [0, 1])
def test_bind_first_linker_histone(tmp_path, prec):
    """From no linker histone bound (n_LH = 0) to one: the context still has
    room for every core's, and continues as one created with the binding."""
    import torch
    from brownian_dynamics_cuda_gb300 import Context, Noise
    from brownian_dynamics_cuda_gb300.fiber_gen import FiberSpec, make_fiber
    full = make_fiber(FiberSpec(4, [30] * 4, lh=True, seed=4), str(tmp_path))
    nlh = full.sizes["n_lh_n"] + full.sizes["n_lh_c"]
    none = np.zeros_like(full.arrays["nc_lh_flag"])
    part = dataclasses.replace(full, sizes=dict(full.sizes, n_LH=0),
                               arrays=dict(full.arrays, nc_lh_flag=none, lh_rad=full.arrays["lh_rad"][:0]),
                               state=dict(full.state, r_lh=full.state["r_lh"][:0]))
    a = Context(part, precision=prec)
    nz = Noise(9)
    for s in range(2):
        a.step(*nz.step(s, full.arrays["r_var"], a.m))
    flags = none.copy()
    flags[2] = 1
    r_lh_new = full.state["r_lh"].reshape(-1, 3)[2 * nlh:3 * nlh].ravel()
    rad_new = full.arrays["lh_rad"][2 * nlh:3 * nlh]
    state = {k: a.get(k) for k in ("r", "a", "b", "c", "r_t")}
    angles = {k: a.get(k) for k in ANGLES}
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    a.set_lh_flags(flags, r_lh_new, rad_new)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert a.n_LH == nlh and a.m == 3 * (full.sizes["n"] + full.sizes["n_tail"] + nlh)
    fib1 = dataclasses.replace(full, sizes=dict(full.sizes, n_LH=nlh),
                               arrays=dict(full.arrays, nc_lh_flag=flags, lh_rad=rad_new),
                               state=dict(state, r_lh=r_lh_new))
    b = Context(fib1, precision=prec, refresh=False, angles=angles)
    for k in ("r", "a", "b", "c", "r_t", "r_lh", "beta", "length", "beta_lh"):
        assert np.array_equal(a.get(k), b.get(k)), k
    for s in range(2, 4):
        rr, p = nz.step(s, full.arrays["r_var"], a.m)
        assert a.step(rr, p) == b.step(rr, p)
        for k in ("r", "a", "r_t", "r_lh"):
            assert np.array_equal(a.get(k), b.get(k)), (s, k)
