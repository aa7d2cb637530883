"""The linker-histone binding Monte Carlo pieces on the host (main.cpp:386-465):
the decision (bd_lh_mc), the bead placement for a new binding (bd_lh_rebind,
build_LH + the keep-old-beads merge) and the split noise draws
(bd_noise_uniforms + bd_noise_draws == bd_noise_step)."""
import ctypes as C

import numpy as np
import pytest

from brownian_dynamics_cuda_gb300 import Noise, load_library
from brownian_dynamics_cuda_gb300.capi import _check, bd_model, bd_state

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def _lib():
    L = load_library()
    L.bd_lh_mc.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, _ip, _ip]
    L.bd_lh_rebind.argtypes = [C.c_int, _ip, C.c_int, _dp, _dp, _dp, _dp, C.c_int, _dp, _dp, _ip, _dp, _ip, _dp, _dp]
    L.bd_system_lh_template.argtypes = [C.c_void_p, _dp, _dp]
    L.bd_noise_uniforms.argtypes = [C.c_void_p, C.c_int, _dp]
    L.bd_noise_draws.argtypes = [C.c_void_p, C.c_int, _dp, C.c_int, _dp, _dp]
    return L


def _p(a, t=_dp):
    return a.ctypes.data_as(t)


def test_split_noise_equals_step():
    L = _lib()
    r_var = np.linspace(0.2, 0.9, 21)
    a, b = Noise(3), Noise(3)
    for step in (0, 1, 99, 100, 101):
        rr_a, p_a = a.step(step, r_var, 57)
        if step % 100 == 0:
            u = np.zeros(2)
            _check(L.bd_noise_uniforms(b._h, 2, _p(u)))
            assert np.all((u >= 0) & (u <= 1))
        rr_b, p_b = np.zeros(21), np.zeros(57)
        _check(L.bd_noise_draws(b._h, 21, _p(r_var), 57, _p(rr_b), _p(p_b)))
        assert np.array_equal(rr_a, rr_b) and np.array_equal(p_a, p_b)


def _mc_ref(flags, u_random, u_core, unbind, pbind):
    """main.cpp:386-412 restated."""
    f = list(flags)
    nc = len(f)
    nb = int(nc * u_core)
    if nb >= nc:
        nb = nc - 1
    if f[nb] > 0.5:
        if u_random <= unbind:
            f[nb] = 0
    elif u_random <= pbind:
        f[nb] = 1
    return f


def test_mc_decision():
    L = _lib()
    rng = np.random.default_rng(0)
    for _ in range(300):
        nc = int(rng.integers(1, 9))
        flags = rng.integers(0, 2, nc).astype(np.int32)
        u_random, u_core = float(rng.random()), float(rng.choice([rng.random(), 1.0, 0.0]))
        unbind, pbind = float(rng.random()), float(rng.random())
        ref = _mc_ref(flags, u_random, u_core, unbind, pbind)
        got, ch = flags.copy(), C.c_int()
        _check(L.bd_lh_mc(nc, u_random, u_core, unbind, pbind, _p(got, _ip), C.byref(ch)))
        assert list(got) == ref and ch.value == int(list(flags) != ref)


def _load(tmp_path):
    from brownian_dynamics_cuda_gb300.fiber_gen import FiberSpec, write_fiber
    L = _lib()
    d = str(tmp_path)
    files = write_fiber(FiberSpec(4, [30] * 4, lh=True, seed=3), d)
    h = C.c_void_p()
    _check(L.bd_system_load(d.encode(), b"data_mod", files["core_file"].encode(), files["tail_file"].encode(),
                            files["lh_file"].encode(), b"LH.in", C.byref(h)))
    m, s = bd_model(), bd_state()
    _check(L.bd_system_model(h, C.byref(m)))
    _check(L.bd_system_state(h, C.byref(s)))
    n, nc, nl = m.n, m.n_c, m.n_LH
    nlh = m.n_lh_n + m.n_lh_c
    arr = lambda p, k: np.ctypeslib.as_array(p, shape=(k,)).copy()
    sysd = {"n": n, "nc": nc, "nlh": nlh, "type": arr(m.type, n).astype(np.int32),
            "flags": arr(m.nc_lh_flag, nc).astype(np.int32), "r_lh": arr(s.r_lh, 3 * nl), "lh_rad": arr(m.lh_rad, nl)}
    for k in ("r", "a", "b", "c"):
        sysd[k] = arr(getattr(s, k), 3 * n)
    tpos, trad = np.zeros(3 * nlh), np.zeros(nlh)
    _check(L.bd_system_lh_template(h, _p(tpos), _p(trad)))
    L.bd_system_free(h)
    return sysd, tpos, trad


def _rebind(S, tpos, trad, old_flags, old_r_lh, new_flags):
    L = _lib()
    nl = int(new_flags.sum()) * S["nlh"]
    out, rad = np.zeros(3 * nl), np.zeros(nl)
    old = old_r_lh if old_r_lh is not None else np.zeros(1)
    _check(L.bd_lh_rebind(S["n"], _p(S["type"], _ip), S["nc"], _p(S["r"]), _p(S["a"]), _p(S["b"]), _p(S["c"]),
                          S["nlh"], _p(tpos), _p(trad), _p(old_flags, _ip), _p(old), _p(new_flags, _ip), _p(out),
                          _p(rad)))
    return out, rad


def test_rebind_places_the_loaders_beads(tmp_path):
    S, tpos, trad = _load(tmp_path)
    assert S["flags"].sum() == S["nc"]
    # every core newly bound: the template in each core frame, as the loader's build_LH
    out, rad = _rebind(S, tpos, trad, np.zeros(S["nc"], np.int32), None, S["flags"])
    assert np.array_equal(out, S["r_lh"]) and np.array_equal(rad, S["lh_rad"])
    # nothing changes: the old beads come back
    moved = S["r_lh"] + 0.25
    out, _ = _rebind(S, tpos, trad, S["flags"], moved, S["flags"])
    assert np.array_equal(out, moved)


def test_rebind_keeps_old_beads_in_order(tmp_path):
    S, tpos, trad = _load(tmp_path)
    nlh = S["nlh"]
    old = np.array([1, 0, 1, 1], np.int32)
    new = np.array([1, 1, 0, 1], np.int32)
    old_r = np.arange(3 * 3 * nlh, dtype=float)
    out, _ = _rebind(S, tpos, trad, old, old_r, new)
    blocks = out.reshape(3, nlh, 3)
    fresh, _ = _rebind(S, tpos, trad, np.zeros(4, np.int32), None, np.ones(4, np.int32))
    fresh = fresh.reshape(4, nlh, 3)
    ob = old_r.reshape(3, nlh, 3)
    assert np.array_equal(blocks[0], ob[0])      # core 0: kept (old block 0)
    assert np.array_equal(blocks[1], fresh[1])   # core 1: newly bound, template
    assert np.array_equal(blocks[2], ob[2])      # core 3: kept (old block 2)
