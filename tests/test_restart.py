"""Binary restart files (bd_restart_*) and the noise generator's state
(bd_noise_get_state / bd_noise_set_state) on the CPU: a generator restored
from a saved state continues the stream bit for bit; a restart file returns
exactly what was written, rejects foreign and truncated files and size
mismatches."""
import numpy as np
import pytest

from brownian_dynamics_cuda_gb300 import BDError, Noise
from brownian_dynamics_cuda_gb300.capi import RESTART_ARRAYS, _restart_len, restart_read, restart_write


def test_noise_state_round_trip():
    r_var = np.linspace(0.1, 1.0, 33)
    g = Noise(7)
    for s in range(3):
        g.step(s, r_var, 100)  # 133 draws per step: a cached deviate is pending after 3 steps
    st = g.get_state()
    assert st[2] == 1
    h = Noise(1)
    h.set_state(st)
    for s in range(3, 6):
        a, b = g.step(s, r_var, 100), h.step(s, r_var, 100)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def _arrays(n=7, nc=2, nt=5, nl=3, seed=0):
    rng = np.random.default_rng(seed)
    return {k: rng.normal(size=_restart_len(k, n, nc, nt, nl)) for k in RESTART_ARRAYS}


def test_restart_round_trip(tmp_path):
    arrays = _arrays()
    flags = np.array([1, 0], dtype=np.int32)
    g = Noise(11)
    g.step(0, np.ones(21), 45)
    path = str(tmp_path / "run.rst")
    restart_write(path, 1234, arrays, flags, g)
    h = Noise(3)
    step, back, fl, has = restart_read(path, h)
    assert step == 1234 and has and np.array_equal(fl, flags)
    for k in RESTART_ARRAYS:
        assert np.array_equal(back[k], arrays[k]), k
    a, b = g.step(1, np.ones(21), 45), h.step(1, np.ones(21), 45)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_restart_rejects_bad_files(tmp_path):
    path = str(tmp_path / "x.rst")
    with open(path, "wb") as f:
        f.write(b"NOTARESTARTFILE" * 4)
    with pytest.raises(BDError):
        restart_read(path)
    good = str(tmp_path / "g.rst")
    restart_write(good, 5, _arrays(), np.array([1, 1], dtype=np.int32))
    data = open(good, "rb").read()
    with open(path, "wb") as f:
        f.write(data[:len(data) // 2])
    with pytest.raises(BDError):
        restart_read(path)


def test_text_restart_is_read_back_by_the_loader(tmp_path):
    """bd_write_restart_text writes the reference's restart_*.txt files
    (write_restart: 15 decimals, one value per line); with restart = 1 in
    setup.txt the loader takes r, a, b, c, r_t and r_lh from them
    (main.cpp:143-153, :218-220, :279-281)."""
    import ctypes as C
    import re
    from brownian_dynamics_cuda_gb300 import Fiber, load_library
    from brownian_dynamics_cuda_gb300.capi import _check
    from brownian_dynamics_cuda_gb300.fiber_gen import FiberSpec, write_fiber
    d = str(tmp_path)
    files = write_fiber(FiberSpec(3, [30] * 3, lh=True, seed=8), d)
    f0 = Fiber.load(d, **files)
    rng = np.random.default_rng(1)
    new = {k: f0.state[k] + rng.normal(scale=0.3, size=f0.state[k].size) for k in ("r", "a", "b", "c", "r_t", "r_lh")}
    L = load_library()
    dp = C.POINTER(C.c_double)
    L.bd_write_restart_text.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int] + [dp] * 7
    sz = f0.sizes
    p = lambda a: a.ctypes.data_as(dp)
    _check(L.bd_write_restart_text(d.encode(), sz["n"], sz["n_tail"], sz["n_LH"], p(new["r"]), p(new["a"]),
                                   p(new["b"]), p(new["c"]), None, p(new["r_t"]), p(new["r_lh"])))
    lines = open(f"{d}/restart_r.txt").read().splitlines()
    assert len(lines) == 3 * sz["n"] and all(re.fullmatch(r"-?\d+\.\d{15}", x) for x in lines)
    setup = open(f"{d}/setup.txt").read()
    setup = re.sub(r"^(restart\s+)0$", r"\g<1>1", setup, flags=re.M)
    open(f"{d}/setup.txt", "w").write(setup)
    f1 = Fiber.load(d, **files)
    for k in new:
        assert np.allclose(f1.state[k], new[k], rtol=0, atol=6e-16 * max(1.0, np.abs(new[k]).max()) * 10), k
    assert f1.sizes == f0.sizes


def test_restart_rejects_generator_index_out_of_range(tmp_path):
    """A restart file whose generator index lies outside [0, 625] is refused
    and leaves the caller's generator as it was (next() would read st[idx])."""
    import struct
    g = Noise(11)
    g.step(0, np.ones(21), 45)
    good = str(tmp_path / "g.rst")
    restart_write(good, 9, _arrays(), np.array([1, 1], dtype=np.int32), g)
    data = bytearray(open(good, "rb").read())
    # the generator's state ends the file: 624 words, index, cached flag, cached deviate
    assert struct.unpack_from("<i", data, len(data) - 16)[0] == g.get_state()[1]
    for bad in (626, 100000, -1):
        struct.pack_into("<i", data, len(data) - 16, bad)
        path = str(tmp_path / f"bad{bad}.rst")
        open(path, "wb").write(bytes(data))
        h, ref = Noise(3), Noise(3)
        with pytest.raises(BDError, match="index"):
            restart_read(path, h)
        a, b = h.step(0, np.ones(21), 45), ref.step(0, np.ones(21), 45)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
