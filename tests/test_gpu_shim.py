"""The drop-in shim run as the reference's main.cpp runs it: the four C++
entry points of func_cuda.h:37-52 (cuda_application_init_D_Chol,
cuda_application_init_data, main_cuda, free_all), called by their mangled
names through ctypes with the reference's own example (golden fixture
ref_testdata_12nuc: 12 nucleosomes with linker histones), in main.cpp's
order (main.cpp:377-517): init with the start-up frames and angles, then one
main_cuda call per step with the reference's noise.  The state main_cuda
copies back must equal the reference's own steps to 1e-10 relative, the
FP64 parity bound.
"""
import ctypes as C
import subprocess

import numpy as np
import pytest

from conftest import load_golden, rel_err

pytestmark = pytest.mark.gpu
_ip, _dp = C.POINTER(C.c_int), C.POINTER(C.c_double)


def _mangled(lib_path, stem):
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True, text=True).stdout
    names = [ln.split()[-1] for ln in out.splitlines() if stem in ln]
    assert len(names) == 1, (stem, names)
    return names[0]


def _d(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(_dp)


def _i(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(_ip)


def test_shim_steps_match_reference():
    from brownian_dynamics_cuda_gb300 import LIB_PATH, load_library
    lib = load_library()
    fib, z = load_golden("ref_testdata_12nuc")
    sz, sc, ar, st = fib.sizes, fib.scalars, fib.arrays, fib.state
    n, n_c, Nq, n_t, n_tail, n_LH = sz["n"], sz["n_c"], sz["Nq"], sz["n_t"], sz["n_tail"], sz["n_LH"]
    keep = []

    def D(a):
        arr, p = _d(a)
        keep.append(arr)
        return p

    def I(a):  # noqa: E743
        arr, p = _i(a)
        keep.append(arr)
        return p

    r_all = np.concatenate([st["r"], st["r_t"], st["r_lh"]])
    rad_all = np.concatenate([ar["rad"], ar["t_rad"], ar["lh_rad"]])
    init_D = getattr(lib, _mangled(LIB_PATH, "cuda_application_init_D_Chol"))
    init_data = getattr(lib, _mangled(LIB_PATH, "cuda_application_init_data"))
    main_cuda = getattr(lib, _mangled(LIB_PATH, "_Z9main_cuda"))
    free_all = getattr(lib, _mangled(LIB_PATH, "free_all"))
    init_D.argtypes = [C.c_int]
    init_D(3 * fib.n_D)
    s0 = {k: z["s0_" + k] for k in ("a", "b", "c", "alpha", "beta", "gamma", "length", "a_dna", "b_dna", "c_dna",
                                     "alpha_p", "beta_p", "gamma_p", "beta_t", "beta_lh")}
    sig = [sc[k] for k in ("sigma_DNA_DNA", "sigma_DNA_Core", "sigma_Core_Core", "sigma_Tail_Tail",
                           "sigma_Tail_Linker", "sigma_Tail_Core")]
    force, torque = np.zeros(3 * n), np.zeros(3 * n)
    t_force, LH_force, energy = np.zeros(max(3 * n_tail, 1)), np.zeros(max(3 * n_LH, 1)), np.zeros(1)
    args = [
        (C.c_int, n_c), (C.c_int, 3 * n_c), (C.c_int, n), (C.c_int, 3 * n), (_ip, I(ar["type"])), (_dp, D(st["r"])),
        (_dp, D(s0["a"])), (_dp, D(s0["b"])), (_dp, D(s0["c"])), (_dp, D(s0["alpha"])), (_dp, D(s0["beta"])),
        (_dp, D(s0["gamma"])), (_dp, D(s0["length"])), (_dp, D(s0["a_dna"])), (_dp, D(s0["b_dna"])),
        (_dp, D(s0["c_dna"])), (_dp, D(s0["alpha_p"])), (_dp, D(s0["beta_p"])), (_dp, D(s0["gamma_p"])),
        (C.c_double, sc["h"]), (C.c_double, sc["g"]), (C.c_double, sc["s"]), (_dp, D(ar["phi_o"])),
        (C.c_double, sc["debyell"]), (C.c_double, sc["debye"]), (C.c_double, sc["q_l"]), (C.c_double, sc["k_e"]),
        (C.c_double, sc["k_ex"]), (C.c_double, sc["k_h1"])] + [(C.c_double, v) for v in sig] + [
        (C.c_int, Nq), (C.c_int, 3 * Nq), (_dp, D(ar["core_pos"])), (_dp, D(ar["core_q"])), (C.c_int, n_t),
        (C.c_int, n_tail), (C.c_int, 3 * n_tail), (_dp, D(ar["tail_pos"])), (_ip, I(ar["tail_fix"])),
        (_ip, I(ar["nc_t_flag"])), (_dp, D(st["r_t"])), (_dp, D(s0["beta_t"])), (_dp, D(ar["h_t"])),
        (_dp, D(ar["g_t"])), (_dp, D(ar["lo_t"])), (_dp, D(ar["beta_o_t"])), (_dp, D(ar["t_q"])),
        (_dp, D(ar["t_rad"])), (_ip, I(ar["t_grp"])), (_ip, I(ar["t_fix"])), (C.c_int, sz["n_lh_n"]),
        (C.c_int, sz["n_lh_g"]), (C.c_int, sz["n_lh_c"]), (C.c_int, n_LH), (C.c_int, 3 * n_LH),
        (_dp, D(ar["LH_g_pos"])), (_ip, I(ar["LH_conn"])), (_ip, I(ar["nc_lh_flag"])), (_dp, D(s0["beta_lh"])),
        (_dp, D(st["r_lh"])), (_dp, D(ar["LH_q"])), (_dp, D(ar["LH_vdw_hh"])), (_dp, D(ar["LH_vdw_hc"])),
        (_dp, D(ar["LH_vdw_hl"])), (_dp, D(ar["LH_vdw_ht"])), (_dp, D(ar["LH_kstr"])), (_dp, D(ar["LH_kben"])),
        (_dp, D(ar["LH_streq"])), (_dp, D(ar["LH_betaeq"])), (_dp, LH_force.ctypes.data_as(_dp)),
        (_dp, t_force.ctypes.data_as(_dp)), (_dp, force.ctypes.data_as(_dp)), (_dp, torque.ctypes.data_as(_dp)),
        (_dp, energy.ctypes.data_as(_dp)), (_dp, D(r_all)), (_dp, D(rad_all))]
    init_data.argtypes = [t for t, _ in args]
    init_data(*[v for _, v in args])
    # host copies main_cuda writes back (main.cpp's arrays)
    h = {k: np.zeros(v) for k, v in (("r", 3 * n), ("a", 3 * n), ("b", 3 * n), ("c", 3 * n),
                                      ("r_t", max(3 * n_tail, 1)), ("r_lh", max(3 * n_LH, 1)))}
    rad_h = rad_all.copy()
    flags = np.ascontiguousarray(ar["nc_lh_flag"], dtype=np.int32)
    main_cuda.argtypes = ([C.c_int] * 4 + [C.c_double] * 2 + [C.c_int] * 2 + [C.c_double] * 15 + [C.c_int] * 12 +
                          [C.c_double] * 3 + [_dp] * 10 + [_ip])
    steps = int(z["steps"])
    try:
        for s in range(steps):
            rr, p = np.ascontiguousarray(z[f"noise{s}_rr"]), np.ascontiguousarray(z[f"noise{s}_p"])
            e = np.zeros(1)
            main_cuda(n_c, 3 * n_c, s, steps, sc["time_step"], sc["del_"], 1, 1, sc["h"], sc["g"], sc["s"],
                      sc["debyell"], sc["debye"], sc["q_l"], sc["k_e"], sc["k_ex"], sc["k_h1"], *sig, Nq, 3 * Nq, n_t,
                      sz["n_lh_n"], sz["n_lh_g"], sz["n_lh_c"], n, 3 * n, n_tail, 3 * n_tail, n_LH, 3 * n_LH,
                      sc["a1"], sc["a2"], sc["s2dt"], rr.ctypes.data_as(_dp), p.ctypes.data_as(_dp),
                      e.ctypes.data_as(_dp), *[h[k].ctypes.data_as(_dp) for k in ("r", "a", "b", "c", "r_t", "r_lh")],
                      rad_h.ctypes.data_as(_dp), flags.ctypes.data_as(_ip))
            e_ref = float(z[f"step{s}_energy"])
            assert abs(e[0] - e_ref) <= 1e-10 * abs(e_ref), s
            for k in ("r", "a", "b", "c", "r_t", "r_lh"):
                ref = z[f"step{s}_{k}"]
                if ref.size:
                    assert rel_err(h[k][:ref.size], ref) <= 1e-10, (s, k)
    finally:
        free_all.argtypes = []
        free_all()
