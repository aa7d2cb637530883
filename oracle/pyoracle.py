"""Test infrastructure: ctypes wrapper of the CPU oracle (oracle/liboracle.so).

Only tests, __graft_entry__.smoke() and the CPU-baseline legs of bench.py use
this module; it checks the product, it is never the product.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libbdref.so")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class orc_system(C.Structure):
    _fields_ = [(k, C.c_int) for k in ("n", "n_c", "Nq", "n_t", "n_tail", "n_lh_n", "n_lh_g", "n_lh_c", "n_LH")] + [
        (k, C.c_double) for k in ("h", "g", "s", "debyell", "debye", "q_l", "k_e", "k_ex", "sigma_DNA_DNA",
                                  "sigma_DNA_Core", "sigma_Core_Core", "sigma_Tail_Tail", "sigma_Tail_Linker",
                                  "sigma_Tail_Core", "a1", "a2", "time_step", "del_", "s2dt")
    ] + [
        ("type", _ip), ("rad", _dp), ("phi_o", _dp), ("core_pos", _dp), ("core_q", _dp), ("tail_pos", _dp),
        ("tail_fix", _ip), ("nc_t_flag", _ip), ("h_t", _dp), ("g_t", _dp), ("lo_t", _dp), ("beta_o_t", _dp),
        ("t_q", _dp), ("t_rad", _dp), ("t_grp", _ip), ("t_fix", _ip), ("LH_g_pos", _dp), ("LH_conn", _ip),
        ("nc_lh_flag", _ip), ("LH_q", _dp), ("LH_vdw_hh", _dp), ("LH_vdw_hc", _dp), ("LH_vdw_hl", _dp),
        ("LH_vdw_ht", _dp), ("LH_kstr", _dp), ("LH_kben", _dp), ("LH_streq", _dp), ("LH_betaeq", _dp),
        ("lh_rad", _dp),
    ]


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_LIB):
            raise FileNotFoundError(ORACLE_LIB + " missing: run make -C oracle")
        L = C.CDLL(ORACLE_LIB)
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.POINTER(orc_system)] + [_dp] * 6 + [C.c_int]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_forces.restype = C.c_double
        L.orc_forces.argtypes = [C.c_void_p] + [_dp] * 4
        L.orc_tensor.argtypes = [C.c_void_p, _dp, _dp]
        L.orc_step.restype = C.c_double
        L.orc_step.argtypes = [C.c_void_p, _dp, _dp]
        L.orc_em_update.argtypes = [C.c_void_p] + [_dp] * 6
        L.orc_get.argtypes = [C.c_void_p, C.c_char_p, _dp]
        L.orc_set.argtypes = [C.c_void_p, C.c_char_p, _dp]
        L.orc_cholesky.argtypes = [C.c_int, _dp, _dp, C.c_int]
        L.orc_rpy.argtypes = [C.c_int, _dp, _dp, C.c_double, C.c_double, _dp]
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_noise_create.restype = C.c_void_p
        L.orc_noise_create.argtypes = [C.c_ulong]
        L.orc_noise_destroy.argtypes = [C.c_void_p]
        L.orc_noise_u32.restype = C.c_uint
        L.orc_noise_u32.argtypes = [C.c_void_p]
        L.orc_noise_normal.restype = C.c_double
        L.orc_noise_normal.argtypes = [C.c_void_p, C.c_double, C.c_double]
        L.orc_noise_step.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp, C.c_int, _dp, _dp]
        _lib = L
    return _lib


def _pd(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(_dp)


class Oracle:
    """CPU oracle for one fiber, built from a product ``Fiber`` (arrays only)."""

    def __init__(self, fiber, refresh: bool = True):
        L = lib()
        self._keep = []
        y = orc_system()
        for k, v in fiber.sizes.items():
            setattr(y, k, v)
        for k in ("h", "g", "s", "debyell", "debye", "q_l", "k_e", "k_ex", "sigma_DNA_DNA", "sigma_DNA_Core",
                  "sigma_Core_Core", "sigma_Tail_Tail", "sigma_Tail_Linker", "sigma_Tail_Core", "a1", "a2",
                  "time_step", "del_", "s2dt"):
            setattr(y, k, fiber.scalars[k])
        for k, v in fiber.arrays.items():
            if not hasattr(orc_system, k):
                continue
            arr = np.ascontiguousarray(v)
            self._keep.append(arr)
            setattr(y, k, arr.ctypes.data_as(_ip if arr.dtype == np.int32 else _dp))
        st = [np.ascontiguousarray(fiber.state[k], dtype=np.float64) for k in ("r", "a", "b", "c", "r_t", "r_lh")]
        self._keep += st
        self.sizes = dict(fiber.sizes)
        self.n_D = fiber.n_D
        self._h = L.orc_create(C.byref(y), *[a.ctypes.data_as(_dp) for a in st], 1 if refresh else 0)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_destroy(self._h)
            self._h = None

    def forces(self) -> dict:
        n, nt, nl = self.sizes["n"], self.sizes["n_tail"], self.sizes["n_LH"]
        F, T, tF, lF = np.zeros(3 * n), np.zeros(3 * n), np.zeros(3 * nt), np.zeros(3 * nl)
        E = lib().orc_forces(self._h, F.ctypes.data_as(_dp), T.ctypes.data_as(_dp), tF.ctypes.data_as(_dp),
                             lF.ctypes.data_as(_dp))
        return {"force": F, "torque": T, "t_force": tF, "LH_force": lF, "energy": E}

    def tensor(self) -> tuple[np.ndarray, np.ndarray]:
        m = 3 * self.n_D
        D, Lm = np.zeros((m, m)), np.zeros((m, m))
        lib().orc_tensor(self._h, D.ctypes.data_as(_dp), Lm.ctypes.data_as(_dp))
        return D, Lm

    def step(self, rr: np.ndarray, p: np.ndarray) -> float:
        return lib().orc_step(self._h, _pd(rr), _pd(p))

    def em_update(self, F, T, tF, lF, rr, rd) -> None:
        """One move with these forces and noise, then the frame refresh (orc_em_update)."""
        a = [np.ascontiguousarray(x, dtype=np.float64) for x in (F, T, tF, lF, rr, rd)]
        lib().orc_em_update(self._h, *[_pd(x) if x.size else None for x in a])

    def get(self, name: str) -> np.ndarray:
        n = lib().orc_get(self._h, name.encode(), None)
        if n < 0:
            raise KeyError(name)
        out = np.zeros(n)
        lib().orc_get(self._h, name.encode(), out.ctypes.data_as(_dp))
        return out

    def set(self, name: str, v: np.ndarray) -> None:
        arr = np.ascontiguousarray(v, dtype=np.float64)
        if lib().orc_set(self._h, name.encode(), arr.ctypes.data_as(_dp)) < 0:
            raise KeyError(name)


def set_threads(n: int) -> None:
    """Host threads for the RPY assembly, Cholesky and rd of Oracle.step (results unchanged)."""
    lib().orc_set_threads(int(n))


def cholesky(D: np.ndarray, nthreads: int = 1) -> tuple[np.ndarray, int]:
    """Reference Cholesky (func.cpp:806-836) of a row-major matrix."""
    D = np.ascontiguousarray(D, dtype=np.float64)
    Lm = np.zeros_like(D)
    neg = lib().orc_cholesky(D.shape[0], D.ctypes.data_as(_dp), Lm.ctypes.data_as(_dp), nthreads)
    return Lm, neg


def rpy(r_all: np.ndarray, rad: np.ndarray, a1: float, a2: float) -> np.ndarray:
    """RPY tensor assembly (func.cpp:737-804), row-major."""
    nD = rad.size
    D = np.zeros((3 * nD, 3 * nD))
    lib().orc_rpy(nD, _pd(r_all), _pd(rad), a1, a2, D.ctypes.data_as(_dp))
    return D


class OracleNoise:
    def __init__(self, seed: int):
        self._h = lib().orc_noise_create(seed)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_noise_destroy(self._h)

    def u32(self, count: int) -> np.ndarray:
        return np.array([lib().orc_noise_u32(self._h) for _ in range(count)], dtype=np.uint32)

    def step(self, step: int, r_var: np.ndarray, n_D3: int) -> tuple[np.ndarray, np.ndarray]:
        rr, p = np.zeros(r_var.size), np.zeros(n_D3)
        lib().orc_noise_step(self._h, step, r_var.size, _pd(r_var), n_D3, rr.ctypes.data_as(_dp), p.ctypes.data_as(_dp))
        return rr, p


# ---------------------------------------------------------------- reference driver
class Reference:
    """The reference's own CPU physics (func.cpp etc. compiled from its sources, oracle/_ref)."""

    def __init__(self, directory: str, core_file: str, tail_file: str, lh_file: str, seed: int = 1):
        if not os.path.exists(REF_LIB):
            raise FileNotFoundError(REF_LIB)
        L = C.CDLL(REF_LIB)
        L.ref_init.argtypes = [C.c_char_p] * 4 + [C.c_ulong]
        L.ref_get.argtypes = [C.c_char_p, _dp]
        L.ref_set.argtypes = [C.c_char_p, _dp]
        L.ref_step.restype = C.c_double
        L.ref_step.argtypes = [_dp, _dp]
        L.ref_forces.restype = C.c_double
        L.ref_forces.argtypes = [_dp] * 4
        L.ref_tensor.argtypes = [_dp, _dp]
        L.ref_draw_noise.argtypes = [C.c_int, _dp, _dp]
        L.ref_mt_raw.argtypes = [C.c_ulong, C.c_int, C.POINTER(C.c_uint)]
        self.L = L
        self.dir = directory
        cwd = os.getcwd()
        rc = L.ref_init(directory.encode(), core_file.encode(), tail_file.encode(), lh_file.encode(), seed)
        os.chdir(cwd)
        if rc != 0:
            raise RuntimeError(f"ref_init failed: {rc}")
        sz = (C.c_int * 13)()
        L.ref_sizes(sz)
        (self.n, self.n_c, self.n_tail, self.n_LH, self.n_D, self.Nq, self.n_t, self.n_lh_n, self.n_lh_g,
         self.n_lh_c, self.nsteps, self.freq, self.Mg) = list(sz)
        sc = (C.c_double * 26)()
        L.ref_scalars(sc)
        self.scalars = dict(zip(("T", "Cs", "q_l", "debye", "debyell", "k_e", "k_ex", "k_h1", "a1", "a2", "h", "g",
                                 "s", "time_step", "del_", "s2dt", "kbt", "sigma_DNA_DNA", "sigma_DNA_Core",
                                 "sigma_Core_Core", "sigma_Tail_Tail", "sigma_Tail_Linker", "sigma_Tail_Core",
                                 "unbind", "Pbind", "energy"), list(sc)))

    def get(self, name: str) -> np.ndarray:
        n = self.L.ref_get(name.encode(), None)
        if n < 0:
            raise KeyError(name)
        out = np.zeros(n)
        self.L.ref_get(name.encode(), out.ctypes.data_as(_dp))
        return out

    def set(self, name: str, v: np.ndarray) -> None:
        arr = np.ascontiguousarray(v, dtype=np.float64)
        self.L.ref_set(name.encode(), arr.ctypes.data_as(_dp))

    def _in_dir(self, fn, *a):
        cwd = os.getcwd()
        os.chdir(self.dir)  # Linker_Histone_force appends to wf.txt in the working directory
        try:
            return fn(*a)
        finally:
            os.chdir(cwd)

    def noise(self, step: int) -> tuple[np.ndarray, np.ndarray]:
        rr, p = np.zeros(3 * self.n), np.zeros(3 * self.n_D)
        self.L.ref_draw_noise(step, rr.ctypes.data_as(_dp), p.ctypes.data_as(_dp))
        return rr, p

    def step(self, rr: np.ndarray, p: np.ndarray) -> float:
        return self._in_dir(self.L.ref_step, _pd(rr), _pd(p))

    def forces(self) -> dict:
        n, nt, nl = self.n, self.n_tail, self.n_LH
        F, T, tF, lF = np.zeros(3 * n), np.zeros(3 * n), np.zeros(max(3 * nt, 1)), np.zeros(max(3 * nl, 1))
        E = self._in_dir(self.L.ref_forces, F.ctypes.data_as(_dp), T.ctypes.data_as(_dp), tF.ctypes.data_as(_dp),
                         lF.ctypes.data_as(_dp))
        return {"force": F, "torque": T, "t_force": tF[:3 * nt], "LH_force": lF[:3 * nl], "energy": E}

    def tensor(self) -> tuple[np.ndarray, np.ndarray]:
        m = 3 * self.n_D
        D, Lm = np.zeros((m, m)), np.zeros((m, m))
        self.L.ref_tensor(D.ctypes.data_as(_dp), Lm.ctypes.data_as(_dp))
        return D, Lm

    def mt_raw(self, seed: int, count: int) -> np.ndarray:
        out = (C.c_uint * count)()
        self.L.ref_mt_raw(seed, count, out)
        return np.array(list(out), dtype=np.uint32)
