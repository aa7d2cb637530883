"""ctypes binding of include/bd_capi.h (libbdgb300.so).

``Fiber`` holds one fiber's model (topology, parameters, per-bead constants)
and initial state as numpy arrays in the reference's layouts; it is built
from the reference input files through the library's own readers
(``Fiber.load``) or directly from arrays (``Fiber.from_arrays``).
``Context`` owns the device state of one fiber and runs steps.  There is no
CPU fallback: a missing library raises at import of the first call.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libbdgb300.so")

BD_OK, BD_ERR_ARG, BD_ERR_IO, BD_ERR_CUDA, BD_ERR_NOMEM, BD_ERR_NONFINITE, BD_ERR_NOT_SPD, BD_ERR_STATE = range(8)
PREC_FP64, PREC_MIXED = 0, 1
NOISE_CHOLESKY, NOISE_KRYLOV = 0, 1
LOG_LIBM, LOG_CR = 0, 1

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class BDError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class bd_model(C.Structure):
    _fields_ = [(k, C.c_int) for k in ("n", "n_c", "Nq", "n_t", "n_tail", "n_lh_n", "n_lh_g", "n_lh_c", "n_LH")] + [
        (k, C.c_double)
        for k in ("h", "g", "s", "debyell", "debye", "q_l", "k_e", "k_ex", "k_h1", "sigma_DNA_DNA", "sigma_DNA_Core",
                  "sigma_Core_Core", "sigma_Tail_Tail", "sigma_Tail_Linker", "sigma_Tail_Core", "a1", "a2",
                  "time_step", "del_", "s2dt")
    ] + [
        ("type", _ip), ("rad", _dp), ("phi_o", _dp), ("r_var", _dp), ("core_pos", _dp), ("core_q", _dp),
        ("tail_pos", _dp), ("tail_fix", _ip), ("nc_t_flag", _ip), ("h_t", _dp), ("g_t", _dp), ("lo_t", _dp),
        ("beta_o_t", _dp), ("t_q", _dp), ("t_rad", _dp), ("t_grp", _ip), ("t_fix", _ip), ("LH_g_pos", _dp),
        ("LH_conn", _ip), ("nc_lh_flag", _ip), ("LH_q", _dp), ("LH_vdw_hh", _dp), ("LH_vdw_hc", _dp),
        ("LH_vdw_hl", _dp), ("LH_vdw_ht", _dp), ("LH_kstr", _dp), ("LH_kben", _dp), ("LH_streq", _dp),
        ("LH_betaeq", _dp), ("lh_rad", _dp),
    ]


class bd_state(C.Structure):
    _fields_ = [("r", _dp), ("a", _dp), ("b", _dp), ("c", _dp), ("r_t", _dp), ("r_lh", _dp), ("refresh_frames", C.c_int),
                ("alpha", _dp), ("beta", _dp), ("gamma", _dp), ("length", _dp), ("a_dna", _dp), ("b_dna", _dp),
                ("c_dna", _dp), ("alpha_p", _dp), ("beta_p", _dp), ("gamma_p", _dp)]


RESTART_ARRAYS = ("r", "a", "b", "c", "alpha", "beta", "gamma", "length", "a_dna", "b_dna", "c_dna", "alpha_p",
                  "beta_p", "gamma_p", "r_t", "r_lh")


class bd_restart(C.Structure):
    _fields_ = [("step", C.c_long), ("n", C.c_int), ("n_c", C.c_int), ("n_tail", C.c_int), ("n_LH", C.c_int)] + \
               [(k, _dp) for k in RESTART_ARRAYS] + [("nc_lh_flag", _ip)]


def _restart_len(k: str, n: int, nc: int, nt: int, nl: int) -> int:
    return {"r": 3 * n, "a": 3 * n, "b": 3 * n, "c": 3 * n, "alpha": n, "beta": n, "gamma": n, "length": n,
            "a_dna": 3 * nc, "b_dna": 3 * nc, "c_dna": 3 * nc, "alpha_p": nc, "beta_p": nc, "gamma_p": nc,
            "r_t": 3 * nt, "r_lh": 3 * nl}[k]


def _restart_struct(step: int, n: int, nc: int, nt: int, nl: int, arrays: dict, flags: np.ndarray) -> bd_restart:
    rs = bd_restart(step=step, n=n, n_c=nc, n_tail=nt, n_LH=nl)
    for k in RESTART_ARRAYS:
        setattr(rs, k, _pd(arrays[k]) if arrays[k].size else None)
    rs.nc_lh_flag = _pi(flags)
    return rs


def restart_write(path: str, step: int, arrays: dict, nc_lh_flag: np.ndarray, noise: "Noise | None" = None) -> None:
    """Binary restart (bd_restart_write): arrays as RESTART_ARRAYS (state, frames, angles)."""
    L = load_library()
    n, nc = arrays["alpha"].size, arrays["alpha_p"].size
    nt, nl = arrays["r_t"].size // 3, arrays["r_lh"].size // 3
    arrays = {k: np.ascontiguousarray(arrays[k], dtype=np.float64) for k in RESTART_ARRAYS}
    flags = np.ascontiguousarray(nc_lh_flag, dtype=np.int32)
    rs = _restart_struct(step, n, nc, nt, nl, arrays, flags)
    _check(L.bd_restart_write(path.encode(), C.byref(rs), noise._h if noise is not None else None))


def restart_read(path: str, noise: "Noise | None" = None) -> tuple:
    """(step, arrays, nc_lh_flag, has_noise) of a restart; noise (if given) takes its generator state."""
    L = load_library()
    head, has = bd_restart(), C.c_int()
    _check(L.bd_restart_info(path.encode(), C.byref(head), C.byref(has)))
    n, nc, nt, nl = head.n, head.n_c, head.n_tail, head.n_LH
    arrays = {k: np.zeros(_restart_len(k, n, nc, nt, nl)) for k in RESTART_ARRAYS}
    flags = np.zeros(nc, dtype=np.int32)
    rs = _restart_struct(0, n, nc, nt, nl, arrays, flags)
    _check(L.bd_restart_read(path.encode(), C.byref(rs), noise._h if noise is not None else None))
    return int(rs.step), arrays, flags, bool(has.value)


class bd_options(C.Structure):
    _fields_ = [("precision", C.c_int), ("frequency_RP", C.c_int), ("use_graph", C.c_int), ("device", C.c_int),
                ("stream", C.c_void_p)]


_lib = None


def load_library(path: str | None = None) -> C.CDLL:
    """Loads libbdgb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise FileNotFoundError(f"{p} is missing: run brownian_dynamics_cuda_gb300.build.build_lib() first")
    L = C.CDLL(p)
    L.bd_last_error.restype = C.c_char_p
    L.bd_version.restype = C.c_char_p
    L.bd_system_load.argtypes = [C.c_char_p] * 6 + [C.POINTER(C.c_void_p)]
    L.bd_system_model.argtypes = [C.c_void_p, C.POINTER(bd_model)]
    L.bd_system_state.argtypes = [C.c_void_p, C.POINTER(bd_state)]
    L.bd_system_setup.argtypes = [C.c_void_p, _dp]
    L.bd_system_free.argtypes = [C.c_void_p]
    L.bd_system_free.restype = None
    L.bd_write_xyz.argtypes = [C.POINTER(bd_model)] + [_dp] * 6 + [C.c_char_p]
    L.bd_noise_create.argtypes = [C.c_ulong, C.POINTER(C.c_void_p)]
    L.bd_noise_step.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp, C.c_int, _dp, _dp]
    L.bd_noise_u32.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_uint32)]
    L.bd_noise_free.argtypes = [C.c_void_p]
    L.bd_noise_free.restype = None
    L.bd_noise_set_log.argtypes = [C.c_void_p, C.c_int]
    L.bd_create.argtypes = [C.POINTER(bd_model), C.POINTER(bd_state), C.POINTER(bd_options), C.POINTER(C.c_void_p)]
    L.bd_destroy.argtypes = [C.c_void_p]
    L.bd_sizes.argtypes = [C.c_void_p, _ip]
    L.bd_step.argtypes = [C.c_void_p, _dp, _dp, _dp]
    L.bd_step_device.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.bd_batch_create.argtypes = [C.c_int, C.POINTER(bd_model), C.POINTER(bd_state), C.POINTER(bd_options),
                                  C.POINTER(C.c_void_p)]
    L.bd_batch_destroy.argtypes = [C.c_void_p]
    L.bd_batch_size.argtypes = [C.c_void_p, _ip]
    L.bd_batch_context.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_void_p)]
    L.bd_batch_step.argtypes = [C.c_void_p, C.POINTER(_dp), C.POINTER(_dp), _dp]
    L.bd_batch_step_device.argtypes = [C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]
    L.bd_batch_run.argtypes = [C.c_void_p, C.c_int, C.c_ulong, _dp]
    L.bd_batch_run_device.argtypes = [C.c_void_p, C.c_int, C.c_ulong, _dp]
    L.bd_batch_phase_times.argtypes = [C.c_void_p, C.POINTER(C.c_float)]
    L.bd_batch_launch_count.argtypes = [C.c_void_p, C.POINTER(C.c_int)]
    L.bd_set_mixed_passes.argtypes = [C.c_void_p, C.c_int]
    L.bd_set_noise_mode.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_int]
    L.bd_krylov_stats.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double)]
    L.bd_batch_set_mixed_passes.argtypes = [C.c_void_p, C.c_int]
    L.bd_step_reference.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, _dp, _dp, _dp] + [_dp] * 6
    L.bd_forces.argtypes = [C.c_void_p] + [_dp] * 5
    L.bd_diffusion_tensor.argtypes = [C.c_void_p, _dp]
    L.bd_cholesky.argtypes = [C.c_void_p, _dp]
    L.bd_noise_displacement.argtypes = [C.c_void_p, _dp, _dp]
    L.bd_get_state.argtypes = [C.c_void_p, C.c_char_p, _dp, _ip]
    L.bd_set_state.argtypes = [C.c_void_p, C.c_char_p, _dp]
    L.bd_dev_rpy.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_void_p, C.c_int]
    L.bd_dev_potrf.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p]
    L.bd_noise_displacement_noalloc.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_double, C.c_void_p,
                                                C.c_void_p]
    L.bd_phase_times.argtypes = [C.c_void_p, C.POINTER(C.c_float)]
    L.bd_launch_count.argtypes = [C.c_void_p, _ip]
    L.bd_kernel_time.argtypes = [C.c_void_p, C.POINTER(C.c_float), _ip, _dp]
    L.bd_kernel_times.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.c_int, _ip]
    L.bd_kernel_bytes.argtypes = [C.c_void_p, _dp]
    L.bd_negative_pivots.argtypes = [C.c_void_p, _ip]
    L.bd_dev_noise_create.argtypes = [C.c_ulong, C.POINTER(C.c_void_p)]
    L.bd_dev_noise_step.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                    C.c_void_p]
    L.bd_dev_noise_free.argtypes = [C.c_void_p]
    L.bd_set_lh_flags.argtypes = [C.c_void_p, _ip, _dp, _dp]
    L.bd_em_update.argtypes = [C.c_void_p] + [_dp] * 6
    L.bd_noise_get_state.argtypes = [C.c_void_p, C.POINTER(C.c_uint32), _ip, _ip, _dp]
    L.bd_noise_set_state.argtypes = [C.c_void_p, C.POINTER(C.c_uint32), C.c_int, C.c_int, C.c_double]
    L.bd_restart_write.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p]
    L.bd_restart_info.argtypes = [C.c_char_p, C.c_void_p, _ip]
    L.bd_restart_read.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p]
    L.bd_restart_from_context.argtypes = [C.c_void_p, C.c_void_p]
    L.bd_adjoint.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, _dp]
    L.bd_rollout_loss.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp, _dp, _dp]
    L.bd_set_moduli.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_double]
    L.bd_adjoint_launches.argtypes = [C.c_void_p, C.POINTER(C.c_long)]
    _lib = L
    return L


def _check(rc: int) -> None:
    if rc != BD_OK:
        raise BDError(rc, load_library().bd_last_error().decode())


def _pd(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def _pi(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(_ip)


SCALARS = ("h", "g", "s", "debyell", "debye", "q_l", "k_e", "k_ex", "k_h1", "sigma_DNA_DNA", "sigma_DNA_Core",
           "sigma_Core_Core", "sigma_Tail_Tail", "sigma_Tail_Linker", "sigma_Tail_Core", "a1", "a2", "time_step",
           "del_", "s2dt")
SIZES = ("n", "n_c", "Nq", "n_t", "n_tail", "n_lh_n", "n_lh_g", "n_lh_c", "n_LH")
INT_ARRAYS = ("type", "tail_fix", "nc_t_flag", "t_grp", "t_fix", "LH_conn", "nc_lh_flag")
DBL_ARRAYS = ("rad", "phi_o", "r_var", "core_pos", "core_q", "tail_pos", "h_t", "g_t", "lo_t", "beta_o_t", "t_q",
              "t_rad", "LH_g_pos", "LH_q", "LH_vdw_hh", "LH_vdw_hc", "LH_vdw_hl", "LH_vdw_ht", "LH_kstr", "LH_kben",
              "LH_streq", "LH_betaeq", "lh_rad")
STATE = ("r", "a", "b", "c", "r_t", "r_lh")


def _array_len(name: str, sz: dict) -> int:
    n, nc, Nq, nt, ntail, nL = sz["n"], sz["n_c"], sz["Nq"], sz["n_t"], sz["n_tail"], sz["n_LH"]
    npar = sz["n_lh_n"] + sz["n_lh_g"] + sz["n_lh_c"]
    return {
        "type": n, "rad": n, "phi_o": n, "r_var": 3 * n, "core_pos": 3 * Nq, "core_q": Nq, "tail_pos": 3 * nt,
        "tail_fix": nt, "nc_t_flag": nc, "h_t": ntail, "g_t": ntail, "lo_t": ntail, "beta_o_t": ntail, "t_q": ntail,
        "t_rad": ntail, "t_grp": ntail, "t_fix": ntail, "LH_g_pos": 3 * sz["n_lh_g"], "LH_conn": npar,
        "nc_lh_flag": nc, "LH_q": npar, "LH_vdw_hh": npar, "LH_vdw_hc": npar, "LH_vdw_hl": npar, "LH_vdw_ht": npar,
        "LH_kstr": npar, "LH_kben": npar, "LH_streq": npar, "LH_betaeq": npar, "lh_rad": nL,
        "r": 3 * n, "a": 3 * n, "b": 3 * n, "c": 3 * n, "r_t": 3 * ntail, "r_lh": 3 * nL,
    }[name]


@dataclass
class Fiber:
    """One fiber: sizes, scalar parameters, per-bead arrays and state (numpy, reference layouts)."""
    sizes: dict
    scalars: dict
    arrays: dict
    state: dict
    setup: np.ndarray = field(default_factory=lambda: np.zeros(15))

    @property
    def n_D(self) -> int:
        return self.sizes["n"] + self.sizes["n_tail"] + self.sizes["n_LH"]

    @property
    def m(self) -> int:
        return 3 * self.n_D

    @staticmethod
    def load(directory: str, core_file: str, tail_file: str, lh_file: str, data_file: str = "data_mod",
             lh_flags_file: str = "LH.in") -> "Fiber":
        """Reads the reference input files with the library's readers (readfile.cpp formats)."""
        L = load_library()
        h = C.c_void_p()
        _check(L.bd_system_load(directory.encode(), data_file.encode(), core_file.encode(), tail_file.encode(),
                                lh_file.encode(), lh_flags_file.encode(), C.byref(h)))
        try:
            m = bd_model()
            _check(L.bd_system_model(h, C.byref(m)))
            s = bd_state()
            _check(L.bd_system_state(h, C.byref(s)))
            setup = np.zeros(15)
            _check(L.bd_system_setup(h, _pd(setup)))
            sizes = {k: int(getattr(m, k)) for k in SIZES}
            scalars = {k: float(getattr(m, k)) for k in SCALARS}
            arrays = {}
            for k in INT_ARRAYS:
                cnt = _array_len(k, sizes)
                p = getattr(m, k)
                arrays[k] = np.ctypeslib.as_array(p, shape=(cnt,)).astype(np.int32).copy() if cnt else np.zeros(0, np.int32)
            for k in DBL_ARRAYS:
                cnt = _array_len(k, sizes)
                p = getattr(m, k)
                arrays[k] = np.ctypeslib.as_array(p, shape=(cnt,)).copy() if cnt else np.zeros(0)
            state = {}
            for k in STATE:
                cnt = _array_len(k, sizes)
                p = getattr(s, k)
                state[k] = np.ctypeslib.as_array(p, shape=(cnt,)).copy() if cnt else np.zeros(0)
        finally:
            L.bd_system_free(h)
        return Fiber(sizes, scalars, arrays, state, setup)

    @staticmethod
    def from_arrays(d: dict) -> "Fiber":
        """Inverse of ``to_arrays`` (e.g. a golden .npz)."""
        sizes = {k: int(d["size_" + k]) for k in SIZES}
        scalars = {k: float(d["scalar_" + k]) for k in SCALARS}
        arrays = {k: np.ascontiguousarray(d["arr_" + k], dtype=np.int32 if k in INT_ARRAYS else np.float64)
                  for k in INT_ARRAYS + DBL_ARRAYS}
        state = {k: np.ascontiguousarray(d["state_" + k], dtype=np.float64) for k in STATE}
        setup = np.asarray(d["setup"], dtype=np.float64) if "setup" in d else np.zeros(15)
        return Fiber(sizes, scalars, arrays, state, setup)

    def to_arrays(self) -> dict:
        out = {"size_" + k: v for k, v in self.sizes.items()}
        out.update({"scalar_" + k: v for k, v in self.scalars.items()})
        out.update({"arr_" + k: v for k, v in self.arrays.items()})
        out.update({"state_" + k: v for k, v in self.state.items()})
        out["setup"] = self.setup
        return out

    def model_struct(self) -> bd_model:
        m = bd_model()
        for k, v in self.sizes.items():
            setattr(m, k, v)
        for k, v in self.scalars.items():
            setattr(m, k, v)
        for k in INT_ARRAYS:
            setattr(m, k, _pi(self.arrays[k]))
        for k in DBL_ARRAYS:
            setattr(m, k, _pd(self.arrays[k]))
        return m

    def state_struct(self, refresh: bool = True, angles: dict | None = None) -> bd_state:
        s = bd_state()
        for k in STATE:
            setattr(s, k, _pd(self.state[k]))
        s.refresh_frames = 1 if refresh else 0
        if angles:
            for k, v in angles.items():
                setattr(s, k, _pd(v))
        return s

    def write_xyz(self, path: str, state: dict | None = None) -> None:
        st = state or self.state
        m = self.model_struct()
        _check(load_library().bd_write_xyz(C.byref(m), *[_pd(st[k]) for k in STATE], path.encode()))


class Noise:
    """Reference-order MT19937 + polar Box-Muller noise (host)."""

    def __init__(self, seed: int, log_mode: int = LOG_LIBM):
        self._L = load_library()
        self._h = C.c_void_p()
        _check(self._L.bd_noise_create(seed, C.byref(self._h)))
        if log_mode != LOG_LIBM:
            self.set_log(log_mode)

    def set_log(self, mode: int) -> None:
        """bd_noise_set_log: LOG_LIBM (the C library's log, the reference) or
        LOG_CR (correctly rounded: the device stream's, bit for bit)."""
        _check(self._L.bd_noise_set_log(self._h, mode))

    def step(self, step: int, r_var: np.ndarray, n_D3: int) -> tuple[np.ndarray, np.ndarray]:
        rr = np.zeros(r_var.size)
        p = np.zeros(n_D3)
        _check(self._L.bd_noise_step(self._h, step, r_var.size, _pd(r_var), n_D3, _pd(rr), _pd(p)))
        return rr, p

    def u32(self, count: int) -> np.ndarray:
        out = np.zeros(count, dtype=np.uint32)
        _check(self._L.bd_noise_u32(self._h, count, out.ctypes.data_as(C.POINTER(C.c_uint32))))
        return out

    def get_state(self) -> tuple:
        """(words[624], index, have_cached, cached) of the generator."""
        w = np.zeros(624, dtype=np.uint32)
        idx, have, cached = C.c_int(), C.c_int(), C.c_double()
        _check(self._L.bd_noise_get_state(self._h, w.ctypes.data_as(C.POINTER(C.c_uint32)), C.byref(idx),
                                          C.byref(have), C.byref(cached)))
        return w, idx.value, have.value, cached.value

    def set_state(self, state: tuple) -> None:
        w, idx, have, cached = state
        w = np.ascontiguousarray(w, dtype=np.uint32)
        _check(self._L.bd_noise_set_state(self._h, w.ctypes.data_as(C.POINTER(C.c_uint32)), idx, have, cached))

    def __del__(self):
        if getattr(self, "_h", None):
            self._L.bd_noise_free(self._h)
            self._h = None


class DevNoise:
    """The reference's MT19937 noise stream generated on the device (bd_dev_noise_*)."""

    def __init__(self, seed: int):
        self._L = load_library()
        self._h = C.c_void_p()
        _check(self._L.bd_dev_noise_create(seed, C.byref(self._h)))

    def step(self, step: int, d_r_var: int, n3: int, n_D3: int, d_rr: int, d_p: int, stream: int = 0) -> None:
        """Step `step`'s draws into device buffers (addresses)."""
        _check(self._L.bd_dev_noise_step(self._h, step, n3, C.c_void_p(d_r_var), n_D3, C.c_void_p(d_rr),
                                         C.c_void_p(d_p), C.c_void_p(stream) if stream else None))

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._L.bd_dev_noise_free(self._h)
            self._h = None

    def __del__(self):
        self.close()


class Context:
    """Device state of one fiber (bd_create / bd_step / bd_destroy)."""

    def __init__(self, fiber: Fiber, precision: int = PREC_FP64, use_graph: bool = False, frequency_RP: int = 1,
                 refresh: bool = True, angles: dict | None = None, device: int = 0, stream: int = 0):
        self._L = load_library()
        self.fiber = fiber
        m = fiber.model_struct()
        s = fiber.state_struct(refresh, angles)
        o = bd_options(precision=precision, frequency_RP=frequency_RP, use_graph=int(use_graph), device=device,
                       stream=C.c_void_p(stream) if stream else None)
        self._h = C.c_void_p()
        _check(self._L.bd_create(C.byref(m), C.byref(s), C.byref(o), C.byref(self._h)))
        sz = (C.c_int * 8)()
        _check(self._L.bd_sizes(self._h, sz))
        self.n, self.n_c, self.n_tail, self.n_LH, self.n_D, self.m, self.lda, self.precision = list(sz)

    @classmethod
    def _view(cls, handle: C.c_void_p, fiber: Fiber) -> "Context":
        """A non-owning Context over a handle another object owns (a batch replica)."""
        self = cls.__new__(cls)
        self._L = load_library()
        self.fiber = fiber
        self._h = handle
        self._owned = False
        sz = (C.c_int * 8)()
        _check(self._L.bd_sizes(self._h, sz))
        self.n, self.n_c, self.n_tail, self.n_LH, self.n_D, self.m, self.lda, self.precision = list(sz)
        return self

    def close(self) -> None:
        if getattr(self, "_h", None):
            if getattr(self, "_owned", True):
                self._L.bd_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def step(self, rr: np.ndarray, p: np.ndarray) -> float:
        e = C.c_double()
        _check(self._L.bd_step(self._h, _pd(rr), _pd(p), C.byref(e)))
        return e.value

    def step_device(self, d_rr: int, d_p: int, d_energy: int = 0) -> None:
        _check(self._L.bd_step_device(self._h, C.c_void_p(d_rr), C.c_void_p(d_p), C.c_void_p(d_energy or None)))

    def step_reference(self, step: int, number_of_steps: int, freq: int, rr: np.ndarray, p: np.ndarray,
                       out: dict) -> float:
        """main_cuda-form step: host noise in, host state copies out (bd_step_reference)."""
        e = C.c_double()
        _check(self._L.bd_step_reference(self._h, step, number_of_steps, freq, _pd(rr), _pd(p), C.byref(e),
                                         *[_pd(out[k]) for k in ("r", "a", "b", "c", "r_t", "r_lh")]))
        return e.value

    def forces(self) -> dict:
        n, nt, nl = self.n, self.n_tail, self.n_LH
        F, T, tF, lF, E = np.zeros(3 * n), np.zeros(3 * n), np.zeros(3 * nt), np.zeros(3 * nl), np.zeros(1)
        _check(self._L.bd_forces(self._h, _pd(F), _pd(T), _pd(tF), _pd(lF), _pd(E)))
        return {"force": F, "torque": T, "t_force": tF, "LH_force": lF, "energy": float(E[0])}

    def diffusion_tensor(self) -> np.ndarray:
        D = np.zeros((self.m, self.m))
        _check(self._L.bd_diffusion_tensor(self._h, _pd(D)))
        return D

    def cholesky(self) -> np.ndarray:
        Lm = np.zeros((self.m, self.m))
        _check(self._L.bd_cholesky(self._h, _pd(Lm)))
        return Lm

    def noise_displacement(self, p: np.ndarray) -> np.ndarray:
        rd = np.zeros(self.m)
        _check(self._L.bd_noise_displacement(self._h, _pd(p), _pd(rd)))
        return rd

    def em_update(self, F: np.ndarray, T: np.ndarray, tF: np.ndarray, lF: np.ndarray, rr: np.ndarray,
                  rd: np.ndarray) -> None:
        """One Ermak-McCammon move with these forces and noise (bd_em_update)."""
        a = [np.ascontiguousarray(x, dtype=np.float64) for x in (F, T, tF, lF, rr, rd)]
        _check(self._L.bd_em_update(self._h, *[_pd(x) if x.size else None for x in a]))

    def get(self, name: str) -> np.ndarray:
        cnt = C.c_int()
        _check(self._L.bd_get_state(self._h, name.encode(), None, C.byref(cnt)))
        out = np.zeros(cnt.value)
        _check(self._L.bd_get_state(self._h, name.encode(), _pd(out), C.byref(cnt)))
        return out

    def set(self, name: str, value: np.ndarray) -> None:
        _check(self._L.bd_set_state(self._h, name.encode(), _pd(np.ascontiguousarray(value, dtype=np.float64))))

    def phase_times(self) -> np.ndarray:
        out = (C.c_float * 9)()
        _check(self._L.bd_phase_times(self._h, out))
        return np.array(list(out))

    def kernel_time(self) -> tuple[float, int, float]:
        """(total ms, launches, tensor flop) of the tensor-core update in the last timed step."""
        ms, n, fl = C.c_float(), C.c_int(), C.c_double()
        _check(self._L.bd_kernel_time(self._h, C.byref(ms), C.byref(n), C.byref(fl)))
        return ms.value, n.value, fl.value

    def kernel_bytes(self) -> float:
        """Algorithmic HBM bytes of the tensor-core update launches of the last timed step."""
        b = C.c_double()
        _check(self._L.bd_kernel_bytes(self._h, C.byref(b)))
        return b.value

    def kernel_times(self) -> np.ndarray:
        """Per-launch ms of the tensor-core update launches of the last timed step."""
        out = (C.c_float * 4096)()
        n = C.c_int()
        _check(self._L.bd_kernel_times(self._h, out, 4096, C.byref(n)))
        return np.array(list(out)[:min(n.value, 4096)])

    def launch_count(self) -> int:
        v = C.c_int()
        _check(self._L.bd_launch_count(self._h, C.byref(v)))
        return v.value

    def set_noise_mode(self, mode: int, tol: float = 1e-6, kmax: int = 64) -> None:
        """bd_set_noise_mode: NOISE_CHOLESKY (the reference's L p) or NOISE_KRYLOV
        (D^{1/2} p by Lanczos, to relative change tol, at most kmax iterations)."""
        _check(self._L.bd_set_noise_mode(self._h, int(mode), float(tol), int(kmax)))

    def krylov_stats(self) -> tuple[int, float]:
        """Iterations and last relative change of the most recent Krylov run."""
        it, ch = C.c_int(), C.c_double()
        _check(self._L.bd_krylov_stats(self._h, C.byref(it), C.byref(ch)))
        return it.value, ch.value

    def set_mixed_passes(self, passes: int) -> None:
        """bd_set_mixed_passes: at most `passes` panels per trailing pass of the mixed
        factorisation (3 fastest, 1 most accurate)."""
        _check(self._L.bd_set_mixed_passes(self._h, int(passes)))

    def negative_pivots(self) -> int:
        v = C.c_int()
        _check(self._L.bd_negative_pivots(self._h, C.byref(v)))
        return v.value

    def restart_state(self) -> dict:
        """The context's state, frames and angles (bd_restart_from_context), as RESTART_ARRAYS."""
        nc = self.n_c
        arrays = {k: np.zeros(_restart_len(k, self.n, nc, self.n_tail, self.n_LH)) for k in RESTART_ARRAYS}
        rs = _restart_struct(0, self.n, nc, self.n_tail, self.n_LH, arrays, np.zeros(nc, dtype=np.int32))
        _check(self._L.bd_restart_from_context(self._h, C.byref(rs)))
        return arrays

    def set_lh_flags(self, nc_lh_flag: np.ndarray, r_lh: np.ndarray, lh_rad: np.ndarray | None = None) -> None:
        """New linker-histone binding (bd_set_lh_flags); the sizes are re-read."""
        f = np.ascontiguousarray(nc_lh_flag, dtype=np.int32)
        r = np.ascontiguousarray(r_lh, dtype=np.float64)
        rad = None if lh_rad is None else np.ascontiguousarray(lh_rad, dtype=np.float64)
        _check(self._L.bd_set_lh_flags(self._h, _pi(f), _pd(r), _pd(rad)))
        sz = (C.c_int * 8)()
        _check(self._L.bd_sizes(self._h, sz))
        self.n, self.n_c, self.n_tail, self.n_LH, self.n_D, self.m, self.lda, self.precision = list(sz)

    def adjoint(self, rr: np.ndarray, p: np.ndarray, window: int, checkpoint_every: int = 20) -> tuple:
        """(loss, d loss / d (h, g, s, Debye length)) of the rollout driven by the
        noise rows rr [steps, 3n], p [steps, 3 n_D] (bd_adjoint)."""
        rr = np.ascontiguousarray(rr, dtype=np.float64)
        p = np.ascontiguousarray(p, dtype=np.float64)
        loss, g = C.c_double(), np.zeros(4)
        _check(self._L.bd_adjoint(self._h, rr.shape[0], checkpoint_every, window, _pd(rr), _pd(p), C.byref(loss),
                                  _pd(g)))
        return loss.value, g

    def rollout_loss(self, rr: np.ndarray, p: np.ndarray, window: int) -> float:
        rr = np.ascontiguousarray(rr, dtype=np.float64)
        p = np.ascontiguousarray(p, dtype=np.float64)
        loss = C.c_double()
        _check(self._L.bd_rollout_loss(self._h, rr.shape[0], window, _pd(rr), _pd(p), C.byref(loss)))
        return loss.value

    def set_moduli(self, h: float, g: float, s: float, debye_length: float) -> None:
        _check(self._L.bd_set_moduli(self._h, h, g, s, debye_length))

    def adjoint_launches(self) -> int:
        v = C.c_long()
        _check(self._L.bd_adjoint_launches(self._h, C.byref(v)))
        return v.value


class Batch:
    """Independent fibers (replicas) advanced together (bd_batch_*): one
    stream, one CUDA graph per batch step running every replica's step."""

    def __init__(self, fibers: list, precision: int = PREC_MIXED, use_graph: bool = True, device: int = 0,
                 stream: int = 0):
        self._L = load_library()
        self.fibers = list(fibers)
        R = len(self.fibers)
        models = (bd_model * R)(*[f.model_struct() for f in self.fibers])
        states = (bd_state * R)(*[f.state_struct() for f in self.fibers])
        o = bd_options(precision=precision, frequency_RP=1, use_graph=int(use_graph), device=device,
                       stream=C.c_void_p(stream) if stream else None)
        self._h = C.c_void_p()
        _check(self._L.bd_batch_create(R, models, states, C.byref(o), C.byref(self._h)))
        self.contexts = []
        for i in range(R):
            h = C.c_void_p()
            _check(self._L.bd_batch_context(self._h, i, C.byref(h)))
            self.contexts.append(Context._view(h, self.fibers[i]))

    def __len__(self) -> int:
        return len(self.fibers)

    def step(self, rrs: list, ps: list) -> np.ndarray:
        R = len(self)
        rrs = [np.ascontiguousarray(x, dtype=np.float64) for x in rrs]  # kept alive for the call
        ps = [np.ascontiguousarray(x, dtype=np.float64) for x in ps]
        rr = (_dp * R)(*[_pd(x) for x in rrs])
        pp = (_dp * R)(*[_pd(x) for x in ps])
        e = np.zeros(R)
        _check(self._L.bd_batch_step(self._h, rr, pp, _pd(e)))
        return e

    def step_device(self, d_rr: list, d_p: list) -> None:
        R = len(self)
        a = (C.c_void_p * R)(*[C.c_void_p(x) for x in d_rr])
        b = (C.c_void_p * R)(*[C.c_void_p(x) for x in d_p])
        _check(self._L.bd_batch_step_device(self._h, a, b))

    def phase_times(self) -> np.ndarray:
        """bd_batch_phase_times: [positions + tensors, factorisation, forces + moves] ms of
        the last eager step; the first call switches timing on."""
        out = (C.c_float * 3)()
        _check(self._L.bd_batch_phase_times(self._h, out))
        return np.array(list(out))

    def set_mixed_passes(self, passes: int) -> None:
        """bd_batch_set_mixed_passes: at most `passes` panels per trailing pass (1 = most accurate)."""
        _check(self._L.bd_batch_set_mixed_passes(self._h, int(passes)))

    def launch_count(self) -> int:
        """Kernel launches of the last batch step enqueued (bd_batch_launch_count)."""
        n = C.c_int()
        _check(self._L.bd_batch_launch_count(self._h, C.byref(n)))
        return n.value

    def run(self, nsteps: int, seed_base: int) -> np.ndarray:
        e = np.zeros(len(self))
        _check(self._L.bd_batch_run(self._h, nsteps, seed_base, _pd(e)))
        return e

    def run_device(self, nsteps: int, seed_base: int) -> np.ndarray:
        """bd_batch_run_device: the same run with the noise generated on the
        device (the correctly rounded log), no host synchronisation between
        steps."""
        e = np.zeros(len(self))
        _check(self._L.bd_batch_run_device(self._h, nsteps, seed_base, _pd(e)))
        return e

    def close(self) -> None:
        if getattr(self, "_h", None):
            for c in self.contexts:
                c._h = None
            self._L.bd_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()
