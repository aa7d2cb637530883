"""The adjoint kernels' force-field terms on the CPU.

The terms (brownian_dynamics_cuda_gb300/csrc/adj_terms.cuh) are compiled for
the host into a test harness (tests/adj_terms_check.cpp):
  * summed the way the adjoint kernels split them, they must give the CPU
    oracle's forces and torques (a restatement check; different summation
    order, so 1e-10 relative);
  * each term's dual-number vector-Jacobian product must match central
    finite differences of the same term (derivative check).
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden_names, load_golden, rel_err

CSRC = os.path.join(ROOT, "brownian_dynamics_cuda_gb300", "csrc")
SRC = os.path.join(ROOT, "tests", "adj_terms_check.cpp")


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("adjh") / "libadjh.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-I" + CSRC, SRC, "-o", so], check=True)
    L = C.CDLL(so)
    L.adjh_vjp_check.argtypes = [C.c_int, C.c_uint, C.POINTER(C.c_double)]
    return L


def test_term_vjps_match_finite_differences(harness):
    out = (C.c_double * 20)()
    harness.adjh_vjp_check(60, 7, out)
    names = ["bond DNA", "bond core", "bond DNA->core", "frame refresh", "rotation", "RPY block", "DNA pair",
             "clamped pair", "tail bend", "anchor"]
    errs = dict(zip(names, list(out)[:10]))
    used = dict(zip(names, list(out)[10:]))
    assert all(v >= 20 for v in used.values()), used
    assert all(v < 1e-6 for v in errs.values()), errs


def _fibers():
    import tempfile
    from brownian_dynamics_cuda_gb300.fiber_gen import FiberSpec, make_fiber
    out = []
    for name in golden_names():
        fib, _ = load_golden(name)
        if fib.sizes["n_LH"] == 0:
            out.append((name, fib))
    out.append(("syn_4nuc_30bp", make_fiber(FiberSpec(4, [30] * 4, lh=False, seed=3), tempfile.mkdtemp())))
    # uneven linkers (2 to 7 beads) at low salt: longer Debye length, more
    # pairs inside the cut-offs, DNA-DNA pairs within the 8 nm LJ range
    out.append(("syn_5nuc_uneven_50mM", make_fiber(FiberSpec(5, [20, 60, 26, 44, 30], lh=False, cs=0.050, seed=7),
                                                   tempfile.mkdtemp())))
    return out


@pytest.mark.parametrize("name,fib", _fibers(), ids=lambda v: v if isinstance(v, str) else "")
def test_terms_sum_to_oracle_forces(harness, name, fib):
    from oracle.pyoracle import Oracle
    o = Oracle(fib)
    ref = o.forces()
    sz, ar, sc = fib.sizes, fib.arrays, fib.scalars
    x = np.concatenate([o.get(k) for k in ("r", "a", "b", "c", "r_t")])
    ints = [np.ascontiguousarray(ar[k], dtype=np.int32) for k in ("type", "tail_fix", "nc_t_flag", "t_grp")]
    dbls = [np.ascontiguousarray(ar[k], dtype=np.float64) for k in
            ("phi_o", "core_pos", "core_q", "tail_pos", "h_t", "g_t", "lo_t", "beta_o_t", "t_q")]
    par = np.array([sc[k] for k in ("h", "g", "s", "debyell", "debye", "q_l", "k_e", "k_ex", "sigma_DNA_DNA",
                                    "sigma_DNA_Core", "sigma_Core_Core", "sigma_Tail_Linker")])
    isz = np.array([sz["n"], sz["n_c"], sz["Nq"], sz["n_t"], sz["n_tail"]], dtype=np.int32)
    n, nt = sz["n"], sz["n_tail"]
    F, T, tF = np.zeros(3 * n), np.zeros(3 * n), np.zeros(3 * nt)
    ip = (C.POINTER(C.c_int) * 4)(*[a.ctypes.data_as(C.POINTER(C.c_int)) for a in ints])
    dp = (C.POINTER(C.c_double) * 9)(*[a.ctypes.data_as(C.POINTER(C.c_double)) for a in dbls])
    d = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    harness.adjh_forces(isz.ctypes.data_as(C.POINTER(C.c_int)), ip, dp, d(par), d(x), d(F), d(T), d(tF))
    assert rel_err(F, ref["force"]) < 1e-10
    assert rel_err(T, ref["torque"]) < 1e-10
    assert rel_err(tF, ref["t_force"]) < 1e-10


def _adjoint_fixture():
    from brownian_dynamics_cuda_gb300 import Fiber
    z = dict(np.load(os.path.join(ROOT, "tests", "golden", "adjoint", "ref_3nuc.npz")))
    fib = Fiber.from_arrays({k[6:]: v for k, v in z.items() if k.startswith("fiber_")})
    return fib, z


def test_adjoint_reference_fixture_is_the_oracle():
    """The oracle's FP64 reference gradient fixture (tests/golden/adjoint/,
    made by make_adjoint_golden.py): its observable is the oracle's rollout
    on the stored fiber and noise, and one of its central differences
    reproduces."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("mkadj", os.path.join(ROOT, "tests", "golden",
                                                                        "make_adjoint_golden.py"))
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    fib, z = _adjoint_fixture()
    assert mk.observable(fib, z["rr"], z["p"]) == float(z["loss"])
    th = mk.theta_of(fib)
    d = 5e-4 * th[3]
    tp, tm = th.copy(), th.copy()
    tp[3] += d
    tm[3] -= d
    g3 = (mk.observable(mk.with_theta(fib, tp), z["rr"], z["p"]) -
          mk.observable(mk.with_theta(fib, tm), z["rr"], z["p"])) / (2 * d)
    assert abs(g3 - z["grad"][3]) <= 1e-5 * abs(z["grad"][3])


def test_cholesky_backward_identity():
    """The Cholesky backward the adjoint kernels implement: for
    f(D) = u_bar . (s L(D) p), D = L L^T, the gradient contracted with any
    symmetric dD is <V (Phi V^T), dD>, V = L^-T, Phi = s tril(u p^T) with the
    diagonal halved, u = L^T u_bar (numpy, against central differences)."""
    rng = np.random.default_rng(4)
    m, s = 24, 0.7
    Q = rng.normal(size=(m, m))
    D = Q @ Q.T + m * np.eye(m)
    p, ub = rng.normal(size=m), rng.normal(size=m)
    f = lambda Dm: ub @ (s * np.linalg.cholesky(Dm) @ p)
    L = np.linalg.cholesky(D)
    u = L.T @ ub
    Phi = s * np.tril(np.outer(u, p))
    Phi[np.diag_indices(m)] *= 0.5
    V = np.linalg.inv(L.T)
    Dbar = V @ (Phi @ V.T)
    for _ in range(5):
        E = rng.normal(size=(m, m))
        E = E + E.T
        h = 1e-6
        fd = (f(D + h * E) - f(D - h * E)) / (2 * h)
        assert abs(np.sum(Dbar * E) - fd) <= 1e-7 * max(1.0, abs(fd))
