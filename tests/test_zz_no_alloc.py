"""The allocation-free noise-displacement entry point
(bd_noise_displacement_noalloc) against the context's own entry point
(bd_noise_displacement) on the same factor, twice in a row.

It exists for hosts that own all device memory through their own pool and
cannot let a library call cudaMalloc/cudaFree; its scratch is a fixed array
inside the library.  Tolerance: the 1e-10 relative bound of the FP64 parity
tests (both paths sum in the same order, so they are expected to agree
exactly)."""
import ctypes

import numpy as np
import pytest

from conftest import load_golden, rel_err

pytestmark = pytest.mark.gpu


def test_noalloc_matches_context_entry_point():
    import torch
    from brownian_dynamics_cuda_gb300 import PREC_FP64, Context, load_library
    fib, _ = load_golden("syn_4nuc_lh")
    ctx = Context(fib, precision=PREC_FP64)
    L_host = ctx.cholesky()                       # row-major lower factor
    m = fib.m
    lda = m
    dL = torch.tensor(np.ascontiguousarray(L_host.T), dtype=torch.float64, device="cuda")  # column-major
    lib = load_library()
    s2dt = fib.scalars["s2dt"]
    rng = np.random.default_rng(123)
    for call in range(2):
        p = rng.normal(size=m)
        ref = ctx.noise_displacement(p)
        dp = torch.tensor(p, dtype=torch.float64, device="cuda")
        drd = torch.full((m,), float("nan"), dtype=torch.float64, device="cuda")
        rc = lib.bd_noise_displacement_noalloc(m, ctypes.c_void_p(dL.data_ptr()), lda, ctypes.c_void_p(dp.data_ptr()),
                                               s2dt, ctypes.c_void_p(drd.data_ptr()), None)
        assert rc == 0, lib.bd_last_error()
        torch.cuda.synchronize()
        got = drd.cpu().numpy()
        assert np.all(np.isfinite(got))
        assert rel_err(got, ref) <= 1e-10, call


def test_noalloc_rejects_oversize():
    from brownian_dynamics_cuda_gb300 import load_library
    lib = load_library()
    one = ctypes.c_void_p(16)
    rc = lib.bd_noise_displacement_noalloc(16385, one, 16385, one, 1.0, one, None)
    assert rc == 1 and b"16384" in lib.bd_last_error()
