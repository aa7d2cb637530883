"""The allocation-free noise-displacement entry point
(bd_noise_displacement_noalloc) against the context's own entry point
(bd_noise_displacement) and against the reference's rd, twice in a row.

It exists for hosts that own all device memory through their own pool and
cannot let a library call cudaMalloc/cudaFree; its scratch is a fixed array
inside the library.  Tolerance: the 1e-10 relative bound of the FP64 parity
tests (both device paths sum in the same order, so they are expected to
agree exactly).  The file is collected last so that a failure here stops a
-x run only after every other test has run."""
import ctypes

import numpy as np
import pytest

from conftest import load_golden, rel_err

pytestmark = pytest.mark.gpu


def _call(lib, m, dL, lda, dp, s2dt, drd):
    rc = lib.bd_noise_displacement_noalloc(m, ctypes.c_void_p(dL.data_ptr()), lda, ctypes.c_void_p(dp.data_ptr()),
                                           s2dt, ctypes.c_void_p(drd.data_ptr()), None)
    assert rc == 0, lib.bd_last_error()


@pytest.mark.parametrize("pad", [0, 45])
def test_noalloc_matches_context_entry_point(pad):
    """Column-major L with lda = m and with a padded lda whose padding is NaN
    (a read of it would poison the result)."""
    import torch
    from brownian_dynamics_cuda_gb300 import PREC_FP64, Context, load_library
    fib, z = load_golden("syn_4nuc_lh")
    ctx = Context(fib, precision=PREC_FP64)
    L_host = ctx.cholesky()                       # row-major lower factor
    m = fib.m
    lda = m + pad
    colmajor = np.full((m, lda), np.nan)
    colmajor[:, :m] = L_host.T                    # row j of this array is column j of L
    dL = torch.tensor(colmajor, dtype=torch.float64, device="cuda")
    lib = load_library()
    s2dt = fib.scalars["s2dt"]
    rng = np.random.default_rng(123)
    # the reference's own rd for its step-0 noise (golden), then random p
    cases = [(z["noise0_p"], z["step0_rd"])] + [(p, None) for p in (rng.normal(size=m), rng.normal(size=m))]
    for call, (p, golden) in enumerate(cases):
        ref = ctx.noise_displacement(p)
        dp = torch.tensor(p, dtype=torch.float64, device="cuda")
        drd = torch.full((m,), float("nan"), dtype=torch.float64, device="cuda")
        _call(lib, m, dL, lda, dp, s2dt, drd)
        torch.cuda.synchronize()
        got = drd.cpu().numpy()
        assert np.all(np.isfinite(got)), call
        assert rel_err(got, ref) <= 1e-10, call
        if golden is not None:
            assert rel_err(got, golden) <= 1e-10, call


def test_noalloc_allocates_nothing_after_warm_up():
    """After one warm-up call (which may load the library's device code and
    with it the fixed scratch array), further calls leave the device's free
    memory and torch's allocator untouched."""
    import torch
    from brownian_dynamics_cuda_gb300 import load_library
    lib = load_library()
    m = 4000
    rng = np.random.default_rng(5)
    L = np.tril(rng.normal(size=(m, m)))
    dL = torch.tensor(np.ascontiguousarray(L.T), dtype=torch.float64, device="cuda")
    dp = torch.tensor(rng.normal(size=m), dtype=torch.float64, device="cuda")
    drd = torch.zeros(m, dtype=torch.float64, device="cuda")
    _call(lib, m, dL, m, dp, 0.5, drd)            # warm-up
    torch.cuda.synchronize()
    free0, alloc0 = torch.cuda.mem_get_info()[0], torch.cuda.memory_allocated()
    for _ in range(5):
        _call(lib, m, dL, m, dp, 0.5, drd)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert torch.cuda.memory_allocated() == alloc0
    assert rel_err(drd.cpu().numpy(), 0.5 * (L @ dp.cpu().numpy())) <= 1e-12


def test_noalloc_rejects_oversize():
    from brownian_dynamics_cuda_gb300 import load_library
    lib = load_library()
    one = ctypes.c_void_p(16)
    rc = lib.bd_noise_displacement_noalloc(16385, one, 16385, one, 1.0, one, None)
    assert rc == 1 and b"16384" in lib.bd_last_error()
