"""The tensor-core GEMM of the adjoint's Cholesky backward (csrc/k_tc_gemm.cu:
FP32 operands as three BF16 slices, six products per K step on tcgen05)
against FP64 products of the same operands: every mode the adjoint uses
(op(B) = B^T and B, the triangular K ranges of kmode 1, 3 and 4, batched
sub-blocks 2b (mp + 1) elements apart as in the doubling inverse), to
3e-6 of |A| |op(B)|, FP32-class; padding columns of C untouched; no
recorded timeout."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def gemm(tmp_path_factory):
    from brownian_dynamics_cuda_gb300 import LIB_PATH, load_library
    load_library()
    so = str(tmp_path_factory.mktemp("tcg") / "tcg.so")
    libdir = os.path.dirname(LIB_PATH)
    subprocess.check_call(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-shared", "-Xcompiler", "-fPIC",
                           os.path.join(ROOT, "tests", "tc_gemm_check.cu"), "-o", so, "-L", libdir, "-lbdgb300",
                           "-Xlinker", "-rpath=" + libdir])
    lib = C.CDLL(so)
    lib.check_tc_gemm.argtypes = [C.c_int, C.c_int, C.c_int, C.c_float, C.c_void_p, C.c_int, C.c_void_p, C.c_int,
                                  C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_long, C.c_void_p]
    return lib


def _ref(A64, B64, M, N, K, kmode, alpha):
    import torch
    ref = torch.zeros(M, N, dtype=torch.float64, device=A64.device)
    for I in range(M // 128):
        for J in range(N // 128):
            kb, ke = 0, K
            if kmode & 1:
                kb = max(kb, 128 * I)
            if kmode & 2:
                kb = max(kb, 128 * J)
            if kmode & 4:
                ke = min(ke, 128 * J + 128)
            if kb < ke:
                ref[128 * I:128 * I + 128, 128 * J:128 * J + 128] = \
                    alpha * A64[128 * I:128 * I + 128, kb:ke] @ B64[kb:ke, 128 * J:128 * J + 128]
    return ref


@pytest.mark.parametrize("M,N,K,tb,kmode,alpha", [(128, 128, 64, 1, 0, 1.0), (256, 384, 512, 1, 0, 1.0),
                                                  (512, 512, 512, 0, 0, -1.0), (512, 512, 512, 1, 3, 1.0),
                                                  (512, 512, 512, 0, 1, 1.0), (512, 512, 512, 0, 4, 0.5)])
def test_modes_against_fp64(gemm, M, N, K, tb, kmode, alpha):
    import torch
    g = torch.Generator(device="cpu").manual_seed(M + N + K + kmode)
    lda, ldb, ldc = K + 64, (K if tb else N) + 32, N + 16
    A = torch.randn(M, lda, generator=g, dtype=torch.float32).cuda()
    B = torch.randn(N if tb else K, ldb, generator=g, dtype=torch.float32).cuda()
    Cm = torch.full((M, ldc), 7.0, dtype=torch.float32, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert gemm.check_tc_gemm(M, N, K, alpha, A.data_ptr(), lda, B.data_ptr(), ldb, Cm.data_ptr(), ldc, tb, kmode, 1, 0,
                              err.data_ptr()) == 0
    assert int(err.item()) == 0
    A64 = A[:, :K].double()
    B64 = B[:, :K].double().T if tb else B[:, :N].double()
    ref = _ref(A64, B64, M, N, K, kmode, alpha)
    scale = float((A64.abs() @ B64.abs()).max())
    assert float((Cm[:, :N].double() - ref).abs().max()) <= 3e-6 * scale
    assert bool((Cm[:, N:] == 7.0).all())


def test_batched_subblocks(gemm):
    """The doubling inverse's form: T = U12 V22 for every diagonal 2b-block
    of an mp x mp matrix in one launch (operands 2b (mp + 1) elements apart)."""
    import torch
    mp, b = 1024, 256
    nodes, zs = mp // (2 * b), 2 * b * (mp + 1)
    g = torch.Generator(device="cpu").manual_seed(5)
    U = torch.triu(torch.randn(mp, mp, generator=g, dtype=torch.float32)).cuda()
    V = torch.triu(torch.randn(mp, mp, generator=g, dtype=torch.float32)).cuda()
    T = torch.zeros(mp, mp, dtype=torch.float32, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert gemm.check_tc_gemm(b, b, b, 1.0, U.data_ptr() + 4 * b, mp, V.data_ptr() + 4 * (b * mp + b), mp,
                              T.data_ptr() + 4 * b, mp, 0, 4, nodes, zs, err.data_ptr()) == 0
    assert int(err.item()) == 0
    for z in range(nodes):
        o = 2 * b * z
        A64, B64 = U[o:o + b, o + b:o + 2 * b].double(), V[o + b:o + 2 * b, o + b:o + 2 * b].double()
        ref = A64 @ B64
        scale = float((A64.abs() @ B64.abs()).max())
        assert float((T[o:o + b, o + b:o + 2 * b].double() - ref).abs().max()) <= 3e-6 * scale
    # nothing outside the nodes' U12 blocks was written
    mask = torch.ones(mp, mp, dtype=torch.bool, device="cuda")
    for z in range(nodes):
        o = 2 * b * z
        mask[o:o + b, o + b:o + 2 * b] = False
    assert bool((T[mask] == 0).all())
