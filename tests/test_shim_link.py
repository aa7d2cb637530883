"""The reference's own main program links against libbdgb300.so unchanged.

main.cpp (with readfile.cpp, func.cpp, mt.cpp and utilities.cpp, compiled
from the reference sources where they lie) is built and linked with the
library in place of func_cuda.cu: every GPU entry point it calls
(func_cuda.h:37-52, main.cpp:377-517) must resolve to the library's shim.
MPI is replaced by a single-rank stand-in header (the reference runs with
one rank; its MPI split is dead code).  Link only: running it needs a GPU,
and the shim's steps are checked on the GPU by tests/test_gpu_shim.py.
Skipped where the reference tree is absent (the GPU host).
"""
import os
import subprocess

import pytest

from oracle.refpath import REF_SRC

MPI_STUB = """#pragma once
typedef int MPI_Comm;
#define MPI_COMM_WORLD 0
static inline int MPI_Init(int*, char***) { return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm, int* s) { *s = 1; return 0; }
static inline int MPI_Finalize() { return 0; }
"""


@pytest.mark.skipif(not os.path.exists(os.path.join(REF_SRC, "main.cpp")), reason="reference sources absent")
def test_reference_main_links_against_library(tmp_path):
    from brownian_dynamics_cuda_gb300 import LIB_PATH
    (tmp_path / "mpi.h").write_text(MPI_STUB)
    srcs = [os.path.join(REF_SRC, f) for f in ("main.cpp", "readfile.cpp", "func.cpp", "mt.cpp", "utilities.cpp")]
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cuda_lib = os.path.join(cuda, "lib64")
    exe = tmp_path / "bd_main"
    cmd = ["g++", "-O1", "-std=c++11", "-w", "-I" + str(tmp_path), "-I" + REF_SRC, "-I" + os.path.join(cuda, "include"), *srcs, "-o", str(exe),
           "-L" + os.path.dirname(LIB_PATH), "-lbdgb300", "-Wl,-rpath-link," + cuda_lib, "-Wl,--no-undefined"]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, p.stderr[-3000:]
    syms = subprocess.run(["nm", "-u", str(exe)], capture_output=True, text=True).stdout
    for name in ("cuda_application_init_D_Chol", "cuda_application_init_data", "main_cuda", "free_all"):
        assert name in syms, name  # resolved by the library, not defined in the program
