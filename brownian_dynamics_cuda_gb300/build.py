"""In-tree build of libbdgb300.so (sm_103a) and of the oracle checker.

Every translation unit is compiled in parallel with one ``-gencode`` for
sm_103a; the physics units are built with ``-fmad=false`` so that FP64
results round like the reference's CPU code (no contracted multiply-adds).
No cmake, no torch extension machinery: plain nvcc/g++ invocations.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT, "libbdgb300.so")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# (source, extra flags)
UNITS = [
    ("host_system.cpp", []),
    ("compat_func_cuda.cpp", []),
    ("bd_capi.cu", []),
    ("k_frames.cu", ["-fmad=false"]),
    ("k_forces.cu", ["-fmad=false"]),
    ("k_rpy_chol.cu", ["-fmad=false"]),
    ("k_tc_chol.cu", []),
    ("k_noalloc.cu", ["-fmad=false"]),
    ("k_adjoint.cu", []),
    ("k_noise.cu", ["-fmad=false"]),
    ("k_krylov.cu", []),
    ("k_tc_gemm.cu", []),
]


def _cmd(src: str, flags: list[str], obj: str) -> list[str]:
    path = os.path.join(CSRC, src)
    inc = ["-I" + CSRC, "-I" + os.path.join(ROOT, "include")]
    if src.endswith(".cpp"):
        return ["g++", "-O2", "-fPIC", "-std=c++17", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
                "-I" + os.path.join(CUDA, "include"), *inc, "-c", path, "-o", obj]
    return [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
            *flags, *inc, "-c", path, "-o", obj]


def _run(cmd: list[str]) -> tuple[list[str], int, str]:
    p = subprocess.run(cmd, capture_output=True, text=True)
    return cmd, p.returncode, p.stdout + p.stderr


def build_lib(verbose: bool = False, extra_nvcc: list[str] | None = None) -> str:
    """Compiles libbdgb300.so into brownian_dynamics_cuda_gb300/_lib/ and returns its path."""
    os.makedirs(OUT, exist_ok=True)
    objs, cmds = [], []
    for src, flags in UNITS:
        obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
        objs.append(obj)
        f = list(flags)
        if extra_nvcc and src.endswith(".cu"):
            f += extra_nvcc
        cmds.append(_cmd(src, f, obj))
    with cf.ThreadPoolExecutor(max_workers=min(len(cmds), os.cpu_count() or 4)) as ex:
        for cmd, rc, log in ex.map(_run, cmds):
            if verbose or rc != 0:
                sys.stderr.write(" ".join(cmd) + "\n" + log)
            if rc != 0:
                raise RuntimeError("compilation failed: " + os.path.basename(cmd[-3] if cmd[-2] == "-o" else cmd[-1]))
    tmp = LIB + ".tmp"
    cmd, rc, log = _run([NVCC, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"])
    if rc != 0:
        sys.stderr.write(log)
        raise RuntimeError("link failed")
    os.replace(tmp, LIB)
    return LIB


def build_oracle(verbose: bool = False) -> None:
    """Builds oracle/liboracle.so and, when the reference tree is present, oracle/_ref/libbdref.so."""
    odir = os.path.join(ROOT, "oracle")
    targets = ["liboracle.so"]
    if subprocess.run(["make", "-s", "-C", odir, "have-ref"], capture_output=True).returncode == 0:
        targets.append("ref")
    for t in targets:
        p = subprocess.run(["make", "-s", "-C", odir, t], capture_output=True, text=True)
        if verbose or p.returncode != 0:
            sys.stderr.write(p.stdout + p.stderr)
        if p.returncode != 0:
            raise RuntimeError("oracle build failed: " + t)


if __name__ == "__main__":
    build_lib(verbose="-v" in sys.argv)
    build_oracle(verbose="-v" in sys.argv)
    print(LIB)
