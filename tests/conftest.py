import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")
from oracle.refpath import REF_TESTDATA  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    _ensure_built()  # before collection: some parameter lists load fibers through the library


def _ensure_built():
    from brownian_dynamics_cuda_gb300 import build
    srcs = [os.path.join(build.CSRC, f) for f in os.listdir(build.CSRC)]
    srcs.append(os.path.join(ROOT, "include", "bd_capi.h"))
    if not os.path.exists(build.LIB) or os.path.getmtime(build.LIB) < max(os.path.getmtime(f) for f in srcs):
        build.build_lib()
    orc = os.path.join(ROOT, "oracle", "liboracle.so")
    osrc = [os.path.join(ROOT, "oracle", f) for f in ("bd_oracle.cpp", "bd_oracle.h", "Makefile")]
    if not os.path.exists(orc) or os.path.getmtime(orc) < max(os.path.getmtime(f) for f in osrc):
        build.build_oracle()


@pytest.fixture(scope="session", autouse=True)
def built():
    _ensure_built()


def golden_names():
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz"))


def load_golden(name):
    from brownian_dynamics_cuda_gb300 import Fiber
    z = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    fib = Fiber.from_arrays({k[6:]: v for k, v in z.items() if k.startswith("fiber_")})
    return fib, z


def have_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def have_ref():
    return os.path.exists(os.path.join(ROOT, "oracle", "_ref", "libbdref.so")) and os.path.isdir(REF_TESTDATA)


def rel_err(x, ref):
    """max |x - ref| / max |ref| (norm-wise, inf norm)."""
    x, ref = np.asarray(x, dtype=np.float64), np.asarray(ref, dtype=np.float64)
    den = np.abs(ref).max() if ref.size else 1.0
    return float(np.abs(x - ref).max() / den) if ref.size else 0.0
