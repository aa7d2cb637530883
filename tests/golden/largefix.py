"""Compact fixtures for the benchmark-size fibers (tests/golden/large/).

The fibers themselves are not stored: the generator (fiber_gen.config) writes
them again from their seeds, and the fixture keeps a SHA-256 digest of the
fiber as the reference readers load it, so a test can tell a different fiber
from a wrong result.  Arrays are stored whole, or, where that would be large,
"packed": a fixed subset of entries plus projections onto fixed weight
vectors (a checksum of the whole array), compared at the same relative
tolerance (|x - ref| <= tol * max|ref| per entry implies
|w.(x - ref)| <= tol * max|ref| * sum|w| per projection).
"""
from __future__ import annotations

import hashlib

import numpy as np

FIBER_KEYS = ("sizes", "scalars", "arrays", "state")
N_SUBSET = 1024
N_PROJ = 8


def fiber_digest(fib) -> np.ndarray:
    """SHA-256 over every size, scalar, array and state entry, keys sorted."""
    h = hashlib.sha256()
    for grp in FIBER_KEYS:
        d = getattr(fib, grp)
        for k in sorted(d):
            v = d[k]
            if isinstance(v, np.ndarray):
                a = np.ascontiguousarray(v, dtype=np.int32 if v.dtype.kind in "iu" else np.float64)
            else:
                a = np.array([v], dtype=np.float64)
            h.update(k.encode())
            h.update(a.tobytes())
    return np.frombuffer(h.digest(), dtype=np.uint8).copy()


def digest_arrays(*arrs) -> np.ndarray:
    h = hashlib.sha256()
    for a in arrs:
        h.update(np.ascontiguousarray(a, dtype=np.float64).tobytes())
    return np.frombuffer(h.digest(), dtype=np.uint8).copy()


def subset(n: int) -> np.ndarray:
    return np.unique((np.arange(N_SUBSET, dtype=np.int64) * 2654435761) % max(n, 1))


def weights(n: int) -> np.ndarray:
    i = np.arange(n, dtype=np.float64) + 1.0
    return np.stack([np.cos(0.7071067811865476 * i * (j + 1) + 0.3 * j) for j in range(N_PROJ)])


def pack(out: dict, key: str, v: np.ndarray, full: bool) -> None:
    v = np.ascontiguousarray(v, dtype=np.float64)
    if full or v.size <= N_SUBSET:
        out[key] = v
        return
    out[key + "__n"] = np.array(v.size)
    out[key + "__amax"] = np.array(np.abs(v).max())
    out[key + "__val"] = v[subset(v.size)]
    out[key + "__proj"] = weights(v.size) @ v


def has(z: dict, key: str) -> bool:
    return key in z or key + "__n" in z


def rel_err_packed(x: np.ndarray, z: dict, key: str) -> float:
    """max relative error of x against the stored array (whole or packed)."""
    x = np.asarray(x, dtype=np.float64)
    if key in z:
        ref = z[key]
        if ref.size == 0:
            return 0.0 if x.size == 0 else float("inf")
        return float(np.abs(x - ref).max() / np.abs(ref).max())
    n = int(z[key + "__n"])
    if x.size != n:
        return float("inf")
    amax = float(z[key + "__amax"])
    e1 = np.abs(x[subset(n)] - z[key + "__val"]).max() / amax
    w = weights(n)
    e2 = (np.abs(w @ x - z[key + "__proj"]) / (amax * np.abs(w).sum(axis=1))).max()
    return float(max(e1, e2))
