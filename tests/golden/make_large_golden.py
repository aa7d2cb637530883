"""Generates the benchmark-size fixtures in tests/golden/large/.

  cfg1_50nuc_44bp_LH.npz  the headline fiber (3N = 11,700): start-state
      forces, torques and energy, and one complete step (noise displacement rd,
      positions, frames, tail and LH beads), all from the reference's own CPU
      code (oracle/_ref/libbdref.so: func.cpp, readfile.cpp, mt.cpp and
      utilities.cpp compiled from the reference sources), its single-threaded
      Cholesky included.  Stored whole.
  cfg4_200nuc_LH.npz  the large fiber (3N = 46,200): start-state forces by the
      reference's code; one complete step by the CPU oracle (whose step is the
      reference's bit for bit at every size it was compared, and whose
      column-blocked Cholesky gives the reference's factor bit for bit), since
      the reference's single-threaded 46,200 x 46,200 factorisation takes hours.
      Packed (largefix.py).
  cfg2_rep<k>.npz  four replicas of the batch workload (smallest, largest, and
      one of each other salt among the first 64): start-state forces and one
      step by the reference's code.  Packed.

The noise of each step is the reference's MT19937 stream (seeded); tests draw
it again with the oracle's restatement of that stream and check its digest.
Fibers are written again by fiber_gen from their seeds and checked against
the stored digest.

Run from the repository root after `make -C oracle ref`:
    python tests/golden/make_large_golden.py [cfg1] [cfg4] [cfg2]
"""
from __future__ import annotations

import os
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from brownian_dynamics_cuda_gb300.fiber_gen import config, write_fiber  # noqa: E402
from oracle import ref_loader  # noqa: E402
from oracle.pyoracle import Oracle, OracleNoise, Reference, set_threads  # noqa: E402
import largefix as lf  # noqa: E402

OUT = os.path.join(HERE, "large")
NOISE_SEED = 777
STATE = ("rd", "r", "a", "b", "c", "r_t", "r_lh")
FORCES = ("force", "torque", "t_force", "LH_force")


def _fiber(cfg: int, replica: int = 0):
    spec = config(cfg, seed=1, replica=replica)
    d = tempfile.mkdtemp(prefix="bdlarge_")
    files = write_fiber(spec, d)
    return spec, d, files, ref_loader.load(d, **files)


def _head(out: dict, cfg: int, replica: int, fib) -> None:
    out.update(cfg=np.array(cfg), seed=np.array(1), replica=np.array(replica), noise_seed=np.array(NOISE_SEED),
               m=np.array(fib.m), fiber_digest=lf.fiber_digest(fib))


def capture(cfg: int, replica: int, full: bool, step_by: str) -> str:
    t0 = time.time()
    spec, d, files, fib = _fiber(cfg, replica)
    out: dict = {}
    _head(out, cfg, replica, fib)
    ref = Reference(d, files["core_file"], files["tail_file"], files["lh_file"], seed=NOISE_SEED)
    f0 = ref.forces()
    for k in FORCES:
        lf.pack(out, "f0_" + k, f0[k], full)
    out["f0_energy"] = np.array(f0["energy"])
    rr, p = ref.noise(0)
    rr_o, p_o = OracleNoise(NOISE_SEED).step(0, fib.arrays["r_var"], fib.m)
    assert np.array_equal(rr, rr_o) and np.array_equal(p, p_o), "oracle noise differs from the reference's"
    out["noise_digest"] = lf.digest_arrays(rr, p)
    if step_by == "reference":
        e = ref.step(rr, p)
        got = {k: ref.get(k) for k in STATE}
    else:
        set_threads(os.cpu_count() or 1)
        o = Oracle(fib)
        fo = o.forces()
        for k in FORCES:
            assert np.array_equal(fo[k], f0[k]), ("oracle forces differ from the reference's", k)
        e = o.step(rr, p)
        got = {k: o.get(k) for k in STATE}
    for k in STATE:
        lf.pack(out, "step0_" + k, got[k], full)
    if not full:  # displacements, for the mixed path's relative bound (whole arrays give them directly)
        for k in ("r", "r_t", "r_lh"):
            lf.pack(out, "step0_d" + k, got[k] - fib.state[k], full)
    out["step0_energy"] = np.array(e)
    out["step0_source"] = np.array(step_by)
    os.makedirs(OUT, exist_ok=True)
    path = os.path.join(OUT, spec.name + ".npz")
    np.savez_compressed(path, **out)
    print(f"{spec.name}: m = {fib.m}, step by the {step_by}, {time.time() - t0:.0f} s -> {path}", flush=True)
    return path


def replicas() -> list[int]:
    """Smallest and largest of the first 64 replicas, plus the first replica
    of each salt that is not already among them."""
    sizes = []
    for i in range(64):
        s = config(2, seed=1, replica=i)
        sizes.append((i, s.cs))
    ms = {}
    for i, _ in sizes:
        _, d, _, fib = _fiber(2, i)
        ms[i] = fib.m
    pick = [min(ms, key=ms.get), max(ms, key=ms.get)]
    salts = {dict(sizes)[i] for i in pick}
    for i, cs in sizes:
        if cs not in salts and len(pick) < 4:
            pick.append(i)
            salts.add(cs)
    for i, _ in sizes:
        if len(pick) >= 4:
            break
        if i not in pick:
            pick.append(i)
    return pick


def main(which: list[str]) -> None:
    if "cfg1" in which:
        capture(1, 0, full=True, step_by="reference")
    if "cfg2" in which:
        for r in replicas():
            capture(2, r, full=False, step_by="reference")
    if "cfg4" in which:
        capture(4, 0, full=False, step_by="oracle")


if __name__ == "__main__":
    main(sys.argv[1:] or ["cfg1", "cfg2", "cfg4"])
