"""Generates the golden fixtures of the parity tests by running the
reference's own CPU physics (oracle/_ref/libbdref.so, compiled from the
reference sources by `make -C oracle ref`).

Each fixture stores the fiber (inputs, as loaded by the library's readers),
the reference's MT19937 noise for each step, and the reference outputs:
forces/torques/energy at the start state, the noise displacement rd, row
sums and diagonal of D and L, and the full state after every step.

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import shutil
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from brownian_dynamics_cuda_gb300 import Fiber  # noqa: E402
from brownian_dynamics_cuda_gb300.fiber_gen import FiberSpec, write_fiber  # noqa: E402
from oracle.pyoracle import Reference  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
from oracle.refpath import REF_TESTDATA as REF_DATA  # noqa: E402


def capture(name: str, directory: str, files: dict, seed: int, steps: int) -> None:
    fib = Fiber.load(directory, **files)
    ref = Reference(directory, files["core_file"], files["tail_file"], files["lh_file"], seed=seed)
    out = {f"fiber_{k}": v for k, v in fib.to_arrays().items()}
    f0 = ref.forces()
    for k in ("force", "torque", "t_force", "LH_force"):
        out["f0_" + k] = f0[k]
    out["f0_energy"] = np.array(f0["energy"])
    for k in ("a", "b", "c", "alpha", "beta", "gamma", "length", "a_dna", "b_dna", "c_dna", "alpha_p", "beta_p",
              "gamma_p", "beta_t", "beta_lh"):
        out["s0_" + k] = ref.get(k)
    D, L = ref.tensor()
    out["D_rowsum"] = D.sum(axis=1)
    out["D_diag"] = np.diag(D).copy()
    out["D_col0"] = D[:, 0].copy()
    out["L_diag"] = np.diag(L).copy()
    out["L_rowsum"] = L.sum(axis=1)
    out["L_col0"] = L[:, 0].copy()
    del D, L
    for s in range(steps):
        rr, p = ref.noise(s)
        e = ref.step(rr, p)
        out[f"noise{s}_rr"] = rr
        out[f"noise{s}_p"] = p
        out[f"step{s}_energy"] = np.array(e)
        for k in ("r", "a", "b", "c", "r_t", "r_lh", "rd", "force", "torque", "t_force", "LH_force"):
            out[f"step{s}_{k}"] = ref.get(k)
    out["steps"] = np.array(steps)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **out)
    print(name, "m =", fib.m, "->", os.path.join(OUT, name + ".npz"))


def main() -> None:
    tmp = tempfile.mkdtemp()
    # 1. the reference's own 12-nucleosome example (test_data), LH on all cores
    d1 = os.path.join(tmp, "refdata")
    shutil.copytree(REF_DATA, d1)
    capture("ref_testdata_12nuc", d1, {"core_file": "core_data.reg.150mM", "tail_file": "tail_data.mod.200mM",
                                       "lh_file": "LH_N0G6C22.in"}, seed=20240601, steps=2)
    # 2. small synthetic fiber with linker histones (fast; all interaction kinds)
    d2 = os.path.join(tmp, "syn_lh")
    spec = FiberSpec(4, [26, 44, 30, 26], lh=True, seed=7, n_sites=120, tail_len=3, lh_charge_range=(0.0, 1.0),
                     cs=0.1)
    files = write_fiber(spec, d2)
    capture("syn_4nuc_lh", d2, files, seed=99, steps=3)
    # 3. synthetic config-0 fiber (12 nucleosomes, 26-bp linkers, no LH)
    from brownian_dynamics_cuda_gb300.fiber_gen import config
    d3 = os.path.join(tmp, "cfg0")
    files = write_fiber(config(0), d3)
    capture("cfg0_12nuc", d3, files, seed=4242, steps=1)
    shutil.rmtree(tmp, ignore_errors=True)


if __name__ == "__main__":
    main()
