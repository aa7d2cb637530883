"""Generates tests/golden/adjoint/ref_3nuc.npz: an FP64 reference gradient of the
rollout observable, computed by the CPU oracle alone.

Fiber: 3 nucleosomes, 30-bp linkers, no linker histone (the synthetic
generator, seed 5); noise: the oracle's MT19937 port, seed 11; 6 steps;
observable = mean over the final 3 states of |r_{n-1} - r_0|^2 + Rg of the
chain beads.  Gradient with respect to (h, g, s, Debye length 1/debye, with
debyell scaled alongside) by central differences with steps of 1e-3 and
5e-4 relative, Richardson-extrapolated.  Every rollout is the oracle's step
(oracle/bd_oracle.cpp, bit for bit the reference's CPU step).

Run from the repository root:  python tests/golden/make_adjoint_golden.py
"""
from __future__ import annotations

import dataclasses
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from brownian_dynamics_cuda_gb300.fiber_gen import FiberSpec, make_fiber  # noqa: E402
from oracle.pyoracle import Oracle, OracleNoise  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "adjoint", "ref_3nuc.npz")
STEPS, WINDOW = 6, 3


def observable(fib, rr, p, steps=STEPS, window=WINDOW) -> float:
    o = Oracle(fib)
    total = 0.0
    for s in range(steps):
        o.step(rr[s], p[s])
        if s + 1 >= steps - window + 1:
            r = o.get("r").reshape(-1, 3)
            e = r[-1] - r[0]
            rg = np.sqrt(np.mean(np.sum((r - r.mean(axis=0)) ** 2, axis=1)))
            total += float(e @ e) + float(rg)
    return total / window


def with_theta(fib, th):
    sc = dict(fib.scalars)
    sc["h"], sc["g"], sc["s"] = th[0], th[1], th[2]
    kappa = 1.0 / th[3]
    sc["debyell"] = sc["debyell"] * kappa / sc["debye"]
    sc["debye"] = kappa
    return dataclasses.replace(fib, scalars=sc)


def theta_of(fib):
    sc = fib.scalars
    return np.array([sc["h"], sc["g"], sc["s"], 1.0 / sc["debye"]])


def reference_gradient(fib, rr, p):
    th = theta_of(fib)
    g = np.zeros(4)
    for k in range(4):
        est = []
        for rel in (1e-3, 5e-4):
            d = rel * th[k]
            tp, tm = th.copy(), th.copy()
            tp[k] += d
            tm[k] -= d
            est.append((observable(with_theta(fib, tp), rr, p) - observable(with_theta(fib, tm), rr, p)) / (2 * d))
        g[k] = (4 * est[1] - est[0]) / 3
    return g


def main():
    fib = make_fiber(FiberSpec(3, [30] * 3, lh=False, seed=5), tempfile.mkdtemp(prefix="bdadjg_"))
    nz = OracleNoise(11)
    rows = [nz.step(s, fib.arrays["r_var"], fib.m) for s in range(STEPS)]
    rr = np.array([r[0] for r in rows])
    p = np.array([r[1] for r in rows])
    loss = observable(fib, rr, p)
    grad = reference_gradient(fib, rr, p)
    out = {f"fiber_{k}": v for k, v in fib.to_arrays().items()}
    out.update(rr=rr, p=p, steps=np.array(STEPS), window=np.array(WINDOW), loss=np.array(loss), grad=grad,
               theta=theta_of(fib))
    np.savez_compressed(OUT, **out)
    print(OUT, loss, grad)


if __name__ == "__main__":
    main()
