"""Seeded synthetic chromatin fibers in the reference's input formats.

The reference ships one 12-nucleosome example and no generator.  This module
builds fibers of the sizes the benchmark configurations name and writes the
six input files the reference reads (readfile.cpp formats):

  setup.txt     15 positional values (readfile.cpp:14-38)
  data_mod      4 lines per bead: x y z type / a / b / c   (readfile.cpp:40-142)
  core_data     300 site lines (x y z, Angstrom) then 300 charge lines
  tail_data     13 columns per tail bead (readfile.cpp:183-250)
  LH_data       N-term / G-head / C-term sections, 15 columns (readfile.cpp:252-337)
  LH.in         one 0/1 flag per core

Model choices (the configurations leave them open):
  * core: 300 sites uniform on the surface of a cylinder (radius 5.5 nm,
    height 5.5 nm; side and caps by area) about the core's c axis; charges
    drawn U[-1, 1] and shifted by a common offset, clipped to [-1, 1], so the
    net charge is -100 e;
  * tails: 10 chains of `tail_len` beads, 0.7 nm apart, growing outward from
    10 anchor points on the core surface; the anchor bead of each chain is
    fixed (fix = 1), the chain is listed tip first as in the reference table;
    file charge +1 (the reference reader scales tail charges by 1.12);
    bond/angle constants of the reference table's first rows (0.09, 115.9 deg,
    1.10);
  * linker histone N0-G6-C22: six globular-head sites near the dyad and a
    22-bead C-terminal chain leaving the last head site; with
    `lh_charge_range=(0, 1)` every LH site charge is drawn U[0, 1];
  * geometry: two-start zigzag - consecutive linkers cross the fiber axis
    with a 36 degree twist per nucleosome and a small rise, each linker
    direction perturbed by a random bend of up to 10 degrees; linker beads sit
    3 nm apart between the exit site of one core and the entry site of the
    next (the first_coord/second_coord sites of func.cpp:687-723).
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass

import numpy as np

RO, D1, THETA = 4.8, 1.8, 1.2 * math.pi / 2
LO = 3.0


def linker_beads(bp: int) -> int:
    """Beads per linker for a linker of `bp` base pairs (0.34 nm per bp, 3 nm beads)."""
    return int(round(bp * 0.34 / 3.0))


@dataclass
class FiberSpec:
    n_nuc: int
    linker_bp: list            # per nucleosome (the linker that follows it)
    lh: bool = False
    cs: float = 0.150          # M
    temperature: float = 293.15
    seed: int = 1
    n_sites: int = 300
    tail_len: int = 5
    lh_charge_range: tuple | None = None   # None: fixed synthetic charges
    steps: int = 1000
    sampling: int = 100
    name: str = "fiber"


def config(idx: int, seed: int = 1, replica: int = 0) -> FiberSpec:
    """The benchmark fiber configurations 0-4 (config 2: one replica)."""
    if idx == 0:
        return FiberSpec(12, [26] * 12, lh=False, seed=seed, steps=1000, name="cfg0_12nuc_26bp")
    if idx == 1:
        return FiberSpec(50, [44] * 50, lh=True, seed=seed, lh_charge_range=(0.0, 1.0), steps=2000,
                         name="cfg1_50nuc_44bp_LH")
    if idx == 2:
        rng = np.random.default_rng(seed * 100003 + replica)
        nn = int(rng.integers(12, 49))
        bps = [int(b) for b in rng.integers(20, 61, size=nn)]
        cs = float(rng.choice([0.050, 0.100, 0.150]))
        return FiberSpec(nn, bps, lh=False, cs=cs, seed=seed * 1000 + replica, steps=500, name=f"cfg2_rep{replica}")
    if idx == 3:
        return FiberSpec(24, [30] * 24, lh=False, seed=seed, steps=200, name="cfg3_24nuc_30bp")
    if idx == 4:
        return FiberSpec(200, [26 if k % 2 == 0 else 44 for k in range(200)], lh=True, seed=seed,
                         lh_charge_range=(0.0, 1.0), steps=1000, name="cfg4_200nuc_LH")
    raise ValueError(idx)


def _unit(v):
    return v / np.linalg.norm(v)


def _rot(axis, ang):
    axis = _unit(axis)
    x, y, z = axis
    c, s = math.cos(ang), math.sin(ang)
    C = 1 - c
    return np.array([[c + x * x * C, x * y * C - z * s, x * z * C + y * s],
                     [y * x * C + z * s, c + y * y * C, y * z * C - x * s],
                     [z * x * C - y * s, z * y * C + x * s, c + z * z * C]])


def _core_sites(rng, n_sites):
    R, H = 5.5, 5.5
    pos = np.zeros((n_sites, 3))
    for k in range(n_sites):
        if rng.random() < 0.5:       # side (area 2 pi R H) vs caps (2 pi R^2): equal for R == H
            phi = rng.uniform(0, 2 * math.pi)
            pos[k] = [R * math.cos(phi), R * math.sin(phi), rng.uniform(-H / 2, H / 2)]
        else:
            rr = R * math.sqrt(rng.random())
            phi = rng.uniform(0, 2 * math.pi)
            pos[k] = [rr * math.cos(phi), rr * math.sin(phi), H / 2 if rng.random() < 0.5 else -H / 2]
    u = rng.uniform(-1.0, 1.0, n_sites)
    target = -100.0 * n_sites / 300.0
    lo, hi = -2.0, 2.0
    for _ in range(200):             # common shift so that sum(clip(u + d)) == target
        mid = 0.5 * (lo + hi)
        if np.clip(u + mid, -1, 1).sum() > target:
            hi = mid
        else:
            lo = mid
    q = np.clip(u + 0.5 * (lo + hi), -1, 1)
    q[-1] += target - q.sum()        # absorb the bisection residue
    return pos, q


def _tail_template(rng, tail_len):
    # 10 anchors around the core surface; chains grow radially outward
    rows = []
    for g in range(10):
        phi = 2 * math.pi * (g + 0.5) / 10 + rng.uniform(-0.1, 0.1)
        zc = (-1) ** g * 1.5
        out = np.array([math.cos(phi), math.sin(phi), 0.15 * (-1) ** g])
        out = _unit(out)
        anchor = np.array([5.8 * math.cos(phi), 5.8 * math.sin(phi), zc])
        chain = [anchor + out * 0.7 * k for k in range(tail_len)]  # anchor first
        for k in reversed(range(tail_len)):                          # listed tip first
            rows.append((g + 1, 1 if k == 0 else 0, chain[k]))
    return rows


def _lh_template(rng, lh_range):
    g = np.array([[5.2, -3.9, 1.1], [4.9, -3.0, -0.7], [5.7, -3.2, 0.5], [4.5, -3.7, 0.4], [4.2, -4.0, -0.8],
                  [5.8, -4.1, -0.5]])
    start = g[-1] + np.array([0.2, -0.4, 0.5])
    d1 = _unit(np.array([0.83, 0.33, 0.0]))
    d2 = _unit(np.array([-0.05, -0.89, 0.0]))
    c = [start]
    for k in range(1, 22):
        c.append(c[-1] + 0.88 * (d1 if k % 2 else d2 * 0.5 + d1 * 0.5))
    c = np.array(c)
    if lh_range is None:
        qg = np.array([-3.29, 4.22, 8.48, 0.28, 2.08, 3.27]) / 5.0
        qc = np.where(np.arange(22) % 3 == 1, 0.0, 0.8)
    else:
        qg = rng.uniform(lh_range[0], lh_range[1], 6)
        qc = rng.uniform(lh_range[0], lh_range[1], 22)
    return g, c, qg, qc


def build_geometry(spec: FiberSpec, rng):
    """Bead list [(pos, a, b, c, type)] of the zigzag chain.

    Each linker leaves its core along a zigzag direction (crossing the fiber
    axis, +36 degrees per nucleosome, small rise) and bends by up to 10
    degrees at every bead; the next core is placed so that its entry site
    (first_coord, func.cpp:687-709) is one bond length past the last bead.
    Core frames are tilted 20 degrees off the exit direction so that no exit
    angle is exactly zero (func.cpp:1228 divides by its sine).
    """
    beads = []
    rise = 1.1

    def zigzag(k):
        psi = k * math.radians(180.0 + 36.0)
        return _unit(np.array([math.cos(psi), math.sin(psi), rise / 10.0]))

    def bend(u):
        ang = math.radians(rng.uniform(-10.0, 10.0))
        axis = _unit(np.cross(u, rng.normal(size=3)))
        return _unit(_rot(axis, ang) @ u)

    u_in = bend(zigzag(-1))
    last = None
    cores = []
    for k in range(spec.n_nuc):
        # draw this nucleosome and its linker; re-draw (bounded) while it
        # clashes with earlier cores
        for attempt in range(256):
            u_out = bend(zigzag(k))
            nrm = np.cross(u_out, u_in)
            nrm = _unit(nrm if np.linalg.norm(nrm) > 1e-6 else np.cross(u_out, [0.0, 0.0, 1.0]))
            a = _unit(_rot(nrm, math.radians(20.0)) @ u_out)
            b = _unit(u_in - np.dot(u_in, a) * a)
            c = np.cross(a, b)
            if last is None:
                r = np.zeros(3)
            else:
                entry = last + LO * u_in
                bm = -math.sin(THETA) * a + math.cos(THETA) * b
                r = entry + RO * bm - D1 * c
            w = linker_beads(spec.linker_bp[k])
            d = r - (RO * b + D1 * c)
            u = u_out
            lk = []
            for q in range(w):
                if q > 0:
                    u = bend(u)
                d = d + LO * u
                bb = _unit(np.cross(u, c) if abs(np.dot(u, c)) < 0.99 else np.cross(u, b))
                lk.append((d.copy(), u.copy(), bb, np.cross(u, bb), 0))
            ok = True
            if cores:
                prev = np.array(cores)
                ok = np.linalg.norm(prev - r, axis=1).min() >= 9.5
                if ok and len(cores) > 1:
                    pts = np.array([x[0] for x in lk])
                    ok = np.linalg.norm(pts[:, None] - prev[None, :-1], axis=-1).min() >= 5.5
            if ok:
                break
            u_in = bend(u_in)
        beads.append((r.copy(), a, b, c, 1))
        beads.extend(lk)
        cores.append(r.copy())
        last = d
        u_in = bend(u)
    return beads


def write_fiber(spec: FiberSpec, directory: str) -> dict:
    """Writes the six reference input files; returns the file names for Fiber.load."""
    os.makedirs(directory, exist_ok=True)
    rng = np.random.default_rng(spec.seed)
    beads = build_geometry(spec, rng)
    with open(os.path.join(directory, "data_mod"), "w") as f:
        for p, a, b, c, t in beads:
            f.write(f"{p[0]:20.13f}{p[1]:20.13f}{p[2]:20.13f}  {t}\n")
            for v in (a, b, c):
                f.write(f"{v[0]:20.13f}{v[1]:20.13f}{v[2]:20.13f}\n")
    pos, q = _core_sites(rng, spec.n_sites)
    with open(os.path.join(directory, "core_data"), "w") as f:
        for p in pos * 10.0:
            f.write(f"{p[0]: .7e} {p[1]: .7e} {p[2]: .7e}\n")
        for v in q:
            f.write(f"{v: .7e}\n")
    with open(os.path.join(directory, "tail_data"), "w") as f:
        for g, fix, p in _tail_template(rng, spec.tail_len):
            p = p * 10.0
            ang_v, ang_c = (115.90, 1.10)
            f.write(f"{'T%02d' % g:>10}{g:10d}{fix:10d}{1.0:10.2f}{6.0:10.2f}{0.0:10.2f}{p[0]:10.3f}{p[1]:10.3f}"
                    f"{p[2]:10.3f}{7.00:10.2f}{0.09:10.2f}{ang_v:10.2f}{ang_c:10.2f}\n")
    g, cpos, qg, qc = _lh_template(rng, spec.lh_charge_range)
    with open(os.path.join(directory, "LH_data"), "w") as f:
        f.write("# bead position (x,y,z)   charge  VdW_hh  VdW_hc  VdW_hl  WdW_ht  kstr  kben  ktor  Seq  Conn  "
                "rstreq [nm]  betaeq [deg]\n# N-term\n# G-head\n")
        for k in range(6):
            conn = 1 if k == 5 else 0
            kstr = 10 if k == 5 else 0
            f.write(f"{g[k][0]:.4f} {g[k][1]:.4f} {g[k][2]:.4f} {qg[k] / 0.66:.6f} 1.5 1.75 2.25 1.65 {kstr} {conn} 0 "
                    f"{k + 1} {conn} 0.0 0.0\n")
        f.write("# C-term\n")
        for k in range(22):
            conn = 0 if k == 21 else 1
            beq = 0.0 if k in (0, 21) else 110.0
            f.write(f"{cpos[k][0]:.5f} {cpos[k][1]:.5f} {cpos[k][2]:.5f} {qc[k] / 0.66:.6f} 1.8 1.8 2.7 1.8 10 1 0 "
                    f"{k + 7} {conn} {1.5 if conn else 0.0} {beq}\n")
    with open(os.path.join(directory, "LH.in"), "w") as f:
        for _ in range(spec.n_nuc):
            f.write(("1" if spec.lh else "0") + "\n")
    vals = [("Temperature", spec.temperature), ("number_of_steps", spec.steps),
            ("frequency_of_sampling", spec.sampling), ("frequency_RP", 1), ("evd_DNA_DNA", 3.6),
            ("evd_DNA_Core", 2.4), ("evd_Core_Core", 1.2), ("evd_Tail_Tail", 1.8), ("evd_Tail_DNA", 2.7),
            ("evd_Tail_Core", 1.8), ("Mg", 0), ("Cs", spec.cs), ("restart", 0), ("unbind", 0),
            ("Pbind", 1 if spec.lh else 0)]
    with open(os.path.join(directory, "setup.txt"), "w") as f:
        f.write("$ configuration file written by fiber_gen\n")
        for k, v in vals:
            f.write(f"{k:24s}{v}\n")
    return {"core_file": "core_data", "tail_file": "tail_data", "lh_file": "LH_data"}


def make_fiber(spec: FiberSpec, directory: str):
    """Writes the files and loads them with the library's reference-format readers."""
    from .capi import Fiber
    files = write_fiber(spec, directory)
    return Fiber.load(directory, **files)
