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
  * geometry: two-column zigzag - consecutive cores on opposite sides of
    the fiber axis with 36 degrees of twist per nucleosome, the rise chosen
    so each linker's beads sit about 3 nm apart between the exit site of one
    core and the entry site of the next (the first_coord/second_coord sites
    of func.cpp:687-723), random bends and frame jitter of up to 10 degrees;
    the construction is checked for charge-site clashes.
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


def _core_frame(toward, rng):
    """Core frame with its disk roughly horizontal (c ~ -z, jittered by up to
    10 degrees) and its exit site (second_coord: r - ro b - d1 c) on the rim
    facing `toward` (a horizontal direction)."""
    tilt = math.radians(rng.uniform(-10.0, 10.0))
    axis = _unit(np.cross([0.0, 0.0, 1.0], rng.normal(size=3)))
    c = _rot(axis, tilt) @ np.array([0.0, 0.0, -1.0])
    b = -toward
    b = _unit(b - np.dot(b, c) * c)
    a = np.cross(b, c)
    return a, b, c


def build_geometry(spec: FiberSpec, rng, sites=None):
    """Bead list [(pos, a, b, c, type)] of a two-column zigzag fiber.

    Core k sits at azimuth k * 216 degrees (consecutive cores on opposite
    sides of the fiber axis, 36 degrees of twist per nucleosome) at radius
    6 nm, its disk about horizontal and its exit site facing the next core;
    the rise to the next core (at least 9 nm) is solved so that its entry
    site (first_coord, func.cpp:687-709) lies (w + 1) * 3 nm from this
    core's exit site (second_coord, :711-723), w being the linker's bead
    count, and the w linker beads are spaced evenly on that segment with a
    random bend of up to 10 degrees.  The reference's core/core and DNA/core
    Lennard-Jones terms are not clamped (func.cpp:1401-1422, 1535-1561), so
    the construction is checked: no two cores' charge sites closer than
    2.5 nm, no linker bead closer than 3.0 nm to the sites of a core it
    interacts with.  A violation raises.
    """
    if sites is None:
        sites = np.zeros((1, 3))
    R, DZ_MIN = 6.0, 9.0
    beads, cores, frames = [], [], []

    def centre(k, z):
        psi = math.radians(216.0 * k)
        return np.array([R * math.cos(psi), R * math.sin(psi), z])

    def horiz(v):
        v = np.array([v[0], v[1], 0.0])
        return _unit(v)

    z = 0.0
    r = centre(0, 0.0)
    a, b, c = _core_frame(horiz(centre(1, 0.0) - r), rng)
    for k in range(spec.n_nuc):
        beads.append((r.copy(), a, b, c, 1))
        cores.append(r)
        frames.append((a, b, c))
        w = linker_beads(spec.linker_bp[k])
        exit_ = r - (RO * b + D1 * c)
        r2_xy = centre(k + 1, 0.0)
        a2, b2, c2 = _core_frame(horiz(centre(k + 2, 0.0) - r2_xy), rng)
        bm2 = -math.sin(THETA) * a2 + math.cos(THETA) * b2
        want = LO * (w + 1)

        def entry_at(dz):
            return centre(k + 1, z + dz) - RO * bm2 + D1 * c2

        lo_, hi_ = DZ_MIN, 80.0
        if np.linalg.norm(entry_at(lo_) - exit_) < want:
            for _ in range(80):
                mid = 0.5 * (lo_ + hi_)
                if np.linalg.norm(entry_at(mid) - exit_) < want:
                    lo_ = mid
                else:
                    hi_ = mid
        dz = lo_
        entry = entry_at(dz)
        seg = entry - exit_
        u = _unit(seg)
        side = _unit(np.cross(u, [0.0, 0.0, 1.0]) if abs(u[2]) < 0.99 else np.cross(u, [1.0, 0.0, 0.0]))
        for q in range(1, w + 1):
            frac = q / (w + 1)
            bulge = math.sin(math.pi * frac) * math.tan(math.radians(rng.uniform(-10.0, 10.0))) * np.linalg.norm(seg) / 4
            p = exit_ + frac * seg + bulge * side
            bb = _unit(np.cross(u, c) if abs(np.dot(u, c)) < 0.99 else np.cross(u, b))
            beads.append((p, u.copy(), bb, np.cross(u, bb), 0))
        z += dz
        r = centre(k + 1, z)
        a, b, c = a2, b2, c2
    _check_clashes(beads, cores, frames, sites)
    return beads


def _check_clashes(beads, cores, frames, sites):
    cores = np.array(cores)
    site_sets = [cores[j] + sites @ np.array(frames[j]) for j in range(len(cores))]
    typ = [bd[4] for bd in beads]
    core_index = np.cumsum(typ) - 1
    for j in range(len(cores)):
        for i in range(j + 1, len(cores)):
            if np.linalg.norm(cores[i] - cores[j]) > 14.0:
                continue
            dmin = np.sqrt(((site_sets[i][:, None] - site_sets[j][None]) ** 2).sum(-1)).min()
            if dmin < 2.5:
                raise RuntimeError(f"fiber_gen: cores {j} and {i} clash ({dmin:.2f} nm between sites)")
    n = len(beads)
    for bi, bd in enumerate(beads):
        if bd[4] != 0:
            continue
        if beads[bi - 1][4] == 1 or (bi + 1 < n and beads[bi + 1][4] == 1):
            continue  # next to a core: no DNA/core interaction (func.cpp:1316-1323)
        for j in range(len(cores)):
            if np.linalg.norm(cores[j] - bd[0]) > 14.0:
                continue
            dmin = np.sqrt(((site_sets[j] - bd[0]) ** 2).sum(-1)).min()
            if dmin < 3.0:
                raise RuntimeError(f"fiber_gen: linker bead {bi} is {dmin:.2f} nm from core {j}")


def write_fiber(spec: FiberSpec, directory: str) -> dict:
    """Writes the six reference input files; returns the file names for Fiber.load."""
    os.makedirs(directory, exist_ok=True)
    rng = np.random.default_rng(spec.seed)
    pos, q = _core_sites(rng, spec.n_sites)
    beads = build_geometry(spec, rng, pos)
    with open(os.path.join(directory, "data_mod"), "w") as f:
        for p, a, b, c, t in beads:
            f.write(f"{p[0]:20.13f}{p[1]:20.13f}{p[2]:20.13f}  {t}\n")
            for v in (a, b, c):
                f.write(f"{v[0]:20.13f}{v[1]:20.13f}{v[2]:20.13f}\n")
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
