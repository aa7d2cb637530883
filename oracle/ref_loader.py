"""Test infrastructure: the reference's input readers and set-up, restated in
numpy, so that the oracle can be built from the reference input files
without the product library.

Every function names the reference lines it restates.  Arithmetic keeps the
reference's operation order (Python floats and numpy element-wise ops round
each operation on its own, as the reference does when built without FMA
contraction), so a fiber loaded here equals the one the reference's main()
sets up bit for bit.  Only tests, bench.py's CPU legs and smoke() use this
module; it is never the product.

Supported: restart = 0 (initial structure from data_mod) and LH models
without N-terminal beads, the cases the product's loader accepts.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np

# constants.h
PI = 3.141592653589790
LO = 3.0
ETA = 1.137076e-12
R_H = 1.2


def _lines(path: str) -> list[list[str]]:
    with open(path) as f:
        return [ln.split() for ln in f]


def read_const(path: str) -> list[float]:
    """readfile.cpp:14-37 (Read_const): every line after the first, second token."""
    rows = _lines(path)
    return [float(t[1]) for t in rows[1:]]


def read_initial_struc(path: str):
    """readfile.cpp:39-134 (Read_initial_struc): four lines per bead (position
    and type, then the a, b, c frame vectors)."""
    rows = _lines(path)
    r, a, b, c, typ = [], [], [], [], []
    for i, t in enumerate(rows):
        k = i % 4
        if k == 0:
            r += [float(t[0]), float(t[1]), float(t[2])]
            typ.append(int(t[3]))
        else:
            (a, b, c)[k - 1].extend(float(x) for x in t[:3])
    typ = np.array(typ, dtype=np.int32)
    rad = np.where(typ == 1, 5.0, 1.5)
    return np.array(r), np.array(a), np.array(b), np.array(c), typ, rad


def read_core(path: str):
    """readfile.cpp:137-171 (Read_core): three-token lines are charge sites (A
    to nm), the others charges."""
    pos, q = [], []
    for t in _lines(path):
        if not t:
            continue
        if len(t) == 3:
            pos += [float(t[0]) / 10, float(t[1]) / 10, float(t[2]) / 10]
        else:
            q.append(float(t[0]))
    return np.array(pos), np.array(q)


def read_tail(path: str) -> dict:
    """readfile.cpp:174-233 (Read_tail): one bead per line."""
    out = {k: [] for k in ("pos", "q", "grp", "fix", "rad", "bond_c", "bond_v", "angle_c", "angle_v")}
    for t in _lines(path):
        if not t:
            continue
        out["pos"] += [float(t[6]) / 10, float(t[7]) / 10, float(t[8]) / 10]
        out["q"].append(float(t[3]) * 1.12)
        out["grp"].append(int(t[1]))
        out["fix"].append(int(t[2]))
        out["rad"].append(float(t[4]) / 10)
        out["bond_c"].append(float(t[10]) * 100 * 4.142e-3 / 0.5962)
        out["bond_v"].append(float(t[9]) / 10)
        out["angle_c"].append(float(t[12]) * 4.142e-3 / 0.5962)
        out["angle_v"].append(float(t[11]) * PI / 180)
    return {k: np.array(v, dtype=np.int32 if k in ("grp", "fix") else np.float64) for k, v in out.items()}


def read_lh(path: str) -> dict:
    """readfile.cpp:235-337 (Read_LH): section headers '# N-term', '# G-head',
    '# C-term'; other '#' lines skipped; parameters kept in file order."""
    sec = None
    pos = {"N": [], "G": [], "C": []}
    par = {k: [] for k in ("q", "vdw_hh", "vdw_hc", "vdw_hl", "vdw_ht", "kstr", "kben", "streq", "betaeq", "conn",
                           "radius")}
    for t in _lines(path):
        if len(t) < 2:
            continue
        if t[1] in ("N-term", "G-head", "C-term"):
            sec = t[1][0]
            continue
        if t[0] == "#":
            continue
        pos[sec] += [float(t[0]), float(t[1]), float(t[2])]
        par["q"].append(float(t[3]) * 0.66)
        par["vdw_hh"].append(float(t[4]))
        par["vdw_hc"].append(float(t[5]))
        par["vdw_hl"].append(float(t[6]))
        par["vdw_ht"].append(float(t[7]))
        par["kstr"].append(float(t[8]) * 4.142e-3 / 0.5962)
        par["kben"].append(float(t[9]) * 4.142e-3 / 0.5962)
        par["streq"].append(float(t[13]))
        par["betaeq"].append(float(t[14]) * PI / 180)
        par["conn"].append(int(t[12]))
        par["radius"].append(0.5)
    out = {k: np.array(v, dtype=np.int32 if k == "conn" else np.float64) for k, v in par.items()}
    out.update({"n_pos": np.array(pos["N"]), "g_pos": np.array(pos["G"]), "c_pos": np.array(pos["C"]),
                "n_lh_n": len(pos["N"]) // 3, "n_lh_g": len(pos["G"]) // 3, "n_lh_c": len(pos["C"]) // 3})
    return out


def read_lh_core(path: str, n_c: int) -> np.ndarray:
    """readfile.cpp:563-584 (Read_LH_core): the first n_c lines, one flag each."""
    flags = np.zeros(n_c, dtype=np.int32)
    for i, t in enumerate(_lines(path)[:n_c]):
        flags[i] = int(t[0])
    return flags


def _c_round(x: float) -> float:
    """C round(): halves away from zero."""
    f = math.floor(abs(x))
    return math.copysign(f + 1.0 if abs(x) - f >= 0.5 else f, x)


def twist_angle_phi(w: int) -> float:
    """func.cpp:13-91: tabulated for 2 <= w <= 11, else from the linker's base pairs."""
    table = {2: 0.9007, 3: -0.6754, 4: -0.3519, 5: -0.1463, 6: 0.0215, 7: 0.1178, 8: 0.2025, 9: 0.2726,
             10: -0.2415, 11: -0.15}
    if w <= 11:
        if w not in table:
            raise ValueError("Wrong DNA linker length!")
        return table[w]
    nbp = (w + 1) * 3 / 0.34
    turns = nbp / 10.3
    rot = _c_round(turns)
    per_bp = rot * 360 / nbp
    twist = per_bp - 34.95
    whole = nbp * twist
    seg = whole / (w + 1)
    return PI * seg / 180.00


def update_phi_o(typ: np.ndarray) -> np.ndarray:
    """func.cpp:412-425: every bead from a core to the next gets the twist of that linker."""
    n = typ.size
    phi = np.zeros(n)
    for i in range(n):
        if typ[i] == 1:
            k = 1
            while i + k < n and typ[i + k] == 0:
                k += 1
            phi[i:i + k] = twist_angle_phi(k - 1)
    return phi


def _place(r, a, b, c, i, tpl):
    """r_i + a_i x + b_i y + c_i z per component, left to right (func.cpp:1693-1695, 2043-2049)."""
    x, y, z = tpl[0::3], tpl[1::3], tpl[2::3]
    out = np.empty((x.size, 3))
    for d in range(3):
        out[:, d] = r[3 * i + d] + a[3 * i + d] * x + b[3 * i + d] * y + c[3 * i + d] * z
    return out.ravel()


@dataclass
class RefFiber:
    """A fiber as the reference's main() sets it up: the fields the oracle reads."""
    sizes: dict
    scalars: dict
    arrays: dict
    state: dict
    setup: np.ndarray = field(default_factory=lambda: np.zeros(15))

    @property
    def n_D(self) -> int:
        return self.sizes["n"] + self.sizes["n_tail"] + self.sizes["n_LH"]

    @property
    def m(self) -> int:
        return 3 * self.n_D


def load(directory: str, core_file: str, tail_file: str, lh_file: str, data_file: str = "data_mod",
         lh_flags_file: str = "LH.in") -> RefFiber:
    """main.cpp:38-297: constants from setup.txt, the initial structure,
    phi_o, core charges, tails (build_tail), linker histones (build_LH) and
    the rotational noise variances r_var."""
    j = lambda f: os.path.join(directory, f)  # noqa: E731
    setup = np.array(read_const(j("setup.txt")))
    T, Cs = setup[0], setup[11]
    if int(setup[12]) != 0:
        raise NotImplementedError("restart = 1: the oracle loader reads the initial structure only")
    mg = int(setup[10])
    # main.cpp:66-99
    kb = 1.380649e-5
    kbt = kb * 300.0
    cs = Cs * 1000
    q_l = LO * (-5.8824) * (1.901912136835033e-8 * math.pow(cs, 3.0) + -8.211102025728157e-6 * math.pow(cs, 2.0)
                            + 7.554037628581672e-3 * cs + 3.524292543853884e-1)
    debye = 0.736 * math.sqrt((Cs / 0.05) * (298 / T))
    per, debyell = (50, debye) if mg == 0 else (30, 2.5)
    time_step = 1e-12
    sc = {"h": 100 * kbt / (LO * LO), "g": per * kbt / LO, "s": 72.429 * kbt / LO, "debyell": debyell,
          "debye": debye, "q_l": q_l, "k_e": 0.4151 * kb * 300, "k_ex": 0.001 * kbt, "k_h1": 10.0 * kbt,
          "sigma_DNA_DNA": setup[4], "sigma_DNA_Core": setup[5], "sigma_Core_Core": setup[6],
          "sigma_Tail_Tail": setup[7], "sigma_Tail_Linker": setup[8], "sigma_Tail_Core": setup[9],
          "a1": kbt / (6 * PI * ETA), "a2": kbt / (8 * PI * ETA), "time_step": time_step,
          "del_": time_step / kbt, "s2dt": math.sqrt(2 * time_step)}
    sc = {k: float(v) for k, v in sc.items()}
    r, a, b, c, typ, rad = read_initial_struc(j(data_file))
    n = typ.size
    n_c = int((typ == 1).sum())
    cores = np.nonzero(typ == 1)[0]
    phi_o = update_phi_o(typ)
    core_pos, core_q = read_core(j(core_file))
    # tails: every core carries one (main.cpp:197-205), build_tail func.cpp:1672-1711
    tl = read_tail(j(tail_file))
    n_t = tl["q"].size
    n_grp = 1 + int(np.count_nonzero(tl["grp"][1:] != tl["grp"][:-1]))
    nc_t_flag = np.ones(n_c, dtype=np.int32)
    r_t = np.concatenate([_place(r, a, b, c, i, tl["pos"]) for i in cores]) if n_t else np.zeros(0)
    rep = lambda v: np.tile(v, n_c)  # noqa: E731
    t_grp = np.concatenate([tl["grp"] + k * n_grp for k in range(n_c)]).astype(np.int32)
    # LH: build_LH func.cpp:2029-2059 for the flagged cores
    lh = read_lh(j(lh_file))
    if lh["n_lh_n"] != 0:
        raise NotImplementedError("LH models with N-terminal beads")
    nc_lh_flag = read_lh_core(j(lh_flags_file), n_c)
    nlh = lh["n_lh_n"] + lh["n_lh_c"]
    tpl = lh["c_pos"][:3 * nlh]
    bound = [i for k, i in enumerate(cores) if nc_lh_flag[k] == 1]
    r_lh = np.concatenate([_place(r, a, b, c, i, tpl) for i in bound]) if bound and nlh else np.zeros(0)
    lh_rad = np.tile(lh["radius"][:nlh], len(bound)) if nlh else np.zeros(0)
    # main.cpp:286-297
    rv_core = 2.0 * time_step * kbt / (8 * PI * ETA * 125.0)
    rv_dna = 2.0 * time_step * kbt / (4 * PI * ETA * R_H * R_H * LO)
    r_var = np.zeros(3 * n)
    for i in range(n):
        if typ[i] != 0:
            r_var[3 * i:3 * i + 3] = rv_core
        else:
            r_var[3 * i] = rv_dna
    sizes = {"n": n, "n_c": n_c, "Nq": core_q.size, "n_t": n_t, "n_tail": n_t * n_c, "n_lh_n": lh["n_lh_n"],
             "n_lh_g": lh["n_lh_g"], "n_lh_c": lh["n_lh_c"], "n_LH": nlh * len(bound)}
    arrays = {"type": typ, "rad": rad, "phi_o": phi_o, "r_var": r_var, "core_pos": core_pos, "core_q": core_q,
              "tail_pos": tl["pos"], "tail_fix": tl["fix"], "nc_t_flag": nc_t_flag, "h_t": rep(tl["bond_c"]),
              "g_t": rep(tl["angle_c"]), "lo_t": rep(tl["bond_v"]), "beta_o_t": rep(tl["angle_v"]),
              "t_q": rep(tl["q"]), "t_rad": rep(tl["rad"]), "t_grp": t_grp, "t_fix": rep(tl["fix"]).astype(np.int32),
              "LH_g_pos": lh["g_pos"], "LH_conn": lh["conn"], "nc_lh_flag": nc_lh_flag, "LH_q": lh["q"],
              "LH_vdw_hh": lh["vdw_hh"], "LH_vdw_hc": lh["vdw_hc"], "LH_vdw_hl": lh["vdw_hl"],
              "LH_vdw_ht": lh["vdw_ht"], "LH_kstr": lh["kstr"], "LH_kben": lh["kben"], "LH_streq": lh["streq"],
              "LH_betaeq": lh["betaeq"], "lh_rad": lh_rad}
    state = {"r": r, "a": a, "b": b, "c": c, "r_t": r_t, "r_lh": r_lh}
    return RefFiber(sizes, sc, arrays, state, setup)
