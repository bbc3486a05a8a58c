"""Decks of the golden cases (LAMMPS subset read by ExaMiniMD and emd_gb300).

Shared by make_golden.py (which runs ExaMiniMD on them) and the parity tests
(which run the GB300 driver on the same decks).  SNAP cases need a
.snapcoeff / .snapparam pair: make_golden.py parses the W files that ship with
ExaMiniMD into numbers (element, radius, weight, coefficients, parameters) and
stores them in the fixture; write_snap_files() writes a plain pair back from
those numbers for either program.
"""
from __future__ import annotations

import os

LJ = """units lj
atom_style atomic
newton {newton}
lattice fcc 0.8442
region box block 0 {n} 0 {n} 0 {n}
create_box {ntypes} box
create_atoms 1 box
{mass_lines}
velocity all create {temp} 87287 loop geom
pair_style {style} 2.5
{coeff_lines}
neighbor 0.3 bin
neigh_modify delay 0 every {every} check no
fix 1 all nve
thermo {thermo}
run {steps}
"""

SNAP = """units metal
newton on
lattice sc {a}
region box block 0 {nx} 0 {ny} 0 {nz}
create_box {ntypes} box
create_atoms 1 box
{mass_lines}
pair_style snap
pair_coeff * * {coeff} {elem_names} {param} {type_elems}
thermo {thermo}
neighbor 1.0 bin
neigh_modify once no every {every} delay 0 check yes
velocity all create 300.0 4928459 loop geom
fix 1 all nve
run {steps}
"""

CASES = {
    # LJ, full CSR list, newton off (the configuration of the LJ-4M workload)
    "lj_fcc6_full_csr": dict(kind="lj", n=6, mass=1.0, temp=1.44, newton="off", every=20, thermo=10, steps=100,
                             args=["--neigh-type", "CSR", "--force-iteration", "NEIGH_FULL", "--comm-type", "SERIAL"],
                             dump_every=1, keep_steps=[0, 20, 21, 100]),
    # LJ, full 2D list (ExaMiniMD's default neighbour module), mass 2 as in.lj
    "lj_fcc4_full_2d": dict(kind="lj", n=4, mass=2.0, temp=1.4, newton="off", every=20, thermo=10, steps=40,
                            args=["--neigh-type", "2D", "--comm-type", "SERIAL"],
                            dump_every=20, keep_steps=[0, 20, 40]),
    # LJ, half CSR list with newton off (ghost pairs kept in both directions)
    "lj_fcc4_half_csr": dict(kind="lj", n=4, mass=1.0, temp=1.44, newton="off", every=10, thermo=10, steps=30,
                             args=["--neigh-type", "CSR", "--force-iteration", "NEIGH_HALF", "--comm-type", "SERIAL"],
                             dump_every=10, keep_steps=[0, 10, 30]),
    # LJ, half 2D list with newton on (exercises CommSerial::update_force)
    "lj_fcc4_half_2d_newton": dict(kind="lj", n=4, mass=1.0, temp=1.44, newton="on", every=10, thermo=10, steps=30,
                                   args=["--neigh-type", "2D", "--force-iteration", "NEIGH_HALF",
                                         "--comm-type", "SERIAL"],
                                   dump_every=10, keep_steps=[0, 10, 30]),
    # LJ with two types of different mass (types drawn by the reference's rand()),
    # three pair_coeff lines of which the last one holds (stack parameters)
    "lj_fcc4_2types_full_csr": dict(kind="lj", n=4, mass=1.0, masses=[1.0, 2.5], temp=1.44, newton="off", every=10,
                                    coeffs=[(1, 1, 1.0, 1.0, 2.5), (1, 2, 1.3, 1.05, 2.5), (2, 2, 0.8, 0.95, 2.5)],
                                    thermo=10, steps=30,
                                    args=["--neigh-type", "CSR", "--force-iteration", "NEIGH_FULL",
                                          "--comm-type", "SERIAL"],
                                    dump_every=10, keep_steps=[0, 10, 30]),
    # LJ intensity dial (pair_style lj/cut/idial: each pair force evaluated 3
    # times at a third), full CSR and half CSR lists
    "lj_idial_fcc4_full_csr": dict(kind="lj_idial", n=4, mass=1.0, temp=1.44, newton="off", every=10,
                                   coeffs=[(1, 1, 1.0, 1.0, 2.5, 3)], thermo=10, steps=30,
                                   args=["--neigh-type", "CSR", "--force-iteration", "NEIGH_FULL",
                                         "--comm-type", "SERIAL"],
                                   dump_every=10, keep_steps=[0, 10, 30]),
    "lj_idial_fcc4_half_csr": dict(kind="lj_idial", n=4, mass=1.0, temp=1.44, newton="off", every=10,
                                   coeffs=[(1, 1, 1.0, 1.0, 2.5, 3)], thermo=10, steps=30,
                                   args=["--neigh-type", "CSR", "--force-iteration", "NEIGH_HALF",
                                         "--comm-type", "SERIAL"],
                                   dump_every=10, keep_steps=[0, 10, 30]),
    # LJ, CSR_MAPCONSTR (neighbor_csr_map_constr.h): the CSR list built through
    # a hash set, so its rows hold the CSR pairs in the hash map's order
    "lj_fcc4_full_csrmap": dict(kind="lj_mapconstr", n=4, mass=1.0, temp=1.44, newton="off", every=10, thermo=10,
                                steps=30,
                                args=["--neigh-type", "CSR_MAPCONSTR", "--force-iteration", "NEIGH_FULL",
                                      "--comm-type", "SERIAL"],
                                dump_every=10, keep_steps=[0, 10, 30]),
    # SNAP W, the shipped in.snap.W geometry (sc 4x8x8 = 256 atoms)
    "snap_W_sc": dict(kind="snap", a=3.1803, nx=4, ny=8, nz=8, mass=183.84, elem="W", every=1, thermo=5, steps=5,
                      coeff="W.snapcoeff", param="W.snapparam",
                      args=["--neigh-type", "CSR", "--comm-type", "SERIAL"], dump_every=5, keep_steps=[0, 5]),
    # two SNAP elements on two types (Ta06A parameters, synthetic second
    # element): type 1 names B, type 2 names A.  ExaMiniMD reads the element
    # of 0-based type t from map[t], which it filled at 1-based indices, so
    # type 0 takes element 0 (A) and type 1 the element named first (B).
    "snap_AB_sc": dict(kind="snap", a=3.316, nx=4, ny=4, nz=4, mass=180.88, masses=[180.88, 150.0],
                       elem="A", elems=["A", "B"], type_elems=["B", "A"], every=1, thermo=5, steps=10,
                       coeff="AB.snapcoeff", param="Ta06A.snapparam", synthetic_second=dict(radius=0.46, weight=0.85,
                                                                                           scale=0.9, seed=11),
                       args=["--neigh-type", "CSR", "--comm-type", "SERIAL"], dump_every=5, keep_steps=[0, 5, 10]),
    # SNAP Ta, the shipped in.snap.Ta06A geometry (sc 4^3 = 64 atoms, twojmax 6), 2D list
    "snap_Ta_sc": dict(kind="snap", a=3.316, nx=4, ny=4, nz=4, mass=180.88, elem="Ta", every=1, thermo=5, steps=10,
                       coeff="Ta06A.snapcoeff", param="Ta06A.snapparam",
                       args=["--neigh-type", "2D", "--comm-type", "SERIAL"], dump_every=5, keep_steps=[0, 5, 10]),
}


def snap_elements(snap: dict) -> list[dict]:
    """The element records of a SNAP number set (one-element sets keep the
    flat elem / radius / weight / beta keys)."""
    if "elements" in snap:
        return snap["elements"]
    return [dict(name=snap["elem"], radius=snap["radius"], weight=snap["weight"], beta=snap["beta"])]


def deck_text(case: dict) -> str:
    if case["kind"] == "snap":
        masses = case.get("masses", [case["mass"]])
        elems = case.get("elems", [case["elem"]])
        fields = {k: v for k, v in case.items() if k not in ("type_elems", "elems", "masses")}
        return SNAP.format(ntypes=len(masses),
                           mass_lines="\n".join(f"mass {t + 1} {m}" for t, m in enumerate(masses)),
                           elem_names=" ".join(elems),
                           type_elems=" ".join(case.get("type_elems", [case["elem"]] * len(masses))), **fields)
    if case["kind"] in ("lj", "lj_idial", "lj_mapconstr"):
        masses = case.get("masses", [case["mass"]])
        coeffs = case.get("coeffs", [(1, 1, 1.0, 1.0, 2.5)])
        style = "lj/cut/idial" if case["kind"] == "lj_idial" else "lj/cut"
        return LJ.format(ntypes=len(masses), style=style,
                         mass_lines="\n".join(f"mass {t + 1} {m}" for t, m in enumerate(masses)),
                         coeff_lines="\n".join("pair_coeff " + " ".join(str(v) for v in c) for c in coeffs),
                         **case)
    return SNAP.format(**case)


def write_snap_files(work: str, case: dict, snap: dict) -> None:
    """snap: elem, radius, weight, beta (ncoeffall floats) -- or a list of
    such records under "elements" -- and params {key: value}."""
    elems = snap_elements(snap)
    with open(os.path.join(work, case["coeff"]), "w") as fp:
        fp.write(f"{len(elems)} {len(elems[0]['beta'])}\n")
        for e in elems:
            fp.write(f"{e['name']} {float(e['radius'])!r} {float(e['weight'])!r}\n")
            for b in e["beta"]:
                fp.write(f"{float(b)!r}\n")
    with open(os.path.join(work, case["param"]), "w") as fp:
        for k, v in snap["params"].items():
            fp.write(f"{k} {v}\n")


def read_snap_files(coeff_path: str, param_path: str) -> dict:
    """Parses a one-element .snapcoeff and a .snapparam into numbers."""
    lines = [ln.split("#")[0].split() for ln in open(coeff_path)]
    lines = [ln for ln in lines if ln]
    ncoeff = int(lines[0][1])
    elem, radius, weight = lines[1][0], float(lines[1][1]), float(lines[1][2])
    beta = [float(ln[0]) for ln in lines[2:2 + ncoeff]]
    params = {}
    for ln in open(param_path):
        if "#" in ln or not ln.strip():
            continue
        k, v = ln.split()[:2]
        params[k] = v
    return dict(elem=elem, radius=radius, weight=weight, beta=beta, params=params)


def write_case(case: dict, work: str, snap: dict | None = None) -> tuple[str, list[str]]:
    """Writes the deck (and SNAP files from `snap`) into work/; returns (deck path, args)."""
    deck = os.path.join(work, "in.deck")
    with open(deck, "w") as fp:
        fp.write(deck_text(case))
    if case["kind"] == "snap":
        write_snap_files(work, case, snap)
    return deck, list(case["args"])


# Cases too large for array fixtures: make_golden.py stores SHA-256 digests of
# the reference's dump arrays (in the reference's atom order) and of its
# probe arrays after init, plus its thermo lines, in CASE.digest.json.
DIGEST_CASES = {
    # LJ-32k, the CPU-runnable LJ configuration: fcc 20^3 = 32,000 atoms, CSR
    # full list, newton off, rebuild every 20, thermo every 10, 100 steps
    "lj_fcc20_full_csr": dict(kind="lj", n=20, mass=1.0, temp=1.44, newton="off", every=20, thermo=10, steps=100,
                              args=["--neigh-type", "CSR", "--force-iteration", "NEIGH_FULL", "--comm-type",
                                    "SERIAL"],
                              dump_every=1, keep_steps=[0, 20, 21, 100]),
}


def digest(a) -> str:
    """SHA-256 of an array's bytes (C order, its own dtype)."""
    import hashlib

    import numpy as np
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def snap_w_synthetic(seed: int = 20261203) -> dict:
    """The SNAP-W workload's coefficient set: element W (radius 0.5, weight
    1), beta_0 = -8 and beta_1..55 ~ N(0, 0.1) from `seed`, with the shipped
    W.snapparam values (twojmax 8, rcutfac 4.73442, rfac0 0.99363, rmin0 0)."""
    import numpy as np
    beta = [-8.0] + [float(b) for b in np.random.default_rng(seed).normal(0.0, 0.1, 55)]
    return dict(elem="W", radius=0.5, weight=1.0, beta=beta,
                params={"rcutfac": "4.73442", "twojmax": "8", "rfac0": "0.99363", "rmin0": "0",
                        "diagonalstyle": "3", "bzeroflag": "0", "quadraticflag": "0"})
