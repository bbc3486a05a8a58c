"""ExaMiniMD's init + timestep sequence (examinimd.cpp:60-276) over a backend.

A backend is anything with the Context method set: the GB300 library
(examinimd_gb300.Context) or the CPU oracle (oracle.orc.Oracle).  Tests run
the same sequence on both and compare the state between calls.
"""
from __future__ import annotations

import math

import numpy as np


class Setup:
    """Deck parameters common to LJ and SNAP runs."""
    lattice_style = 1  # 0 sc, 1 fcc, 2 bcc
    boltz, mvv2e = 1.0, 1.0

    def __init__(self, n, mass, temp, seed, cut, skin, every, newton, half, kind, a, dt, ny=None, nz=None):
        self.nx, self.ny, self.nz = n, (ny or n), (nz or n)
        self.mass, self.temp, self.seed = mass, temp, seed
        self.cut, self.skin, self.every = cut, skin, every
        self.newton, self.half, self.kind = newton, half, kind
        self.a, self.dt = a, dt
        self.neigh_cut = cut + skin
        self.masses = [mass]  # per type

    @property
    def domain(self):
        return [self.a * self.nx, self.a * self.ny, self.a * self.nz]

    def force_init(self, b, precision=0):
        raise NotImplementedError

    def force_compute(self, b):
        raise NotImplementedError

    def energy(self, b):
        raise NotImplementedError


class LJSetup(Setup):
    """fcc LJ deck (in.lj style; lattice constant (4/rho)^(1/3), input.cpp:311-323)."""

    def __init__(self, n, mass=1.0, temp=1.44, seed=87287, cut=2.5, skin=0.3, every=20, newton=False, half=False,
                 kind=0, rho=0.8442, dt=0.005, masses=None, coeffs=None):
        super().__init__(n, mass, temp, seed, cut, skin, every, newton, half, kind, math.pow(4.0 / rho, 1.0 / 3.0), dt)
        self.masses = list(masses) if masses else [mass]
        nt = len(self.masses)
        # pair_coeff lines (t1, t2, eps, sigma, cut); with at most 12 types
        # ForceLJNeigh keeps stack parameters and every pair_coeff line
        # overwrites all pairs, so the last line holds (force_lj_neigh_impl.h:67-74)
        coeffs = coeffs or [(1, 1, 1.0, 1.0, cut)]
        lj1, lj2, cutsq = np.zeros((nt, nt)), np.zeros((nt, nt)), np.zeros((nt, nt))
        for t1, t2, eps, sig, c in coeffs:
            if nt <= 12:
                lj1[:], lj2[:], cutsq[:] = 48.0 * eps * math.pow(sig, 12.0), 24.0 * eps * math.pow(sig, 6.0), c * c
            else:
                lj1[t1 - 1, t2 - 1] = lj1[t2 - 1, t1 - 1] = 48.0 * eps * math.pow(sig, 12.0)
                lj2[t1 - 1, t2 - 1] = lj2[t2 - 1, t1 - 1] = 24.0 * eps * math.pow(sig, 6.0)
                cutsq[t1 - 1, t2 - 1] = cutsq[t2 - 1, t1 - 1] = c * c
        self.lj1, self.lj2, self.cutsq = lj1.ravel(), lj2.ravel(), cutsq.ravel()

    def force_init(self, b, precision=0):
        b.lj_init(self.lj1, self.lj2, self.cutsq, half=self.half, precision=precision)

    def force_compute(self, b):
        b.lj_compute()

    def energy(self, b):
        return b.lj_energy()


class SnapSetup(Setup):
    """SNAP deck in metal units (in.snap.W style); sc by default, bcc optional."""
    boltz, mvv2e = 8.617343e-5, 1.0364269e-4

    def __init__(self, nx, ny, nz, snap: dict, a=3.1803, mass=183.84, temp=300.0, seed=4928459, skin=1.0, every=1,
                 lattice_style=0, dt=0.001, kind=0, masses=None, type_elems=None):
        elems = snap["elements"] if "elements" in snap else [
            dict(name=snap["elem"], radius=snap["radius"], weight=snap["weight"], beta=snap["beta"])]
        # ExaMiniMD's read_files deep-copies each element's radius and weight
        # into the whole radelem / wjelem views (force_snap_neigh_impl.h:458-461):
        # every element ends with the values of the last one read
        elems = [dict(e, radius=elems[-1]["radius"], weight=elems[-1]["weight"]) for e in elems]
        # force cutoff: the largest 2 radelem rcutfac (force_snap_neigh_impl.h:327-333)
        cut = max(2.0 * float(e["radius"]) * float(snap["params"]["rcutfac"]) for e in elems)
        super().__init__(nx, mass, temp, seed, cut, skin, every, True, False, kind, a, dt, ny, nz)
        self.elements = elems
        self.masses = list(masses) if masses else [mass]
        names = [e["name"] for e in elems]
        nt = len(self.masses)
        type_elems = type_elems or [names[0]] * nt
        # ExaMiniMD fills map[1..ntypes] from the element names and reads
        # map[type] with 0-based types (force_snap_neigh_impl.h:294-306, 598):
        # type 0 gets element 0, type t >= 1 the element named for type t
        self.type_map = [0] + [names.index(type_elems[t - 1]) for t in range(1, nt)]
        self.lattice_style = lattice_style
        self.snap = snap
        p = snap["params"]
        self.twojmax = int(p["twojmax"])
        self.rcutfac = float(p["rcutfac"])
        self.rfac0 = float(p.get("rfac0", 0.99363))
        self.rmin0 = float(p.get("rmin0", 0.0))
        self.switchflag = int(p.get("switchflag", 1))

    def force_init(self, b, precision=0):
        elems = self.elements
        b.snap_init(self.twojmax, self.rfac0, self.rmin0, self.switchflag, self.rcutfac,
                    [e["radius"] for e in elems], [e["weight"] for e in elems],
                    np.asarray([e["beta"] for e in elems], float), self.type_map, precision=precision)

    def force_compute(self, b):
        b.snap_compute()

    def energy(self, b):
        return b.snap_energy()


def make_lattice(setup: Setup, threads=1):
    """Initial owned particles from the oracle's Input::create_lattice restatement."""
    from oracle.orc import Oracle
    o = Oracle(threads)
    o.system_init(setup.masses, setup.boltz, setup.mvv2e, setup.dt, setup.domain)
    o.create_lattice(setup.lattice_style, setup.a, setup.nx, setup.ny, setup.nz, setup.temp, setup.seed)
    return o.get()


def init(b, setup: Setup, state: dict, precision=0):
    """ExaMiniMD::init from the lattice on (examinimd.cpp:120-144)."""
    b.system_init(setup.masses, setup.boltz, setup.mvv2e, setup.dt, setup.domain)
    b.set_local(state["x"], state["type"], state["id"], v=state["v"], q=state.get("q"))
    setup.force_init(b, precision)
    b.comm_init(setup.neigh_cut)
    b.neigh_init(setup.kind, setup.neigh_cut, setup.newton)
    c = setup.neigh_cut
    b.comm_exchange()
    b.binning_create(c, c, c, 1, True, False, True)
    b.comm_exchange_halo()
    b.binning_create(c, c, c, 1, True, True, False)
    total = b.neigh_create(setup.half)
    b.zero_forces()
    setup.force_compute(b)
    if setup.newton:
        b.comm_update_force()
    return total


def step(b, setup: Setup, step_no: int):
    """One pass of the ExaMiniMD::run loop body (examinimd.cpp:192-276)."""
    c = setup.neigh_cut
    b.nve_initial()
    if step_no % setup.every == 0:
        b.comm_exchange()
        b.binning_create(c, c, c, 1, True, False, True)
        b.comm_exchange_halo()
        b.binning_create(c, c, c, 1, True, True, False)
        b.neigh_create(setup.half)
    else:
        b.comm_update_halo()
    b.zero_forces()
    setup.force_compute(b)
    if setup.newton:
        b.comm_update_force()
    b.nve_final()


def thermo(b, setup: Setup, natoms: int):
    """T, PE/N, ETot/N as printed by ExaMiniMD (examinimd.cpp:252-267)."""
    mv2 = b.thermo_mv2()
    T = mv2 * (setup.mvv2e / (1.0 * (3 * natoms - 3) * setup.boltz))
    pe = setup.energy(b) / natoms
    ke = mv2 * (0.5 * setup.mvv2e) / natoms
    return T, pe, pe + ke


def by_id(state: dict) -> dict:
    """Rows sorted by atom id (the correctness check's matching, examinimd.cpp:397-408)."""
    order = np.argsort(state["id"], kind="stable")
    return {k: v[order] for k, v in state.items()}


def rows(num, ent):
    off = np.concatenate([[0], np.cumsum(num)])
    return [ent[off[i]:off[i + 1]] for i in range(len(num))]


def golden_snap(g) -> dict:
    """SNAP file numbers stored in a golden fixture."""
    out = dict(elem=str(g["snap_elem"]), radius=float(g["snap_radius"]), weight=float(g["snap_weight"]),
               beta=list(g["snap_beta"]), params=dict(zip([str(k) for k in g["snap_param_keys"]],
                                                          [str(v) for v in g["snap_param_vals"]])))
    if "snap_elems" in g.files and len(g["snap_elems"]) > 1:
        out["elements"] = [dict(name=str(n), radius=float(r), weight=float(w), beta=list(b))
                           for n, r, w, b in zip(g["snap_elems"], g["snap_radii"], g["snap_weights"],
                                                 g["snap_betas"])]
    return out


def setup_for_case(name: str, case: dict, g=None) -> Setup:
    if case["kind"] in ("lj", "lj_mapconstr"):
        return LJSetup(case["n"], mass=case["mass"], temp=case["temp"], every=case["every"],
                       newton=case["newton"] == "on", half="NEIGH_HALF" in case["args"],
                       kind=1 if "2D" in case["args"] else 0, masses=case.get("masses"), coeffs=case.get("coeffs"))
    return SnapSetup(case["nx"], case["ny"], case["nz"], golden_snap(g), a=case["a"], mass=case["mass"],
                     every=case["every"], kind=1 if "2D" in case["args"] else 0, masses=case.get("masses"),
                     type_elems=case.get("type_elems"))
