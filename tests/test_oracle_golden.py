"""Pins the CPU oracle to ExaMiniMD's own outputs (CPU only).

Every golden fixture was produced by ExaMiniMD's unmodified sources (built
against the serial Kokkos shim): the reference's binning, ghosts, neighbour
rows and initial forces right after init, its --dumpbinary state at selected
steps and its thermo lines.  The oracle restatement must reproduce all of
them bit for bit (thermo to the printed precision).
"""
import numpy as np
import pytest

from oracle.orc import Oracle
from tests import mdloop
from tests.golden.decks import CASES

# the intensity-dial LJ style has no oracle restatement: its fixtures pin the
# GB300 driver directly (tests/test_gpu_lj.py)
ORACLE_CASES = [k for k, v in CASES.items() if v["kind"] not in ("lj_idial", "lj_mapconstr")]


@pytest.mark.parametrize("name", ORACLE_CASES)
def test_oracle_matches_reference_init(name, golden):
    g = golden(name)
    case = CASES[name]
    setup = mdloop.setup_for_case(name, case, g)
    o = Oracle()
    state = mdloop.make_lattice(setup)
    mdloop.init(o, setup, state)
    nl, ng, nt = o.info()
    assert (nl, ng) == tuple(g["probe_counts"])
    # binning of owned + ghost particles (binning.h:50-59)
    nb = tuple(g["probe_nbin"][:3])
    bc, bo, perm, bounds = o.binning_get(int(np.prod(nb)), nt)
    np.testing.assert_array_equal(bc, g["probe_bincount"])
    np.testing.assert_array_equal(bo, g["probe_binoffsets"])
    np.testing.assert_array_equal(perm, g["probe_permute"])
    np.testing.assert_array_equal(bounds, g["probe_bounds"])
    # every particle, ghosts included, in the reference's order
    allp = o.get(0, nt)
    np.testing.assert_array_equal(allp["x"].ravel(), g["probe_x"])
    np.testing.assert_array_equal(allp["id"], g["probe_id"])
    np.testing.assert_array_equal(allp["type"], g["probe_type"])
    # neighbour rows in the reference's order
    total = int(g["probe_num_neighs"].sum())
    num, ent = o.neigh_get(total)
    np.testing.assert_array_equal(num, g["probe_num_neighs"])
    np.testing.assert_array_equal(ent, g["probe_neighs"])
    if "probe_maxneighs" in g.files:
        assert o.neigh_maxneighs() == int(g["probe_maxneighs"][0])
    # initial forces of the owned atoms
    np.testing.assert_array_equal(allp["f"][:nl].ravel(), g["probe_f"][:3 * nl])


@pytest.mark.parametrize("name", ORACLE_CASES)
def test_oracle_matches_reference_run(name, golden):
    g = golden(name)
    case = CASES[name]
    setup = mdloop.setup_for_case(name, case, g)
    o = Oracle()
    state = mdloop.make_lattice(setup)
    mdloop.init(o, setup, state)
    keep = list(g["keep_steps"])
    thermo_ref = {int(r[0]): r[1:] for r in g["thermo"]}
    nl, _, _ = o.info()
    for s in range(0, max(keep) + 1):
        if s > 0:
            mdloop.step(o, setup, s)
        if s in keep:
            cur = o.get(0, nl)
            for k in ("id", "type", "x", "v", "f"):
                np.testing.assert_array_equal(cur[k], g[f"s{s}_{k}"], err_msg=f"{name} step {s} field {k}")
        if s in thermo_ref:
            if case["kind"] == "snap":
                # ExaMiniMD has no SNAP energy (force.h:54 returns 0): only T is comparable
                T = o.thermo_mv2() * (setup.mvv2e / (1.0 * (3 * nl - 3) * setup.boltz))
                assert thermo_ref[s][1] == 0.0
                np.testing.assert_allclose(T, thermo_ref[s][0], rtol=0, atol=1.5e-6)
            else:
                T, pe, et = mdloop.thermo(o, setup, nl)
                np.testing.assert_allclose([T, pe, et], thermo_ref[s], rtol=0, atol=1.5e-6,
                                           err_msg=f"{name} thermo step {s}")


def test_oracle_matches_reference_lj32k_digests():
    """LJ-32k (fcc 20^3, CSR full, newton off, every 20, 100 steps): the
    oracle's bins, permutation, particles, neighbour rows and forces after
    init, and its owned state at steps 0, 20, 21 and 100, carry exactly the
    bytes of ExaMiniMD's probe and --dumpbinary output (SHA-256 digests);
    thermo to the printed precision."""
    import json
    import os

    from tests.golden.decks import DIGEST_CASES, digest
    name = "lj_fcc20_full_csr"
    case = DIGEST_CASES[name]
    with open(os.path.join(os.path.dirname(__file__), "golden", f"{name}.digest.json")) as fp:
        D = json.load(fp)
    setup = mdloop.setup_for_case(name, case)
    o = Oracle(os.cpu_count() or 1)
    mdloop.init(o, setup, mdloop.make_lattice(setup))
    nl, ng, nt = o.info()
    assert [nl, ng] == D["probe_counts"]
    nb = int(np.prod(D["probe_nbin"][:3]))
    bc, bo, perm, bounds = o.binning_get(nb, nt)
    for k, v in (("bincount", bc), ("binoffsets", bo), ("permute", perm), ("bounds", bounds)):
        assert digest(v) == D["probe"][k], k
    allp = o.get(0, nt)
    for k in ("x", "v", "id", "type"):
        assert digest(allp[k].ravel()) == D["probe"][k], k
    num, ent = o.neigh_get()
    assert digest(num) == D["probe"]["num_neighs"] and digest(ent) == D["probe"]["neighs"]
    thermo_ref = {int(r[0]): r[1:] for r in D["thermo"]}
    for s in range(0, case["steps"] + 1):
        if s > 0:
            mdloop.step(o, setup, s)
        if str(s) in D["steps"]:
            cur = o.get(0, nl)
            for k in ("id", "type", "q", "x", "v", "f"):
                assert digest(cur[k]) == D["steps"][str(s)][k], f"step {s} field {k}"
        if s in thermo_ref:
            np.testing.assert_allclose(mdloop.thermo(o, setup, nl), thermo_ref[s], rtol=0, atol=1.5e-6)


def _sorted_rows(num, ent):
    off = np.concatenate([[0], np.cumsum(num)])
    return [np.sort(ent[off[i]:off[i + 1]]) for i in range(len(num))]


def test_oracle_matches_reference_mapconstr_sets():
    """CSR_MAPCONSTR (neighbor_csr_map_constr.h) builds the CSR pairs through a
    hash set, so its rows list the same neighbours in the hash map's order.
    The restatement's stencil-order rows must hold exactly the reference's
    sets; bins and ghosts are the CSR build's, and the run agrees to 1e-12
    (the per-atom force sums add the same pairs in another order)."""
    name = "lj_fcc4_full_csrmap"
    g = golden_load(name)
    case = CASES[name]
    setup = mdloop.setup_for_case(name, case)
    o = Oracle()
    total = mdloop.init(o, setup, mdloop.make_lattice(setup))
    nl, ng, nt = o.info()
    assert (nl, ng) == tuple(g["probe_counts"])
    num, ent = o.neigh_get(total)
    np.testing.assert_array_equal(num, g["probe_num_neighs"])
    for a, b in zip(_sorted_rows(num, ent), _sorted_rows(g["probe_num_neighs"], g["probe_neighs"])):
        np.testing.assert_array_equal(a, b)
    for s in range(0, max(case["keep_steps"]) + 1):
        if s > 0:
            mdloop.step(o, setup, s)
        if s in case["keep_steps"]:
            cur = o.get(0, nl)
            np.testing.assert_array_equal(cur["id"], g[f"s{s}_id"])
            for k in ("x", "v", "f"):
                ref = g[f"s{s}_{k}"]
                assert np.abs(cur[k] - ref).max() <= 1e-12 * max(np.abs(ref).max(), 1.0), (s, k)


def golden_load(name):
    import os
    return np.load(os.path.join(os.path.dirname(__file__), "golden", f"{name}.npz"))
