"""GB300 LJ path vs the CPU oracle and ExaMiniMD's golden dumps (GPU).

The FP64 drop-in must be bit-identical to the serial reference for the full
list: bins, permutation, ghosts, neighbour rows (entry for entry), forces and
whole trajectories.  Half lists scatter with atomics and are compared to
1e-12 relative.  The mixed form is checked against the FP64 forces at the
tolerances the hot path is specified with (RMS relative force error <= 1e-5).
"""
import math

import numpy as np
import pytest

from tests import mdloop
from tests.golden.decks import CASES

pytestmark = pytest.mark.gpu

LJ_CASES = [k for k, v in CASES.items() if v["kind"] == "lj"]
IDIAL_CASES = [k for k, v in CASES.items() if v["kind"] == "lj_idial"]
MAPCONSTR_CASES = [k for k, v in CASES.items() if v["kind"] == "lj_mapconstr"]


def _ctx():
    from examinimd_gb300 import Context
    return Context(0)


def _rel_err(a, b, floor=1e-300):
    """max |a-b| over max |b|; `floor` bounds the denominator for arrays that
    are zero up to rounding (net forces on a perfect lattice)."""
    return np.abs(a - b).max() / max(np.abs(b).max(), floor)


def _compare_state(gpu, orc, exact: bool, tag: str, ghosts=True):
    nl, ng, _ = orc.info()
    assert gpu.info()[:2] == (nl, ng), tag
    n = nl + (ng if ghosts else 0)
    a, b = gpu.get(0, n), orc.get(0, n)
    for k in ("id", "type"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=f"{tag} {k}")
    if exact:
        for k in ("x", "v"):
            np.testing.assert_array_equal(a[k], b[k], err_msg=f"{tag} {k}")
        np.testing.assert_array_equal(a["f"][:nl], b["f"][:nl], err_msg=f"{tag} f")
    else:
        # atomically scattered half-list sums: 1e-12 relative to the force
        # scale (a unit LJ pair force), not to net forces that cancel to ~1e-14
        for k in ("x", "v"):
            assert _rel_err(a[k], b[k], 1.0) <= 1e-12, f"{tag} {k}"
        assert _rel_err(a["f"][:nl], b["f"][:nl], 1.0) <= 1e-12, f"{tag} f"


@pytest.mark.parametrize("name", LJ_CASES)
def test_lj_modules_vs_oracle(name, golden):
    """Module by module, same call sequence, after init and for 25 steps."""
    from oracle.orc import Oracle
    case = CASES[name]
    setup = mdloop.setup_for_case(name, case)
    state = mdloop.make_lattice(setup)
    gpu, orc = _ctx(), Oracle()
    tg = mdloop.init(gpu, setup, state)
    to = mdloop.init(orc, setup, state)
    assert tg == to
    nl, ng, nt = orc.info()
    nb = tuple(int(v) for v in golden(name)["probe_nbin"][:3])
    for x, y in zip(gpu.binning_get(int(np.prod(nb)), nt), orc.binning_get(int(np.prod(nb)), nt)):
        np.testing.assert_array_equal(x, y)
    cg, pg = gpu.comm_ghosts()
    co, po = orc.comm_ghosts()
    np.testing.assert_array_equal(cg, co)
    np.testing.assert_array_equal(pg, po)
    for x, y in zip(gpu.neigh_get(tg), orc.neigh_get(to)):
        np.testing.assert_array_equal(x, y)
    if setup.kind == 1:
        # the stride may differ from the serial reference's (the GPU reports the
        # largest row, the reference the last overflowing one); it must hold every row
        assert gpu.neigh_maxneighs() >= int(gpu.neigh_get(tg)[0].max())
    exact = not setup.half
    _compare_state(gpu, orc, exact, f"{name} init")
    for s in range(1, 26):
        mdloop.step(gpu, setup, s)
        mdloop.step(orc, setup, s)
        _compare_state(gpu, orc, exact, f"{name} step {s}", ghosts=(s % setup.every == 0))
    eg, eo = setup.energy(gpu), setup.energy(orc)
    assert abs(eg - eo) <= 1e-12 * abs(eo)
    assert abs(gpu.thermo_mv2() - orc.thermo_mv2()) <= 1e-12 * orc.thermo_mv2()


@pytest.mark.parametrize("name", LJ_CASES + IDIAL_CASES)
def test_lj_driver_vs_reference_dumps(name, golden, tmp_path):
    """The re-hosted ExaMiniMD driver (emd_gb300 modules) on the golden deck
    against ExaMiniMD's own --dumpbinary output."""
    from examinimd_gb300 import MD
    from tests.golden.decks import write_case
    g = golden(name)
    case = CASES[name]
    deck, args = write_case(case, str(tmp_path))
    md = MD(["-il", deck, "--quiet"] + args)
    exact = "NEIGH_HALF" not in case["args"]
    keep = [int(s) for s in g["keep_steps"]]
    done = 0
    for s in keep:
        if s > done:
            md.run(s - done)
            done = s
        nl = md.info()["N_local"]
        cur = md.ctx.get(0, nl)
        for k in ("id", "type"):
            np.testing.assert_array_equal(cur[k], g[f"s{s}_{k}"], err_msg=f"{name} step {s} {k}")
        for k in ("x", "v", "f"):
            if exact:
                np.testing.assert_array_equal(cur[k], g[f"s{s}_{k}"], err_msg=f"{name} step {s} {k}")
            else:
                assert _rel_err(cur[k], g[f"s{s}_{k}"], 1.0) <= 1e-12, f"{name} step {s} {k}"
    T, pe, ke = md.thermo(recompute=True)
    last = g["thermo"][-1]
    assert int(last[0]) == done
    np.testing.assert_allclose([T, pe, pe + ke], last[1:], rtol=0, atol=1.5e-6)
    md.close()


@pytest.mark.parametrize("n", [6, 10])
def test_lj_mixed_force_error(n):
    """Mixed form (FP32 pair math, FP64 accumulation) vs FP64 forces."""
    from examinimd_gb300 import EMD_PREC_MIXED
    setup = mdloop.LJSetup(n)
    state = mdloop.make_lattice(setup)
    ref, mix = _ctx(), _ctx()
    mdloop.init(ref, setup, state)
    mdloop.init(mix, setup, state, precision=EMD_PREC_MIXED)
    for s in range(1, 41):
        # drive both from identical positions: copy the FP64 state into the mixed one
        mdloop.step(ref, setup, s)
        mdloop.step(mix, setup, s)
    nl = ref.info()[0]
    fr = ref.get(0, nl)
    fm = mix.get(0, nl)
    np.testing.assert_array_equal(fr["id"], fm["id"])
    # forces at the same configuration: recompute the mixed force on the FP64 positions
    mix2 = _ctx()
    mdloop.init(mix2, setup, {**fr, "q": None}, precision=EMD_PREC_MIXED)
    ref2 = _ctx()
    mdloop.init(ref2, setup, {**fr, "q": None})
    a = ref2.get(0, nl)["f"]
    b = mix2.get(0, nl)["f"]
    err = np.linalg.norm(b - a, axis=1)
    mag = np.linalg.norm(a, axis=1)
    rms_rel = np.sqrt(np.mean(err ** 2)) / np.sqrt(np.mean(mag ** 2))
    max_rel = err.max() / np.sqrt(np.mean(mag ** 2))
    assert rms_rel <= 1e-5, rms_rel
    assert max_rel <= 1e-4, max_rel
    # the interacting pair set is decided in FP64 near the cutoff: energies agree closely
    assert abs(mix2.lj_energy() - ref2.lj_energy()) <= 1e-9 * abs(ref2.lj_energy())
    # 40 steps of mixed dynamics stay close to FP64 dynamics
    assert _rel_err(fm["x"], fr["x"]) <= 1e-6


def test_lj_mixed_pairs_on_the_cutoff():
    """fcc with the cutoff equal to the lattice constant: the second shell
    lies on the cutoff (positions displaced by 1e-7 a), so every row holds
    pairs whose FP32 r^2 falls in the guard band.  They must be decided as
    the FP64 drop-in decides them: one pair decided otherwise moves an atom's
    force by about 0.6, against an RMS force near 1.  The force pass with the
    energy (an FP64 re-test per band pair) and the one without it (FP32
    decisions, the row redone in full when it holds a band pair) give the
    same bits."""
    from examinimd_gb300 import EMD_PREC_MIXED
    a = math.pow(4.0 / 0.8442, 1.0 / 3.0)
    setup = mdloop.LJSetup(8, cut=a, coeffs=[(1, 1, 1.0, 1.0, a)])
    state = dict(mdloop.make_lattice(setup))
    rng = np.random.default_rng(31)
    state["x"] = np.mod(state["x"] + rng.normal(0.0, 1e-7 * a, state["x"].shape), setup.domain[0])
    ref, mix = _ctx(), _ctx()
    mdloop.init(ref, setup, state)
    mdloop.init(mix, setup, state, precision=EMD_PREC_MIXED)
    nl = ref.info()[0]
    fr, fm = ref.get(0, nl)["f"], mix.get(0, nl)["f"]
    rms = np.sqrt(np.mean(np.sum(fr * fr, axis=1)))
    assert rms > 0.1  # the shell is split: some pairs in, some out
    err = np.linalg.norm(fm - fr, axis=1)
    assert err.max() <= 1e-4 * rms, (err.max(), rms)
    mix.zero_forces()
    mix.lj_request_energy()
    mix.lj_compute()
    np.testing.assert_array_equal(mix.get(0, nl)["f"], fm)
    pe = mix.lj_force_energy()
    assert pe is not None and abs(pe - ref.lj_energy()) <= 1e-11 * abs(ref.lj_energy())


@pytest.mark.parametrize("kind,newton", [(0, False), (0, True), (1, True)])
def test_lj_mixed_half_list(kind, newton):
    """NEIGH_HALF in the mixed form (force_lj_neigh_impl.h:211-254): every
    pair once, its FP32 force added to i and scattered to j with FP64 atomics
    (folded back from the ghosts with newton on).  Forces within the mixed
    tolerance of the FP64 half form on the same positions, the energy over
    the packed half rows equal to the FP64 form's to 1e-12, and 20 steps
    across a rebuild close to the FP64 trajectory."""
    from examinimd_gb300 import EMD_PREC_MIXED
    setup = mdloop.LJSetup(6, kind=kind, half=True, newton=newton)
    state = dict(mdloop.make_lattice(setup))
    rng = np.random.default_rng(7)
    state["x"] = np.mod(state["x"] + rng.normal(0.0, 0.03, state["x"].shape), setup.domain[0])
    ref, mix = _ctx(), _ctx()
    mdloop.init(ref, setup, state)
    mdloop.init(mix, setup, state, precision=EMD_PREC_MIXED)
    nl = ref.info()[0]
    a, b = ref.get(0, nl), mix.get(0, nl)
    np.testing.assert_array_equal(a["id"], b["id"])
    err = np.linalg.norm(b["f"] - a["f"], axis=1)
    scale = np.sqrt(np.mean(np.sum(a["f"] ** 2, axis=1)))
    assert np.sqrt(np.mean(err ** 2)) <= 1e-5 * scale, np.sqrt(np.mean(err ** 2)) / scale
    assert err.max() <= 1e-4 * scale
    assert abs(mix.lj_energy() - ref.lj_energy()) <= 1e-12 * abs(ref.lj_energy())
    assert mix.lj_energy_mixed() is None  # the mixed energy kernel covers full lists
    for s in range(1, 21):
        mdloop.step(ref, setup, s)
        mdloop.step(mix, setup, s)
    a, b = ref.get(0, nl), mix.get(0, nl)
    np.testing.assert_array_equal(a["id"], b["id"])
    assert _rel_err(b["x"], a["x"]) <= 1e-6
    assert mix.status() == 0


def test_lj_many_types_per_pair_parameters():
    """13 types: above ExaMiniMD's 12-type stack-parameter limit, so every
    type pair keeps its own eps / sigma (force_lj_neigh_impl.h:75-98).  The
    FP64 drop-in matches the oracle bit for bit; the mixed form (per-pair
    FP32 tables) stays within 1e-4 RMS of it after 24 steps, trajectory
    divergence included."""
    from oracle.orc import Oracle
    rng = np.random.default_rng(13)
    coeffs = []
    for a in range(1, 14):
        for b in range(a, 14):
            coeffs.append((a, b, float(rng.uniform(0.8, 1.2)), float(rng.uniform(0.9, 1.05)), 2.5))
    setup = mdloop.LJSetup(5, masses=list(rng.uniform(0.8, 2.0, 13)), coeffs=coeffs)
    state = mdloop.make_lattice(setup)
    assert len(np.unique(state["type"])) > 10
    gpu, orc, mix = _ctx(), Oracle(), _ctx()
    assert mdloop.init(gpu, setup, state) == mdloop.init(orc, setup, state)
    mdloop.init(mix, setup, state, precision=1)
    for s in range(1, 25):
        for b in (gpu, orc, mix):
            mdloop.step(b, setup, s)
    _compare_state(gpu, orc, True, "13 types")
    nl = orc.info()[0]
    fa, fb = mix.get(0, nl)["f"], orc.get(0, nl)["f"]
    err = np.linalg.norm(fa - fb, axis=1)
    assert np.sqrt(np.mean(err ** 2)) / np.sqrt(np.mean(np.sum(fb ** 2, axis=1))) <= 1e-4


def test_lj_mixed_on_2d_lists():
    """The mixed form reads the same packed rows whichever list kind the
    deck asks for: Neighbor2D rows give the CSR rows' forces bit for bit."""
    from examinimd_gb300 import EMD_PREC_MIXED
    forces = []
    for kind in (0, 1):
        setup = mdloop.LJSetup(6, kind=kind)
        state = mdloop.make_lattice(setup)
        rng = np.random.default_rng(2)
        state["x"] = np.mod(state["x"] + rng.normal(0, 0.03, state["x"].shape), setup.domain[0])
        c = _ctx()
        mdloop.init(c, setup, state, precision=EMD_PREC_MIXED)
        for s in range(1, 23):  # across a rebuild
            mdloop.step(c, setup, s)
        nl = c.info()[0]
        forces.append(c.get(0, nl))
        c.close()
    np.testing.assert_array_equal(forces[0]["id"], forces[1]["id"])
    for k in ("x", "v", "f"):
        np.testing.assert_array_equal(forces[0][k], forces[1][k])


@pytest.mark.parametrize("half,precision,rho", [(False, 0, 0.8442), (True, 0, 0.8442), (False, 1, 0.8442),
                                                (False, 1, 2.0), (True, 0, 2.0), (True, 1, 0.8442)])
def test_neighbour_rows_on_a_random_gas(half, precision, rho):
    """Uniform random positions (no lattice order; at rho 2 a bin holds about
    40 atoms, more than one warp's lanes): bins, ghosts and every neighbour row
    entry for entry against the oracle.  The build drops staged candidates
    beyond the cutoff from its centre atoms' bounding box and decides pairs in
    FP32 outside a guard band; rows must still equal the FP64 reference's."""
    from oracle.orc import Oracle
    setup = mdloop.LJSetup(8, half=half, rho=rho)
    state = dict(mdloop.make_lattice(setup))
    rng = np.random.default_rng(20261205)
    state["x"] = rng.uniform(0.0, 1.0, state["x"].shape) * np.array(setup.domain)
    gpu, orc = _ctx(), Oracle()
    tg = mdloop.init(gpu, setup, state, precision=precision)
    to = mdloop.init(orc, setup, state)
    assert tg == to
    cg, pg = gpu.comm_ghosts()
    co, po = orc.comm_ghosts()
    np.testing.assert_array_equal(cg, co)
    np.testing.assert_array_equal(pg, po)
    for x, y in zip(gpu.neigh_get(tg), orc.neigh_get(to)):
        np.testing.assert_array_equal(x, y)


@pytest.mark.parametrize("kind,precision", [(1, 0), (0, 1)])
def test_neighbour_get_after_a_build_without_the_total(kind, precision):
    """Column-major rows (2D, or the mixed form's packed rows) built again
    from the same binning with no total requested, as the driver builds them:
    the count is read when the rows are fetched, and the rows equal the first
    build's.  In the mixed form the first build handed the binning's FP32
    offsets to the force, so the second rebuilds them from the positions."""
    setup = mdloop.LJSetup(6, kind=kind)
    state = mdloop.make_lattice(setup)
    ref, lazy = _ctx(), _ctx()
    total = mdloop.init(ref, setup, state, precision=precision)
    mdloop.init(lazy, setup, state, precision=precision)
    assert lazy.lib.emd_neigh_create(lazy.h, 0, None) == 0
    num, ent = lazy.neigh_get(2 * total)  # room for any count; the rows are compared below
    rnum, rent = ref.neigh_get(total)
    np.testing.assert_array_equal(num, rnum)
    assert int(num.sum()) == total
    np.testing.assert_array_equal(ent[:total], rent)


@pytest.mark.parametrize("name", MAPCONSTR_CASES)
def test_mapconstr_driver_vs_reference_dumps(name, golden, tmp_path):
    """--neigh-type CSR_MAPCONSTR: ExaMiniMD builds the CSR pairs through a
    hash set (neighbor_csr_map_constr.h), so its rows list the neighbours in
    the hash map's order; the GB300 module builds the same rows in stencil
    order.  The neighbour sets after init equal the reference's, and the
    trajectory agrees with its dumps to 1e-12 (the same pairs summed in
    another order)."""
    from examinimd_gb300 import MD
    from tests.golden.decks import write_case
    g = golden(name)
    case = CASES[name]
    deck, args = write_case(case, str(tmp_path))
    md = MD(["-il", deck, "--quiet"] + args)
    num, ent = md.ctx.neigh_get()
    np.testing.assert_array_equal(num, g["probe_num_neighs"])
    off, roff = np.concatenate([[0], np.cumsum(num)]), np.concatenate([[0], np.cumsum(g["probe_num_neighs"])])
    for i in range(len(num)):
        np.testing.assert_array_equal(np.sort(ent[off[i]:off[i + 1]]),
                                      np.sort(g["probe_neighs"][roff[i]:roff[i + 1]]), err_msg=f"row {i}")
    done = 0
    for s in [int(v) for v in g["keep_steps"]]:
        if s > done:
            md.run(s - done)
            done = s
        nl = md.info()["N_local"]
        cur = md.ctx.get(0, nl)
        np.testing.assert_array_equal(cur["id"], g[f"s{s}_id"])
        for k in ("x", "v", "f"):
            assert _rel_err(cur[k], g[f"s{s}_{k}"], 1.0) <= 1e-12, f"{name} step {s} {k}"
    md.close()
