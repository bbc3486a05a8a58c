"""Parity on the benchmark configurations themselves (GPU).

* LJ-32k (fcc 20^3 = 32,000 atoms, CSR full list, newton off, rebuild every
  20, thermo every 10, 100 steps): the re-hosted driver's owned particles at
  steps 0, 20, 21 and 100 carry the same bytes as ExaMiniMD's own
  --dumpbinary files (SHA-256 digests in tests/golden/lj_fcc20_full_csr.
  digest.json); module by module against the oracle, bins, ghosts, neighbour
  rows and the whole particle state are bit-identical at the same steps, and
  the thermo values agree to 1e-12 (PE against a compensated sum of the
  reference's pair terms: its own serial sum rounds at ~1e-11 here).
* LJ-4M in the FP64 drop-in (fcc 100^3 = 4,000,000 atoms), 25 steps across
  one rebuild, against the OpenMP oracle: neighbour rows after init and the
  owned x, v, f after step 25, bit for bit.
* SNAP-W geometry (bcc tungsten, the synthetic 2J = 8 coefficient set, newton
  on, rebuild every step) at 6^3 and 8^3 cells against the oracle: forces
  within 1e-12 of the RMS force, positions and velocities within 1e-12 of
  their own scale, at every step.
"""
import json
import os

import numpy as np
import pytest

from tests import mdloop
from tests.golden.decks import DIGEST_CASES, digest, snap_w_synthetic, write_case

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def _ctx():
    from examinimd_gb300 import Context
    return Context(0)


def _load_digests(name):
    with open(os.path.join(HERE, "golden", f"{name}.digest.json")) as fp:
        return json.load(fp)


def test_lj32k_driver_matches_reference_dump_digests(tmp_path):
    """The emd_gb300 driver on the LJ-32k deck: id, type, q, x, v, f of the
    owned atoms, in atom order, byte for byte the reference's dumps."""
    from examinimd_gb300 import MD
    name = "lj_fcc20_full_csr"
    case, D = DIGEST_CASES[name], _load_digests(name)
    deck, args = write_case(case, str(tmp_path))
    md = MD(["-il", deck, "--quiet"] + args)
    done = 0
    for s in case["keep_steps"]:
        if s > done:
            md.run(s - done)
            done = s
        nl = md.info()["N_local"]
        assert nl == D["probe_counts"][0]
        cur = md.ctx.get(0, nl)
        for k in ("id", "type", "q", "x", "v", "f"):
            assert digest(cur[k]) == D["steps"][str(s)][k], f"step {s} field {k}"
    T, pe, ke = md.thermo(recompute=True)
    last = D["thermo"][-1]
    assert int(last[0]) == done
    np.testing.assert_allclose([T, pe, pe + ke], last[1:], rtol=0, atol=1.5e-6)
    md.close()


def test_lj32k_modules_vs_oracle():
    """Module by module on LJ-32k: bins, ghosts and rows at every rebuild,
    the particle state at steps 0, 20, 21 and 100 bit for bit, and T, PE and
    ETot every 10 steps to 1e-12 relative."""
    from oracle.orc import Oracle
    setup = mdloop.LJSetup(20)
    state = mdloop.make_lattice(setup)
    gpu, orc = _ctx(), Oracle(os.cpu_count() or 1)
    tg, to = mdloop.init(gpu, setup, state), mdloop.init(orc, setup, state)
    assert tg == to == _load_digests("lj_fcc20_full_csr")["neigh_total"]
    nb = 13 ** 3

    def same_build(tag, total=None):
        nl, ng, nt = orc.info()
        assert gpu.info()[:2] == (nl, ng), tag
        for x, y in zip(gpu.binning_get(nb, nt), orc.binning_get(nb, nt)):
            np.testing.assert_array_equal(x, y, err_msg=tag)
        for x, y in zip(gpu.comm_ghosts(), orc.comm_ghosts()):
            np.testing.assert_array_equal(x, y, err_msg=tag)
        for x, y in zip(gpu.neigh_get(total), orc.neigh_get(total)):
            np.testing.assert_array_equal(x, y, err_msg=tag)

    def same_state(tag, ghosts):
        nl, ng, _ = orc.info()
        n = nl + (ng if ghosts else 0)
        a, b = gpu.get(0, n), orc.get(0, n)
        for k in ("id", "type", "x", "v"):
            np.testing.assert_array_equal(a[k], b[k], err_msg=f"{tag} {k}")
        np.testing.assert_array_equal(a["f"][:nl], b["f"][:nl], err_msg=f"{tag} f")

    def same_thermo(tag):
        # T from the same velocities; PE: the GPU sums per atom and then in
        # a fixed tree, ExaMiniMD adds its 3.5 million pair terms one after
        # another into one double, which carries ~1e-11 relative rounding at
        # this size.  So PE is held to 1e-12 of the oracle's compensated sum
        # of the same terms, and to the serial sum within the recursive-sum
        # error bound (terms x unit roundoff ~ 1e-9 relative).
        n = orc.info()[0]
        mv_g, mv_o = gpu.thermo_mv2(), orc.thermo_mv2()
        assert abs(mv_g - mv_o) <= 1e-12 * mv_o, (tag, mv_g, mv_o)
        pe_g, pe_exact, pe_serial = gpu.lj_energy(), orc.lj_energy_compensated(), orc.lj_energy()
        assert abs(pe_g - pe_exact) <= 1e-12 * abs(pe_exact), (tag, pe_g, pe_exact)
        assert abs(pe_serial - pe_exact) <= 1e-9 * abs(pe_exact), (tag, pe_serial, pe_exact)
        tg_ = mdloop.thermo(gpu, setup, n)
        assert abs(tg_[2] - (pe_exact + 0.5 * setup.mvv2e * mv_o) / n) <= 1e-12 * abs(tg_[2]), tag

    same_build("init", tg)
    same_state("init", True)
    same_thermo("step 0")
    for s in range(1, 101):
        mdloop.step(gpu, setup, s)
        mdloop.step(orc, setup, s)
        if s % setup.every == 0:
            same_build(f"step {s}")
        if s in (20, 21, 100):
            same_state(f"step {s}", s % setup.every == 0)
        if s % 10 == 0:
            same_thermo(f"step {s}")


def test_lj4m_fp64_vs_openmp_oracle():
    """LJ-4M, FP64 drop-in, 25 steps with one rebuild: neighbour rows after
    init and the owned state after step 25 equal the oracle's bit for bit."""
    from oracle.orc import Oracle
    threads = os.cpu_count() or 1
    setup = mdloop.LJSetup(100)
    state = mdloop.make_lattice(setup, threads)
    gpu, orc = _ctx(), Oracle(threads)
    tg, to = mdloop.init(gpu, setup, state), mdloop.init(orc, setup, state)
    assert tg == to
    assert gpu.info()[:2] == orc.info()[:2]
    ng_, eg = gpu.neigh_get(tg)
    no_, eo = orc.neigh_get(to)
    np.testing.assert_array_equal(ng_, no_)
    assert digest(eg) == digest(eo)
    del eg, eo
    for s in range(1, 26):
        mdloop.step(gpu, setup, s)
        mdloop.step(orc, setup, s)
        if s == 20:
            nl, ng, _ = orc.info()
            assert gpu.info()[:2] == (nl, ng)
            a, b = gpu.get(0, nl + ng, fields=("x", "id")), orc.get(0, nl + ng, fields=("x", "id"))
            np.testing.assert_array_equal(a["id"], b["id"])
            assert digest(a["x"]) == digest(b["x"])
    nl = orc.info()[0]
    a, b = gpu.get(0, nl), orc.get(0, nl)
    for k in ("id", "x", "v", "f"):
        assert digest(a[k]) == digest(b[k]), k


def _snap_w_setup(cells):
    return mdloop.SnapSetup(cells, cells, cells, snap_w_synthetic(), a=3.1803, mass=183.84, temp=300.0,
                            seed=4928459, skin=1.0, every=1, lattice_style=2, dt=0.0005)


def _rms(f):
    return float(np.sqrt(np.mean(np.sum(f * f, axis=1))))


def _snap_compare(gpu, orc, tag):
    nl = orc.info()[0]
    a, b = gpu.get(0, nl), orc.get(0, nl)
    np.testing.assert_array_equal(a["id"], b["id"], err_msg=tag)
    scale = _rms(b["f"])
    err = np.abs(a["f"] - b["f"]).max()
    for k in ("x", "v"):
        assert np.abs(a[k] - b[k]).max() <= 1e-12 * np.abs(b[k]).max(), (tag, k)
    return err, scale


@pytest.mark.parametrize("cells,steps", [(6, 6)])
def test_snap_w_bcc_deck_vs_oracle(cells, steps):
    """The SNAP-W deck at 6^3 cells (432 atoms): perfect bcc lattice, 300 K
    loop-geom velocities, dt 0.5 fs, neighbour rebuild every step.  On the
    perfect lattice (step 0) every force cancels by symmetry in both codes;
    from step 1 on, forces agree to 1e-12 of the step's RMS force."""
    from oracle.orc import Oracle
    setup = _snap_w_setup(cells)
    state = mdloop.make_lattice(setup)
    gpu, orc = _ctx(), Oracle()
    mdloop.init(gpu, setup, state)
    mdloop.init(orc, setup, state)
    err, scale = _snap_compare(gpu, orc, "step 0")
    assert scale <= 1e-10 and err <= 1e-10, (err, scale)
    for s in range(1, steps + 1):
        mdloop.step(gpu, setup, s)
        mdloop.step(orc, setup, s)
        err, scale = _snap_compare(gpu, orc, f"step {s}")
        assert scale > 1e-4 and err <= 1e-12 * scale, (s, err, scale)


@pytest.mark.parametrize("cells,steps", [(8, 3)])
def test_snap_w_bcc_displaced_vs_oracle(cells, steps):
    """SNAP-W at 8^3 cells (1,024 atoms) with positions displaced by a
    seeded 0.05 A Gaussian, so every force is of order 1 eV/A: forces within
    1e-12 of the RMS force at every step."""
    from oracle.orc import Oracle
    setup = _snap_w_setup(cells)
    state = dict(mdloop.make_lattice(setup))
    rng = np.random.default_rng(20261203)
    state["x"] = state["x"] + rng.normal(0.0, 0.05, state["x"].shape)
    gpu, orc = _ctx(), Oracle()
    mdloop.init(gpu, setup, state)
    mdloop.init(orc, setup, state)
    for s in range(0, steps + 1):
        if s > 0:
            mdloop.step(gpu, setup, s)
            mdloop.step(orc, setup, s)
        err, scale = _snap_compare(gpu, orc, f"step {s}")
        assert scale > 0.1 and err <= 1e-12 * scale, (s, err, scale)
