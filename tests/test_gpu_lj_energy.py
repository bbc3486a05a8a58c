"""The mixed-precision LJ energy of a thermo step, delivered by the force call (GPU).

On thermo steps the driver asks for the energy with the force
(emd_lj_request_energy): the force call then runs the energy kernel over the
same rows and pair decisions, and emd_lj_force_energy returns it while the
positions stay unchanged.  It is compared with the FP64 energy of the same
positions (emd_lj_energy).  Every pair is carried as an FP32 value and its
first-order remainder (the exact pair difference including the rounding of
the FP32 positions, the rounding of r^2, the reciprocal's and the products'
remainders) and the per-atom sums keep every addition's rounding error, so
what is left is second order: the bound is 1e-11 relative everywhere, on
perfect fcc lattices (where all pairs of a shell share one distance and any
FP32 rounding would add up coherently, 5e-8 relative) as on thermalised
ones, from 864 atoms to LJ-4M.
"""
import numpy as np
import pytest

from tests import mdloop

pytestmark = pytest.mark.gpu


def _ctx():
    from examinimd_gb300 import Context
    return Context(0)


def _rms_rel(a, b):
    return np.sqrt(np.mean(np.sum((a - b) ** 2, axis=1))) / np.sqrt(np.mean(np.sum(b ** 2, axis=1)))


@pytest.mark.parametrize("n,tol", [(6, 1e-11), (10, 1e-11), (100, 1e-11)])
def test_thermo_energy_matches_fp64_energy(n, tol):
    setup = mdloop.LJSetup(n)
    state = dict(mdloop.make_lattice(setup, 8))
    rng = np.random.default_rng(n)
    state["x"] = np.mod(state["x"] + rng.normal(0.0, 0.03, state["x"].shape), setup.domain[0])
    mix = _ctx()
    mdloop.init(mix, setup, state, precision=1)
    for s in range(1, 4):
        mdloop.step(mix, setup, s)
    assert mix.lj_force_energy() is None  # not asked for
    mix.zero_forces()
    mix.lj_request_energy()
    mix.lj_compute()
    delivered = mix.lj_force_energy()
    exact = mix.lj_energy()  # FP64 over the same list and positions
    assert delivered is not None
    assert abs(delivered - exact) <= tol * abs(exact), (delivered, exact, (delivered - exact) / exact)
    # the request served one compute only; a moved position retires the value
    mix.lj_compute()
    assert mix.lj_force_energy() is None
    mix.lj_request_energy()
    mix.lj_compute()
    assert mix.lj_force_energy() is not None
    mix.nve_initial()
    assert mix.lj_force_energy() is None
    mix.close()


@pytest.mark.parametrize("n", [20, 100])
def test_thermo_energy_on_the_perfect_lattice(n):
    """The thermo step 0 of the LJ decks: every pair of a neighbour shell
    has the same distance, so an FP32 rounding of the pair energy would add
    up coherently (5e-8 relative); the carried remainders do not."""
    setup = mdloop.LJSetup(n)
    mix = _ctx()
    mdloop.init(mix, setup, mdloop.make_lattice(setup, 8), precision=1)
    mix.zero_forces()
    mix.lj_request_energy()
    mix.lj_compute()
    delivered, exact = mix.lj_force_energy(), mix.lj_energy()
    assert delivered is not None
    assert abs(delivered - exact) <= 1e-11 * abs(exact), (delivered, exact, (delivered - exact) / exact)
    mix.close()


@pytest.mark.parametrize("n,moved", [(20, False), (10, True)])
def test_standalone_mixed_energy(n, moved):
    """emd_lj_energy_mixed: the energy kernel alone on the current positions
    and list, without a force call: within 1e-11 of emd_lj_energy, the
    forces untouched."""
    setup = mdloop.LJSetup(n)
    mix = _ctx()
    mdloop.init(mix, setup, mdloop.make_lattice(setup, 8), precision=1)
    if moved:
        for s in range(1, 8):
            mdloop.step(mix, setup, s)
    nl = mix.info()[0]
    f0 = mix.get(0, nl)["f"]
    e, exact = mix.lj_energy_mixed(), mix.lj_energy()
    assert e is not None
    assert abs(e - exact) <= 1e-11 * abs(exact), (e, exact, (e - exact) / exact)
    np.testing.assert_array_equal(mix.get(0, nl)["f"], f0)
    mix.close()


def test_thermo_energy_does_not_change_the_forces():
    """A compute with the energy gives the same force bits as one without."""
    setup = mdloop.LJSetup(8)
    state = mdloop.make_lattice(setup)
    a, b = _ctx(), _ctx()
    for c in (a, b):
        mdloop.init(c, setup, state, precision=1)
        for s in range(1, 25):
            if c is b and s % 5 == 0:
                c.lj_request_energy()
            mdloop.step(c, setup, s)
    nl = a.info()[0]
    ga, gb = a.get(0, nl), b.get(0, nl)
    for k in ("x", "v", "f"):
        np.testing.assert_array_equal(ga[k], gb[k])


def test_driver_thermo_uses_the_delivered_energy(tmp_path):
    """The driver asks for the energy on thermo steps: its thermo PE in the
    mixed form stays within the delivered-energy bound of the FP64 value."""
    from examinimd_gb300 import MD
    from tests.golden.decks import CASES, write_case
    case = dict(CASES["lj_fcc6_full_csr"])
    deck, args = write_case(case, str(tmp_path))
    md = MD(["-il", deck, "--quiet", "--precision", "mixed"] + args)
    md.run(20)  # thermo every 10: step 20 asked for the energy
    assert md.ctx.lj_force_energy() is not None
    T, pe, ke = md.thermo(recompute=True)
    exact = md.ctx.lj_energy() / md.info()["N_local"]
    assert abs(pe - exact) <= 1e-11 * abs(exact)
    md.close()


def test_several_types_have_no_delivered_energy():
    """The delivered energy covers one type pair; with per-pair parameters the
    caller falls back to emd_lj_energy."""
    rng = np.random.default_rng(13)
    coeffs = [(a, b, float(rng.uniform(0.8, 1.2)), float(rng.uniform(0.9, 1.05)), 2.5)
              for a in range(1, 14) for b in range(a, 14)]
    setup = mdloop.LJSetup(5, masses=list(rng.uniform(0.8, 2.0, 13)), coeffs=coeffs)
    mix = _ctx()
    mdloop.init(mix, setup, mdloop.make_lattice(setup), precision=1)
    mix.zero_forces()
    mix.lj_request_energy()
    mix.lj_compute()
    assert mix.lj_force_energy() is None
    assert mix.lj_energy_mixed() is None


def test_large_cutoff_rows_and_forces():
    """rc = 6: bins of about 250 particles; rows equal the oracle's, mixed
    forces within the mixed tolerance of FP64, and the delivered energy within
    its bound."""
    from oracle.orc import Oracle
    setup = mdloop.LJSetup(12, cut=6.0, skin=0.3, coeffs=[(1, 1, 1.0, 1.0, 6.0)])
    state = dict(mdloop.make_lattice(setup))
    rng = np.random.default_rng(4)
    state["x"] = np.mod(state["x"] + rng.normal(0.0, 0.03, state["x"].shape), setup.domain[0])
    mix, ref, orc = _ctx(), _ctx(), Oracle(8)
    tm = mdloop.init(mix, setup, state, precision=1)
    mdloop.init(ref, setup, state)
    to = mdloop.init(orc, setup, state)
    assert tm == to
    for x, y in zip(mix.neigh_get(tm), orc.neigh_get(to)):
        np.testing.assert_array_equal(x, y)
    nl = ref.info()[0]
    assert _rms_rel(mix.get(0, nl)["f"], ref.get(0, nl)["f"]) <= 1e-5
    mix.zero_forces()
    mix.lj_request_energy()
    mix.lj_compute()
    delivered, exact = mix.lj_force_energy(), ref.lj_energy()
    assert delivered is not None and abs(delivered - exact) <= 1e-11 * abs(exact)
