"""GB300 SNAP force vs the CPU oracle, ExaMiniMD's dumps, and finite differences (GPU).

The GPU evaluates SNAP in the adjoint form (Y = sum_t cY_t Z_t contracted
with dU/dr); the oracle evaluates the reference formulation (U, Z, dU, dB
per neighbour, sna_impl.hpp).  They agree to rounding: 1e-12 of the RMS
force for FP64 (on a perfect lattice, where every force cancels, both must
vanish).  The SNAP energy (absent from ExaMiniMD) is
checked against the oracle's explicit bispectrum sum and against central
finite differences of the forces.
"""
import numpy as np
import pytest

from tests import mdloop
from tests.golden.decks import CASES, write_case

pytestmark = pytest.mark.gpu


def _ctx():
    from examinimd_gb300 import Context
    return Context(0)


def _max_rel(a, b):
    """max |a-b| over max |b| (positions, velocities)."""
    return np.abs(a - b).max() / np.abs(b).max()


# On a perfect lattice every SNAP force cancels by symmetry: below this RMS
# force (eV/A) a state counts as one, and both force sets must vanish to it.
LATTICE_RMS = 1e-10


def _force_ok(a, b, tol=1e-12):
    """max |a-b| within `tol` of the RMS force of b; on a perfect lattice
    (RMS below LATTICE_RMS) both force sets must cancel instead."""
    rms = float(np.sqrt(np.mean(np.sum(b * b, axis=1))))
    err = float(np.abs(a - b).max())
    if rms < LATTICE_RMS:
        return float(np.abs(a).max()) < LATTICE_RMS, (err, rms)
    return err <= tol * rms, (err, rms)


def _snap_setup(golden, nx=None, ny=None, nz=None, lattice_style=0, a=3.1803):
    g = golden("snap_W_sc")
    snap = mdloop.golden_snap(g)
    c = CASES["snap_W_sc"]
    return mdloop.SnapSetup(nx or c["nx"], ny or c["ny"], nz or c["nz"], snap, a=a, mass=c["mass"],
                            lattice_style=lattice_style), g


SNAP_CASES = [k for k, v in CASES.items() if v["kind"] == "snap"]


@pytest.mark.parametrize("name", SNAP_CASES)
def test_snap_modules_vs_oracle(name, golden):
    """Every golden deck from positions displaced by a seeded 0.05 A
    Gaussian, so forces are of order 1 eV/A and 1e-12 of the RMS force is a
    relative test from the first step (on the undisplaced decks the forces of
    the first steps nearly cancel; the dump test below covers those)."""
    from oracle.orc import Oracle
    g = golden(name)
    setup = mdloop.setup_for_case(name, CASES[name], g)
    state = dict(mdloop.make_lattice(setup))
    rng = np.random.default_rng(20261206)
    state["x"] = state["x"] + rng.normal(0.0, 0.05, state["x"].shape)
    gpu, orc = _ctx(), Oracle()
    mdloop.init(gpu, setup, state)
    mdloop.init(orc, setup, state)
    nl = orc.info()[0]
    a, b = gpu.get(0, nl), orc.get(0, nl)
    np.testing.assert_array_equal(a["id"], b["id"])
    ok, info = _force_ok(a["f"], b["f"])
    assert ok, info
    for s in range(1, 6):
        mdloop.step(gpu, setup, s)
        mdloop.step(orc, setup, s)
        a, b = gpu.get(0, nl), orc.get(0, nl)
        np.testing.assert_array_equal(a["id"], b["id"])
        for k in ("x", "v"):
            assert _max_rel(a[k], b[k]) <= 1e-12, (s, k)
        ok, info = _force_ok(a["f"], b["f"])
        assert ok, (s, info)
    # energy: adjoint identity vs the oracle's explicit bispectrum sum
    eg, eo = gpu.snap_energy(), orc.snap_energy()
    assert abs(eg - eo) <= 1e-11 * abs(eo)


@pytest.mark.parametrize("name", SNAP_CASES)
def test_snap_driver_vs_reference_dumps(name, golden, tmp_path, monkeypatch):
    from examinimd_gb300 import MD
    monkeypatch.chdir(tmp_path)  # the deck names its SNAP files relative to the working directory
    g = golden(name)
    case = CASES[name]
    deck, args = write_case(case, str(tmp_path), mdloop.golden_snap(g))
    md = MD(["-il", deck, "--quiet"] + args)
    done = 0
    for s in [int(v) for v in g["keep_steps"]]:
        if s > done:
            md.run(s - done)
            done = s
        nl = md.info()["N_local"]
        cur = md.ctx.get(0, nl)
        np.testing.assert_array_equal(cur["id"], g[f"s{s}_id"])
        for k in ("x", "v"):
            assert _max_rel(cur[k], g[f"s{s}_{k}"]) <= 1e-12, (s, k)
        ok, info = _force_ok(cur["f"], g[f"s{s}_f"])
        assert ok, (s, info)
    md.close()


def test_snap_energy_finite_difference(golden):
    """F = -dE/dx for the SNAP energy plus the 1.25e5/r^12 pair term."""
    setup, _ = _snap_setup(golden, 3, 3, 3, lattice_style=2)
    state = mdloop.make_lattice(setup)
    rng = np.random.default_rng(7)
    state["x"] = state["x"] + rng.normal(0, 0.05, state["x"].shape)
    gpu = _ctx()
    mdloop.init(gpu, setup, state)
    nl = gpu.info()[0]
    st = gpu.get(0, nl)
    f = st["f"]
    h = 1e-6
    for atom in (0, 7, 31):
        for d in range(3):
            e = []
            for sgn in (+1, -1):
                x = st["x"].copy()
                x[atom, d] += sgn * h
                c2 = _ctx()
                mdloop.init(c2, setup, {**st, "x": x, "q": None})
                e.append(c2.snap_energy())
            fd = -(e[0] - e[1]) / (2 * h)
            assert abs(fd - f[atom, d]) <= 1e-6 * max(1.0, np.abs(f).max()), (atom, d, fd, f[atom, d])


def test_snap_mixed_force_error(golden):
    from examinimd_gb300 import EMD_PREC_MIXED
    setup, _ = _snap_setup(golden, 4, 4, 4, lattice_style=2)
    state = mdloop.make_lattice(setup)
    rng = np.random.default_rng(3)
    state["x"] = state["x"] + rng.normal(0, 0.05, state["x"].shape)
    ref, mix = _ctx(), _ctx()
    mdloop.init(ref, setup, state)
    mdloop.init(mix, setup, state, precision=EMD_PREC_MIXED)
    nl = ref.info()[0]
    a, b = ref.get(0, nl)["f"], mix.get(0, nl)["f"]
    err = np.linalg.norm(b - a, axis=1)
    scale = np.sqrt(np.mean(np.linalg.norm(a, axis=1) ** 2))
    assert np.sqrt(np.mean(err ** 2)) / scale <= 1e-5
    assert err.max() / scale <= 1e-4


@pytest.mark.parametrize("name", SNAP_CASES)
def test_snap_mixed_force_error_on_golden_decks(name, golden):
    """The mixed form against the FP64 form on every SNAP golden deck
    (one and two elements), at displaced positions."""
    from examinimd_gb300 import EMD_PREC_MIXED
    g = golden(name)
    setup = mdloop.setup_for_case(name, CASES[name], g)
    state = mdloop.make_lattice(setup)
    rng = np.random.default_rng(5)
    state["x"] = state["x"] + rng.normal(0, 0.05, state["x"].shape)
    ref, mix = _ctx(), _ctx()
    mdloop.init(ref, setup, state)
    mdloop.init(mix, setup, state, precision=EMD_PREC_MIXED)
    nl = ref.info()[0]
    a, b = ref.get(0, nl), mix.get(0, nl)
    np.testing.assert_array_equal(a["id"], b["id"])
    err = np.linalg.norm(b["f"] - a["f"], axis=1)
    scale = np.sqrt(np.mean(np.linalg.norm(a["f"], axis=1) ** 2))
    assert np.sqrt(np.mean(err ** 2)) / scale <= 1e-5, (name, np.sqrt(np.mean(err ** 2)) / scale)
    assert err.max() / scale <= 1e-4
    ref.close()
    mix.close()


def test_snap_energy_from_the_force_pass(golden):
    """After emd_snap_request_energy the FP64 force kernel also writes every
    atom's energy term with the energy pass's arithmetic and order: the sum
    equals emd_snap_energy bit for bit, and the forces are those of a plain
    compute (to the rounding of their atomic scatter).  A moved position retires the value; the mixed form offers none."""
    from examinimd_gb300 import EMD_PREC_MIXED
    setup, _ = _snap_setup(golden, 4, 4, 4, lattice_style=2)
    state = dict(mdloop.make_lattice(setup))
    state["x"] = state["x"] + np.random.default_rng(9).normal(0, 0.05, state["x"].shape)
    a, b = _ctx(), _ctx()
    mdloop.init(a, setup, state)
    mdloop.init(b, setup, state)
    nl = a.info()[0]
    b.zero_forces()
    b.snap_request_energy()
    b.snap_compute()
    b.comm_update_force()
    fused = b.snap_force_energy()
    assert fused is not None and fused == b.snap_energy() == a.snap_energy()
    # f_j is scattered with FP64 atomics: two computes agree to rounding
    ok, info = _force_ok(b.get(0, nl)["f"], a.get(0, nl)["f"])
    assert ok, info
    b.nve_initial()
    assert b.snap_force_energy() is None
    mix = _ctx()
    mdloop.init(mix, setup, state, precision=EMD_PREC_MIXED)
    mix.zero_forces()
    mix.snap_request_energy()
    mix.snap_compute()
    assert mix.snap_force_energy() is None
