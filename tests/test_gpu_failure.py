"""Failure detection, injected on the host (GPU).

No test here faults, traps or hangs the GPU: every failure is made by the
caller's inputs, and every device-side check it reaches clamps or skips the
access and latches a status bit instead.

* Capacities that start tiny grow and the call is redone, as CommSerial
  (comm_serial.cpp:73-89) and Neighbor2D (neighbor_2d.h:304-330) do:
  particle arrays, ghost lists and the 2D row stride sized for 108 lattice
  atoms then serve 2,048 atoms at twice the lattice density, with the
  oracle's rows, ghosts and forces.
* The batched ensemble has fixed capacities: a row capacity below the real
  row length returns EMD_ERR_OVERFLOW_NEIGH (rows are clamped to the
  capacity on the device), and the process can go on using the GPU.
* A particle outside the binned box (not wrapped by an exchange) latches
  EMD_ERR_BOUNDS in the status word; the binning keeps it in the nearest bin.
* A truncated deck, a truncated .snapcoeff and a malformed .snapparam give an
  error status from emd_md_create instead of ending the process.
"""
import numpy as np
import pytest

from tests import mdloop

pytestmark = pytest.mark.gpu


def _ctx():
    from examinimd_gb300 import Context
    return Context(0)


def _gas(setup, rho, seed):
    """A uniform random gas filling setup's box at reduced density rho."""
    L = np.array(setup.domain)
    n = int(round(rho * L.prod()))
    rng = np.random.default_rng(seed)
    return {"x": rng.uniform(0.0, 1.0, (n, 3)) * L, "v": rng.normal(0.0, 1.0, (n, 3)),
            "type": np.zeros(n, np.int32), "id": np.arange(1, n + 1, dtype=np.int32)}


@pytest.mark.parametrize("kind", [0, 1])
def test_tiny_capacities_grow_to_the_oracle_result(kind):
    from oracle.orc import Oracle
    gpu = _ctx()
    small = mdloop.LJSetup(3, kind=kind, every=2)
    mdloop.init(gpu, small, mdloop.make_lattice(small))
    for s in range(1, 4):
        mdloop.step(gpu, small, s)
    assert gpu.info()[0] == 108
    m0 = gpu.neigh_maxneighs()
    # the same context, 8^3 fcc cells compressed to rho 1.7: 19x the atoms,
    # twice the neighbours per row
    big = mdloop.LJSetup(8, kind=kind, every=2, rho=1.7)
    state = mdloop.make_lattice(big)
    orc = Oracle()
    tg, to = mdloop.init(gpu, big, state), mdloop.init(orc, big, state)
    assert tg == to
    nl, ng, nt = orc.info()
    assert gpu.info()[:2] == (nl, ng) and nl == 2048 and ng > 20 * 108
    for x, y in zip(gpu.comm_ghosts(), orc.comm_ghosts()):
        np.testing.assert_array_equal(x, y)
    for x, y in zip(gpu.neigh_get(tg), orc.neigh_get(to)):
        np.testing.assert_array_equal(x, y)
    if kind == 1:
        rows = gpu.neigh_get(tg)[0]
        assert gpu.neigh_maxneighs() >= rows.max() > m0
    for s in range(1, 5):
        mdloop.step(gpu, big, s)
        mdloop.step(orc, big, s)
    a, b = gpu.get(0, nl), orc.get(0, nl)
    for k in ("id", "x", "v", "f"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    assert gpu.status() == 0


def _fcc_batch_inputs(cells, seed=5):
    from examinimd_gb300 import fit
    a = (4.0 / 0.8442) ** (1.0 / 3.0)
    rng = np.random.default_rng(seed)
    xs, vs, boxes, ns = [], [], [], []
    for c in cells:
        x = np.mod(fit.lattice("fcc", a, c) + rng.normal(0.0, 0.02, size=(4 * c ** 3, 3)), c * a)
        xs.append(x)
        vs.append(rng.normal(0.0, 1.0, x.shape))
        boxes.append([c * a] * 3)
        ns.append(len(x))
    return np.array(ns), np.array(boxes), np.concatenate(xs), np.concatenate(vs)


def test_batch_row_capacity_overflow_is_a_status():
    from examinimd_gb300 import Batch, EmdError
    ns, boxes, x, v = _fcc_batch_inputs([5, 6])
    # rows hold about 77 entries: the first build, inside emd_batch_create,
    # overflows a capacity of 8 and the call returns the status
    with pytest.raises(EmdError, match="neighbour capacity overflow"):
        Batch(ns, boxes, x, v, max_neigh=8)
    # the GPU and the library stay usable: the same ensemble with room runs
    ok = Batch(ns, boxes, x, v, max_neigh=128)
    ok.run(5)
    ok.close()
    gpu = _ctx()
    setup = mdloop.LJSetup(4)
    mdloop.init(gpu, setup, mdloop.make_lattice(setup))
    mdloop.step(gpu, setup, 1)
    assert gpu.status() == 0


def test_particle_outside_the_box_latches_bounds():
    from examinimd_gb300 import EMD_ERR_BOUNDS
    setup = mdloop.LJSetup(4)
    state = dict(mdloop.make_lattice(setup))
    L = setup.domain[0]
    state["x"] = state["x"].copy()
    state["x"][7] = [3.5 * L, 0.5 * L, -2.5 * L]
    gpu = _ctx()
    gpu.system_init(setup.masses, setup.boltz, setup.mvv2e, setup.dt, setup.domain)
    gpu.set_local(state["x"], state["type"], state["id"], v=state["v"])
    assert gpu.status() == 0
    c = setup.neigh_cut
    gpu.binning_create(c, c, c, 1, True, False, True)
    assert gpu.status() & (1 << EMD_ERR_BOUNDS)
    # the binning clamped the particle into the grid: counts still add up
    nb = gpu.binning_create(c, c, c, 1, True, False, False)
    bc, bo, perm, _ = gpu.binning_get(int(np.prod(nb)), len(state["x"]))
    assert int(bc.sum()) == len(state["x"])
    np.testing.assert_array_equal(np.sort(perm), np.arange(len(state["x"])))
    # a fresh context on the same device runs normally
    ok = _ctx()
    mdloop.init(ok, setup, mdloop.make_lattice(setup))
    assert ok.status() == 0


def _lj_deck(path, lines):
    with open(path, "w") as fp:
        fp.write("\n".join(lines) + "\n")
    return str(path)


LJ_DECK = ["units lj", "atom_style atomic", "lattice fcc 0.8442", "region box block 0 4 0 4 0 4",
           "create_box 1 box", "create_atoms 1 box", "mass 1 1.0", "velocity all create 1.44 87287 loop geom",
           "pair_style lj/cut 2.5", "pair_coeff 1 1 1.0 1.0 2.5", "neighbor 0.3 bin",
           "neigh_modify delay 0 every 20 check no", "fix 1 all nve", "thermo 10", "run 10"]


@pytest.mark.parametrize("cut", [3, 5, 9])
def test_truncated_deck_is_an_error_status(tmp_path, cut):
    """A deck cut off before its pair_style (or in the middle of a line)."""
    from examinimd_gb300 import MD, EmdError
    lines = LJ_DECK[:cut]
    if cut == 9:
        lines = LJ_DECK[:8] + ["pair_style"]
    deck = _lj_deck(tmp_path / "in.cut", lines)
    with pytest.raises(EmdError):
        MD(["-il", deck, "--quiet"])
    # the process goes on: the whole deck runs
    md = MD(["-il", _lj_deck(tmp_path / "in.ok", LJ_DECK), "--quiet"])
    md.run(2)
    md.close()


@pytest.mark.parametrize("which", ["coeff_short", "coeff_empty", "param_bad"])
def test_truncated_snap_files_are_an_error_status(tmp_path, monkeypatch, which):
    from examinimd_gb300 import MD, EmdError
    from tests.golden.decks import snap_w_synthetic
    monkeypatch.chdir(tmp_path)
    snap = snap_w_synthetic()
    coeff = ["1 56", "W 0.5 1"] + [repr(b) for b in snap["beta"]]
    param = [f"{k} {v}" for k, v in snap["params"].items()]
    if which == "coeff_short":
        coeff = coeff[:30]
    elif which == "coeff_empty":
        coeff = []
    else:
        param = ["rcutfac", "twojmax 8"]
    (tmp_path / "W.snapcoeff").write_text("\n".join(coeff) + "\n")
    (tmp_path / "W.snapparam").write_text("\n".join(param) + "\n")
    deck = _lj_deck(tmp_path / "in.snap", [
        "units metal", "atom_style atomic", "newton on", "lattice bcc 3.1803", "region box block 0 3 0 3 0 3",
        "create_box 1 box", "create_atoms 1 box", "mass 1 183.84", "pair_style snap",
        "pair_coeff * * W.snapcoeff W W.snapparam W", "neighbor 1.0 bin",
        "neigh_modify once no every 1 delay 0 check yes", "velocity all create 300.0 4928459 loop geom",
        "fix 1 all nve", "run 1"])
    with pytest.raises(EmdError, match="SNAP"):
        MD(["-il", deck, "--quiet"])


def test_no_list_from_a_binning_that_sorted():
    """A binning that re-sorted the particles leaves a permutation that no
    longer refers to them: a neighbour build from it is refused with
    EMD_ERR_STATE, and the next unsorted binning allows it again."""
    from examinimd_gb300 import EmdError
    setup = mdloop.LJSetup(4)
    st = mdloop.make_lattice(setup)
    gpu = _ctx()
    gpu.system_init(setup.masses, setup.boltz, setup.mvv2e, setup.dt, setup.domain)
    gpu.set_local(st["x"], st["type"], st["id"], v=st["v"])
    setup.force_init(gpu)
    gpu.comm_init(setup.neigh_cut)
    gpu.neigh_init(setup.kind, setup.neigh_cut, setup.newton)
    c = setup.neigh_cut
    gpu.comm_exchange()
    gpu.binning_create(c, c, c, 1, True, False, True)  # no ghosts yet: this binning covers every particle
    with pytest.raises(EmdError, match="re-sorted"):
        gpu.neigh_create(False)
    gpu.comm_exchange_halo()
    gpu.binning_create(c, c, c, 1, True, True, False)
    assert gpu.neigh_create(False) > 0
