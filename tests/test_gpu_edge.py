"""Edge cases of the hot path (GPU, through the C ABI).

* an empty system goes through every module call and yields nothing;
* a box only slightly wider than the halo depth (every atom imaged on both
  sides of a dimension) still matches the oracle bit for bit;
* at the full LJ-4M size, properties that do not depend on the size: the
  net force of a full list vanishes to rounding, FP64 and mixed, and the
  mixed forces stay within the mixed tolerance of the FP64 ones.
"""
import numpy as np
import pytest

from tests import mdloop

pytestmark = pytest.mark.gpu


def _ctx():
    from examinimd_gb300 import Context
    return Context(0)


def test_empty_system_runs_every_module():
    setup = mdloop.LJSetup(4)
    c = _ctx()
    state = {"x": np.zeros((0, 3)), "v": np.zeros((0, 3)), "type": np.zeros(0, np.int32),
             "id": np.zeros(0, np.int32)}
    total = mdloop.init(c, setup, state)
    assert total == 0
    for s in range(1, 22):  # across a rebuild step
        mdloop.step(c, setup, s)
    assert c.info()[:2] == (0, 0)
    assert c.lj_energy() == 0.0
    assert c.thermo_mv2() == 0.0
    c.close()


@pytest.mark.parametrize("half,kind", [(False, 0), (True, 1)])
def test_box_narrower_than_two_halo_depths(half, kind):
    """fcc 3^3: L = 5.04 < 2 x 2.8, so atoms are imaged on both faces."""
    from oracle.orc import Oracle
    setup = mdloop.LJSetup(3, half=half, kind=kind, every=5)
    assert setup.domain[0] < 2 * setup.neigh_cut
    state = mdloop.make_lattice(setup)
    gpu, orc = _ctx(), Oracle()
    assert mdloop.init(gpu, setup, state) == mdloop.init(orc, setup, state)
    for s in range(1, 12):
        mdloop.step(gpu, setup, s)
        mdloop.step(orc, setup, s)
    nl, ng, _ = orc.info()
    assert gpu.info()[:2] == (nl, ng)
    a, b = gpu.get(0, nl), orc.get(0, nl)
    np.testing.assert_array_equal(a["id"], b["id"])
    if half:  # atomically scattered sums: rounding-level agreement
        for k in ("x", "v", "f"):
            assert np.abs(a[k] - b[k]).max() <= 1e-12 * max(np.abs(b[k]).max(), 1.0)
    else:
        for k in ("x", "v", "f"):
            np.testing.assert_array_equal(a[k], b[k])
    gpu.close()


def test_full_size_net_force_and_mixed_error():
    """LJ-4M (fcc 100^3): sum of forces ~ 0, mixed vs FP64 within 1e-5 RMS."""
    setup = mdloop.LJSetup(100)
    state = mdloop.make_lattice(setup, 8)
    rng = np.random.default_rng(1)
    state["x"] = np.mod(state["x"] + rng.normal(0, 0.02, state["x"].shape), setup.domain[0])
    forces = {}
    for prec in (0, 1):
        c = _ctx()
        mdloop.init(c, setup, state, precision=prec)
        nl = c.info()[0]
        g = c.get(0, nl)
        f = np.empty_like(g["f"])
        f[g["id"] - 1] = g["f"]
        forces[prec] = f
        net = np.abs(f.sum(axis=0)).max()
        assert net <= (1e-11 if prec == 0 else 1e-5) * np.abs(f).sum(axis=0).max(), (prec, net)
        c.close()
    err = np.linalg.norm(forces[1] - forces[0], axis=1)
    scale = np.sqrt(np.mean(np.sum(forces[0] ** 2, axis=1)))
    assert np.sqrt(np.mean(err ** 2)) / scale <= 1e-5


def test_kernel_timing_restricted_to_named_kernels():
    """emd_timing_only: events on the named kernels only, every launch counted;
    the results do not depend on the timing mode."""
    setup = mdloop.LJSetup(5)
    state = mdloop.make_lattice(setup)
    runs = []
    for only in (None, "lj_full_fp64"):
        c = _ctx()
        mdloop.init(c, setup, state)
        c.timing(True)
        c.timing_only(only)
        c.timing_reset()
        for s in range(1, 22):
            mdloop.step(c, setup, s)
        rep = c.timing_report()
        c.timing(False)
        runs.append((rep, c.get(0, c.info()[0])))
        c.close()
    full, part = runs[0][0], runs[1][0]
    assert set(full) == set(part)
    for k in full:
        assert full[k][1] == part[k][1], k  # the same launches counted
        if k == "lj_full_fp64":
            assert part[k][0] > 0.0
        else:
            assert part[k][0] == 0.0 and full[k][0] > 0.0, k
    for k in ("x", "v", "f"):
        np.testing.assert_array_equal(runs[0][1][k], runs[1][1][k])
