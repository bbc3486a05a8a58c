"""Batched LJ ensemble (GPU, through the C ABI) against the single-system
FP64 drop-in on the same systems.

The batch runs the mixed form, so forces agree with FP64 to the mixed
tolerance (RMS relative error <= 1e-5), and short trajectories stay within
2e-5 of the FP64 ones (mixed-precision force error grown over 45 steps).
"""
import numpy as np
import pytest

from examinimd_gb300 import fit

pytestmark = pytest.mark.gpu

RHO, A = 0.8442, (4.0 / 0.8442) ** (1.0 / 3.0)


def _ensemble(cells, seed=3):
    rng = np.random.default_rng(seed)
    xs, vs, boxes, ns = [], [], [], []
    for c in cells:
        # displaced lattice: the net forces of a perfect lattice cancel to rounding
        x = np.mod(fit.lattice("fcc", A, c) + rng.normal(0.0, 0.05, size=(4 * c ** 3, 3)), c * A)
        v = rng.normal(0.0, 1.2, size=x.shape)
        v -= v.mean(axis=0)
        xs.append(x)
        vs.append(v)
        boxes.append([c * A] * 3)
        ns.append(len(x))
    return ns, np.array(boxes), xs, vs


def _fp64_context(x, v, box):
    from examinimd_gb300 import Context
    from tests import mdloop
    setup = mdloop.LJSetup(1)
    setup.nx = setup.ny = setup.nz = 1
    setup.a = box[0]  # domain = a * n: the whole box
    st = {"x": x, "v": v, "type": np.zeros(len(x), np.int32), "id": np.arange(1, len(x) + 1, dtype=np.int32)}
    ctx = Context(0)
    mdloop.init(ctx, setup, st)
    return ctx, setup


def _by_id(ctx, n, key):
    g = ctx.get(0, n)
    out = np.empty_like(g[key])
    out[g["id"] - 1] = g[key]
    return out


def _rms_rel(a, b):
    return np.sqrt(np.mean(np.sum((a - b) ** 2, axis=1))) / np.sqrt(np.mean(np.sum(b ** 2, axis=1)))


def test_batch_forces_and_trajectory_match_fp64():
    from examinimd_gb300 import Batch
    from tests import mdloop
    cells = [5, 7, 6, 5, 8]
    ns, boxes, xs, vs = _ensemble(cells)
    b = Batch(ns, boxes, np.concatenate(xs), np.concatenate(vs))
    offs = np.concatenate([[0], np.cumsum(ns)])
    _, _, f0 = b.get()
    refs = []
    for k in range(len(ns)):
        ctx, setup = _fp64_context(xs[k], vs[k], boxes[k])
        fr = _by_id(ctx, ns[k], "f")
        assert _rms_rel(f0[offs[k]:offs[k + 1]], fr) <= 1e-5
        refs.append((ctx, setup))
    steps = 45  # two rebuilds and a partial period
    b.run(steps)
    x1, v1, _ = b.get()
    for k, (ctx, setup) in enumerate(refs):
        for s in range(1, steps + 1):
            mdloop.step(ctx, setup, s)
        xr = _by_id(ctx, ns[k], "x")
        d = x1[offs[k]:offs[k + 1]] - xr
        d -= boxes[k] * np.round(d / boxes[k])  # either side of a periodic wrap
        assert np.abs(d).max() <= 2e-5, (k, np.abs(d).max())
        ctx.close()
    b.close()


def test_batch_energy_conservation_and_tune_restores_state():
    from examinimd_gb300 import Batch
    ns, boxes, xs, vs = _ensemble([5, 6, 9, 5], seed=4)
    b = Batch(ns, boxes, np.concatenate(xs), np.concatenate(vs))
    x0, v0, _ = b.get()
    threads, spl = b.tune(40)
    assert threads in (256, 512, 1024) and (spl == 0 or spl >= 20)  # 0: the phased form
    x1, v1, _ = b.get()
    np.testing.assert_array_equal(x0, x1)
    np.testing.assert_array_equal(v0, v1)
    mv2, pe = b.thermo()
    e0 = 0.5 * mv2 + pe
    b.run(400)
    mv2, pe = b.thermo()
    e1 = 0.5 * mv2 + pe
    assert np.all(np.abs(e1 - e0) / np.abs(e0) <= 1e-3), (e1 - e0) / np.abs(e0)
    assert b.info()["steps_done"] == 400
    b.close()


def test_batch_phased_equals_persistent():
    """The phased form (one launch per phase over all systems) performs the
    same per-atom arithmetic in the same order as the persistent form."""
    from examinimd_gb300 import Batch
    ns, boxes, xs, vs = _ensemble([5, 8, 6], seed=5)
    out = []
    for threads, spl in ((1024, 20), (512, 0)):
        b = Batch(ns, boxes, np.concatenate(xs), np.concatenate(vs))
        b.set_shape(threads, spl)
        b.run(45)
        out.append(b.get())
        assert b.info()["steps_per_launch"] == spl
        b.close()
    for a, c in zip(out[0], out[1]):
        np.testing.assert_array_equal(a, c)
