"""emd_md_run_host: run(nsteps) with the particle state in host arrays (GPU).

Every step uploads x, v, f, runs, and reads them back with the read-backs
overlapped with the step's own work.  The result must equal, bit for bit,
the plain sequence emd_system_update -> run(1) -> emd_system_get that the
overlap replaces, across a neighbour rebuild (which re-sorts the atoms), in
both precision forms.
"""
import numpy as np
import pytest

from tests.golden.decks import CASES, write_case

pytestmark = pytest.mark.gpu


def _host_arrays(src, pinned):
    """x, v, f of ``src`` in new host arrays: pageable numpy arrays, or
    page-locked ones (the staged uploads and read-backs then overlap for
    real instead of each copy waiting on the host)."""
    out = []
    for k in ("x", "v", "f"):
        if pinned:
            import torch
            a = torch.empty(src[k].shape, dtype=torch.float64, pin_memory=True).numpy()
            a[...] = src[k]
        else:
            a = np.ascontiguousarray(src[k])
        out.append(a)
    return out


# 6^3 fcc cells (864 atoms) fit in one chunk of the step start (chunk edges
# fall on multiples of 512 rows); 9^3 cells (2,916 atoms) split into two
@pytest.mark.parametrize("cells", [6, 9])
@pytest.mark.parametrize("precision,pinned", [("fp64", False), ("mixed", False), ("fp64", True), ("mixed", True)])
def test_run_host_equals_update_run_get(precision, pinned, cells, tmp_path):
    from examinimd_gb300 import MD
    case = dict(CASES["lj_fcc6_full_csr"], n=cells)
    deck, args = write_case(case, str(tmp_path))
    args = args + ["--precision", precision]
    a, b = MD(["-il", deck, "--quiet"] + args), MD(["-il", deck, "--quiet"] + args)
    n = a.info()["N_local"]
    ref = a.ctx.get(0, n)
    hx, hv, hf = (np.ascontiguousarray(ref[k]) for k in ("x", "v", "f"))
    steps = 45  # the rebuilds at steps 20 and 40 re-sort the atoms in between
    for _ in range(steps):
        a.ctx.update(0, hx, hv, hf)
        a.run(1)
        cur = a.ctx.get(0, n)
        hx, hv, hf = (np.ascontiguousarray(cur[k]) for k in ("x", "v", "f"))
    bx, bv, bf = _host_arrays(b.ctx.get(0, n), pinned)
    b.run_host(steps, bx, bv, bf)
    for name, p, q in (("x", hx, bx), ("v", hv, bv), ("f", hf, bf)):
        np.testing.assert_array_equal(p, q, err_msg=name)
    # the device state agrees with the host arrays
    fin = b.ctx.get(0, n)
    for name, q in (("x", bx), ("v", bv), ("f", bf)):
        np.testing.assert_array_equal(fin[name], q, err_msg=name)
    a.close()
    b.close()


def test_run_host_rejects_wrong_arrays(tmp_path):
    from examinimd_gb300 import MD, EmdError
    deck, args = write_case(dict(CASES["lj_fcc6_full_csr"]), str(tmp_path))
    md = MD(["-il", deck, "--quiet"] + args)
    n = md.info()["N_local"]
    with pytest.raises(EmdError):
        md.run_host(1, np.zeros((n, 3), np.float32), np.zeros((n, 3)), np.zeros((n, 3)))
    md.close()


def test_stage_commit_equals_update(tmp_path):
    """emd_system_stage + emd_system_commit leave the same state as
    emd_system_update with the same arrays; unstaged fields stay as they were."""
    from examinimd_gb300 import MD
    deck, args = write_case(dict(CASES["lj_fcc6_full_csr"]), str(tmp_path))
    a, b = MD(["-il", deck, "--quiet"] + args), MD(["-il", deck, "--quiet"] + args)
    n = a.info()["N_local"]
    st = a.ctx.get(0, n)
    rng = np.random.default_rng(5)
    x = np.ascontiguousarray(st["x"] + rng.uniform(-0.01, 0.01, (n, 3)))
    v = np.ascontiguousarray(rng.normal(size=(n, 3)))
    f = np.ascontiguousarray(rng.normal(size=(n, 3)))
    a.ctx.update(0, x, v, f)
    for field, arr in ((0, x), (1, v), (2, f)):
        b.ctx.stage(field, arr)
    b.ctx.commit()
    ga, gb = a.ctx.get(0, n), b.ctx.get(0, n)
    for k in ("x", "v", "f", "type", "id"):
        np.testing.assert_array_equal(ga[k], gb[k], err_msg=k)
    # one field staged: the others are untouched
    v2 = np.ascontiguousarray(v * 0.5)
    b.ctx.stage(1, v2)
    b.ctx.commit()
    gc = b.ctx.get(0, n)
    np.testing.assert_array_equal(gc["v"], v2)
    np.testing.assert_array_equal(gc["x"], gb["x"])
    np.testing.assert_array_equal(gc["f"], gb["f"])
    # a commit with nothing staged changes nothing
    b.ctx.commit()
    np.testing.assert_array_equal(b.ctx.get(0, n)["v"], v2)
    # the runs continue identically from the two states
    a.ctx.update(0, None, v2, None)
    a.run(3)
    b.run(3)
    ga, gb = a.ctx.get(0, n), b.ctx.get(0, n)
    for k in ("x", "v", "f"):
        np.testing.assert_array_equal(ga[k], gb[k], err_msg=k)
    a.close()
    b.close()


def test_stage_rejects_bad_arguments(tmp_path):
    from examinimd_gb300 import MD, EmdError
    deck, args = write_case(dict(CASES["lj_fcc6_full_csr"]), str(tmp_path))
    md = MD(["-il", deck, "--quiet"] + args)
    n = md.info()["N_local"]
    with pytest.raises(EmdError):
        md.ctx.stage(3, np.zeros((n, 3)))
    with pytest.raises(TypeError):
        md.ctx.stage(0, np.zeros((n, 3), np.float32))
    md.close()


def test_ranged_stage_commit_and_initial_integration(tmp_path):
    """Rows staged and committed chunk by chunk, then integrated chunk by
    chunk, leave the bits of update + one whole initial integration."""
    from examinimd_gb300 import MD
    deck, args = write_case(dict(CASES["lj_fcc6_full_csr"]), str(tmp_path))
    for precision in ("fp64", "mixed"):
        a, b = (MD(["-il", deck, "--quiet", "--precision", precision] + args) for _ in range(2))
        n = a.info()["N_local"]
        st = a.ctx.get(0, n)
        rng = np.random.default_rng(7)
        x = np.ascontiguousarray(st["x"] + rng.uniform(-0.01, 0.01, (n, 3)))
        v = np.ascontiguousarray(rng.normal(size=(n, 3)))
        f = np.ascontiguousarray(rng.normal(size=(n, 3)))
        a.ctx.update(0, x, v, f)
        a.ctx.nve_initial()
        cuts = [0, n // 3, n // 2, n]
        for lo, hi in zip(cuts[:-1], cuts[1:]):
            for field, arr in ((0, x), (1, v), (2, f)):
                b.ctx.stage_range(field, np.ascontiguousarray(arr[lo:hi]), lo)
        for lo, hi in zip(cuts[:-1], cuts[1:]):
            b.ctx.commit_range(lo, hi - lo)
            b.ctx.nve_initial_range(lo, hi - lo)
        ga, gb = a.ctx.get(0, n), b.ctx.get(0, n)
        for k in ("x", "v", "f"):
            np.testing.assert_array_equal(ga[k], gb[k], err_msg=f"{precision} {k}")
        a.close()
        b.close()


def test_commit_range_rejects_a_straddling_stage(tmp_path):
    from examinimd_gb300 import MD, EmdError
    deck, args = write_case(dict(CASES["lj_fcc6_full_csr"]), str(tmp_path))
    md = MD(["-il", deck, "--quiet"] + args)
    n = md.info()["N_local"]
    v = np.ascontiguousarray(md.ctx.get(0, n)["v"])
    md.ctx.stage_range(1, np.ascontiguousarray(v[: n // 2]), 0)
    with pytest.raises(EmdError):
        md.ctx.commit_range(0, n // 4)
    md.ctx.commit_range(0, n)  # the whole range takes it
    np.testing.assert_array_equal(md.ctx.get(0, n)["v"], v)
    with pytest.raises(EmdError):
        md.ctx.commit_range(0, n + 1)
    md.close()


def test_staged_ranges_from_before_a_count_change_are_dropped(tmp_path):
    """Rows staged before N_local changed no longer name the same particles:
    a commit that finds them fails, and a new stage starts afresh."""
    from examinimd_gb300 import MD, EmdError
    deck, args = write_case(dict(CASES["lj_fcc6_full_csr"]), str(tmp_path))
    md = MD(["-il", deck, "--quiet"] + args)
    ctx = md.ctx
    n = md.info()["N_local"]
    st = ctx.get(0, n)
    x, v, t, i = (np.ascontiguousarray(st[k]) for k in ("x", "v", "type", "id"))
    stale = np.ascontiguousarray(np.full((n, 3), 7.0))
    ctx.stage(1, stale)
    m = n - 4
    ctx.set_local(x[:m], t[:m], i[:m], v=v[:m])
    with pytest.raises(EmdError):
        ctx.commit()
    # the stale range is gone: a new stage and commit move only the new rows
    ctx.commit()
    with pytest.raises(EmdError):  # the whole-array form wants all N_local rows
        ctx.stage(1, stale)
    ctx.stage(1, np.ascontiguousarray(v[:m] * 2.0))
    ctx.commit()
    np.testing.assert_array_equal(ctx.get(0, m)["v"], v[:m] * 2.0)
    md.close()
