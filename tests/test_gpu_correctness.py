"""ExaMiniMD's --correctness report on the GB300 driver (GPU).

`--correctness N DIR FILE` compares the current owned particles, matched by
id, against DIR/output.<step>.000 dumps every N steps and appends
"step |dr| max|dr| |dv| max|dv| |df| max|df|" to FILE
(examinimd.cpp:355-482).  Fed ExaMiniMD's own dumps of the same deck, the
FP64 drop-in must report zeros; a planted difference must show up with its
exact size; rows in another order must still match by id; and the mixed form
reports force differences within its tolerance.
"""
import os

import numpy as np
import pytest

from tests.golden.decks import CASES, write_case

pytestmark = pytest.mark.gpu

NAME = "lj_fcc6_full_csr"


def _write_dump(path, d):
    n = len(d["id"])
    with open(path, "wb") as fp:
        np.array([n], np.int32).tofile(fp)
        d["id"].astype(np.int32).tofile(fp)
        d["type"].astype(np.int32).tofile(fp)
        d["q"].astype(np.float64).tofile(fp)
        for k in ("x", "v", "f"):
            np.ascontiguousarray(d[k], np.float64).tofile(fp)


def _reference_dumps(golden, directory, steps, edit=None):
    g = golden(NAME)
    for s in steps:
        d = {k: g[f"s{s}_{k}"].copy() for k in ("id", "type", "q", "x", "v", "f")}
        if edit:
            d = edit(s, d)
        _write_dump(os.path.join(directory, f"output.{s:010d}.000"), d)


def _report(path):
    rows = [ln.split() for ln in open(path) if not ln.startswith("#")]
    return {int(r[0]): np.array([float(v) for v in r[1:]]) for r in rows}


def _run(tmp_path, ref_dir, precision="fp64", steps=20):
    from examinimd_gb300 import MD
    deck, args = write_case(dict(CASES[NAME]), str(tmp_path))
    out = tmp_path / f"correctness_{precision}.txt"
    md = MD(["-il", deck, "--quiet", "--precision", precision] + args
            + ["--correctness", "20", str(ref_dir), str(out)])
    md.run(steps)
    md.close()
    return _report(out)


def test_fp64_report_is_zero_against_the_reference_dumps(tmp_path, golden):
    ref = tmp_path / "ref"
    ref.mkdir()
    _reference_dumps(golden, str(ref), (0, 20))
    rep = _run(tmp_path, ref)
    assert sorted(rep) == [0, 20]
    for s, r in rep.items():
        np.testing.assert_array_equal(r, np.zeros(6), err_msg=f"step {s}")


def test_report_finds_a_planted_difference_and_matches_rows_by_id(tmp_path, golden):
    ref = tmp_path / "ref"
    ref.mkdir()
    rng = np.random.default_rng(3)

    def edit(s, d):
        order = rng.permutation(len(d["id"]))  # rows in another order
        d = {k: v[order] for k, v in d.items()}
        if s == 20:
            d["x"][5, 1] += 1e-3
            d["f"][9, 2] -= 2e-3
        return d

    _reference_dumps(golden, str(ref), (0, 20), edit)
    rep = _run(tmp_path, ref)
    np.testing.assert_array_equal(rep[0], np.zeros(6))
    dr, mr, dv, mv, df, mf = rep[20]
    assert dv == 0.0 and mv == 0.0
    # the report prints %g (6 significant digits)
    assert dr == pytest.approx(1e-3, rel=1e-5) and mr == pytest.approx(1e-3, rel=1e-5)
    assert df == pytest.approx(2e-3, rel=1e-5) and mf == pytest.approx(2e-3, rel=1e-5)


def test_mixed_form_report_is_within_its_tolerance(tmp_path, golden):
    ref = tmp_path / "ref"
    ref.mkdir()
    _reference_dumps(golden, str(ref), (0, 20))
    rep = _run(tmp_path, ref, precision="mixed")
    g = golden(NAME)
    f0 = g["s0_f"]
    scale = np.sqrt(np.mean(np.sum(f0 * f0, axis=1)))
    dr, mr, dv, mv, df, mf = rep[0]
    assert dr == 0.0 and dv == 0.0  # the initial state is the same input
    assert mf <= 1e-4 * max(scale, 1.0)
    dr, mr, dv, mv, df, mf = rep[20]
    assert mr <= 1e-6 and mf <= 1e-3
