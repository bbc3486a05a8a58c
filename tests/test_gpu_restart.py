"""Checkpoint / resume through the --dumpbinary format (GPU).

A run dumped every 20 steps and a second run started from the step-20 dump
(--restart) must agree bit for bit at step 40: the dump holds the atom order,
positions and velocities of a rebuild step, and the restart rebuilds the
same halo, bins and neighbour list from them.
"""
import os

import numpy as np
import pytest

from tests.golden.decks import CASES, write_case

pytestmark = pytest.mark.gpu


def _read_dump(path):
    with open(path, "rb") as fp:
        n = int(np.fromfile(fp, np.int32, 1)[0])
        out = {"id": np.fromfile(fp, np.int32, n), "type": np.fromfile(fp, np.int32, n),
               "q": np.fromfile(fp, np.float64, n)}
        for k in ("x", "v", "f"):
            out[k] = np.fromfile(fp, np.float64, 3 * n).reshape(n, 3)
    return out


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_restart_from_dump_is_bit_identical(precision, tmp_path):
    from examinimd_gb300 import MD
    case = dict(CASES["lj_fcc6_full_csr"])
    deck, args = write_case(case, str(tmp_path))
    d1, d2 = tmp_path / "full", tmp_path / "resumed"
    d1.mkdir()
    d2.mkdir()
    base = ["-il", deck, "--quiet", "--precision", precision] + args
    md = MD(base + ["--dumpbinary", "20", str(d1)])
    md.run(40)
    md.close()
    dump20 = os.path.join(d1, "output.0000000020.000")
    md = MD(base + ["--dumpbinary", "20", str(d2), "--restart", dump20])
    assert md.info()["steps_done"] == 20
    md.run(20)
    md.close()
    for step in (20, 40):
        a = _read_dump(os.path.join(d1, f"output.{step:010d}.000"))
        b = _read_dump(os.path.join(d2, f"output.{step:010d}.000"))
        for k in ("id", "type", "q", "x", "v", "f"):
            np.testing.assert_array_equal(a[k], b[k], err_msg=f"{precision} step {step} {k}")
