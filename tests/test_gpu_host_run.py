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


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_run_host_equals_update_run_get(precision, tmp_path):
    from examinimd_gb300 import MD
    case = dict(CASES["lj_fcc6_full_csr"])
    deck, args = write_case(case, str(tmp_path))
    args = args + ["--precision", precision]
    a, b = MD(["-il", deck, "--quiet"] + args), MD(["-il", deck, "--quiet"] + args)
    n = a.info()["N_local"]
    ref = a.ctx.get(0, n)
    hx, hv, hf = (np.ascontiguousarray(ref[k]) for k in ("x", "v", "f"))
    steps = 25  # the rebuild at step 20 re-sorts the atoms in between
    for _ in range(steps):
        a.ctx.update(0, hx, hv, hf)
        a.run(1)
        cur = a.ctx.get(0, n)
        hx, hv, hf = (np.ascontiguousarray(cur[k]) for k in ("x", "v", "f"))
    st = b.ctx.get(0, n)
    bx, bv, bf = (np.ascontiguousarray(st[k]) for k in ("x", "v", "f"))
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
