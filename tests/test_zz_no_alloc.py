"""emd_lj_energy_noalloc against emd_lj_energy (GPU, through the C ABI).

The allocation-free entry point runs the same kernels and summation order on
a fixed array inside the library, so its energy must equal the allocating
entry point's.  Each check makes two calls in a row (the first one also looks
up the array's device address).  The file sorts last so that the check also
runs after every other GPU test has used the device.
"""
import numpy as np
import pytest

from tests import mdloop

pytestmark = pytest.mark.gpu

# both entry points reduce in the same fixed order: identical up to this
# relative tolerance (zero in practice)
RTOL = 1e-14


def _lj_system(n, precision, half=False, kind=0):
    from examinimd_gb300 import Context
    setup = mdloop.LJSetup(n, half=half, kind=kind)
    state = mdloop.make_lattice(setup)
    ctx = Context(0)
    mdloop.init(ctx, setup, state, precision=precision)
    for s in range(1, 4):
        mdloop.step(ctx, setup, s)
    return ctx


@pytest.mark.parametrize("precision,half,kind", [(0, False, 0), (0, True, 1), (1, False, 0)])
def test_noalloc_energy_matches_lj_energy(precision, half, kind):
    ctx = _lj_system(6, precision, half=half, kind=kind)
    for _ in range(2):
        ref = ctx.lj_energy()
        got = ctx.lj_energy_noalloc()
        assert np.isfinite(ref) and ref < 0.0
        assert abs(got - ref) <= RTOL * abs(ref), (got, ref)
    # and twice in a row on its own, with no device allocation in the library
    from examinimd_gb300._lib import device_allocations
    n0 = device_allocations()
    a = ctx.lj_energy_noalloc()
    b = ctx.lj_energy_noalloc()
    assert a == b
    assert device_allocations() == n0
    ctx.close()


def test_noalloc_energy_rejects_more_atoms_than_its_scratch():
    from examinimd_gb300 import Context, EmdError
    from examinimd_gb300._lib import EMD_LJ_ENERGY_NOALLOC_MAX_LOCAL as cap
    n = cap + 1
    ctx = Context(0)
    side = 200.0
    ctx.system_init([1.0], 1.0, 1.0, 0.005, [side] * 3)
    rng = np.random.default_rng(5)
    x = rng.uniform(0.0, side, size=(n, 3))
    ctx.set_local(x, np.zeros(n, np.int32), np.arange(1, n + 1, dtype=np.int32))
    with pytest.raises(EmdError, match="4,194,304"):
        ctx.lj_energy_noalloc()
    ctx.close()
