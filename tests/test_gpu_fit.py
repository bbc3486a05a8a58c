"""Fitting adjoints (GPU, through the C ABI): SNAP dL/dbeta and LJ dL/d(eps,
sigma) against a gradient assembled from the FP64 forward path and against
central finite differences (h = 1e-6).

SNAP energy and forces are linear in beta, so the assembled gradient uses
unit coefficient vectors: E(e_k) - E(0) = sum_i B_ik and F(e_k) - F(0) is the
force field of component k.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _snap_setup(n_cfg=6):
    from examinimd_gb300 import fit
    ncoef = fit.ncoeffall_for(8)
    cfgs = [fit.SnapConfig(x, box, fit.W_PARAMS) for x, box in fit.snap_config_set(n_cfg)[:n_cfg]]
    beta_star = fit.synthetic_beta(7, ncoef)
    E_ref, F_ref = fit.SnapEnergyForces.apply(torch.tensor(beta_star), cfgs)
    return fit, cfgs, ncoef, E_ref.detach(), F_ref.detach()


def _snap_loss(fit, cfgs, beta, E_ref, F_ref):
    E, F = fit.SnapEnergyForces.apply(beta, cfgs)
    return fit.loss_fn(E, F, E_ref, F_ref, w_E=1e-2, w_F=1.0)


def test_snap_adjoint_vs_assembled_and_fd():
    fit, cfgs, ncoef, E_ref, F_ref = _snap_setup()
    beta = torch.tensor(fit.synthetic_beta(11, ncoef), requires_grad=True)
    loss = _snap_loss(fit, cfgs, beta, E_ref, F_ref)
    loss.backward()
    g = beta.grad.numpy().copy()
    assert np.all(np.isfinite(g)) and np.abs(g).max() > 0

    # assembled from the FP64 forward path
    with torch.no_grad():
        E, F = fit.SnapEnergyForces.apply(beta.detach(), cfgs)
        rE = 2e-2 * (E - E_ref).numpy() / len(cfgs)
        rF = 2.0 * (F - F_ref).numpy() / (3 * F.shape[0])
        E0, F0 = fit.SnapEnergyForces.apply(torch.zeros(ncoef, dtype=torch.float64), cfgs)
        ga = np.zeros(ncoef)
        for k in range(ncoef):
            ek = torch.zeros(ncoef, dtype=torch.float64)
            ek[k] = 1.0
            Ek, Fk = fit.SnapEnergyForces.apply(ek, cfgs)
            ga[k] = np.dot(rE, (Ek - E0).numpy()) + np.sum(rF * (Fk - F0).numpy())
    scale = np.abs(ga).max()
    assert np.abs(g - ga).max() <= 1e-9 * scale, np.abs(g - ga).max() / scale

    # central finite differences on a spread of coefficients
    h = 1e-6
    for k in (0, 1, 5, 17, 33, ncoef - 1):
        with torch.no_grad():
            bp, bm = beta.detach().clone(), beta.detach().clone()
            bp[k] += h
            bm[k] -= h
            fd = (_snap_loss(fit, cfgs, bp, E_ref, F_ref) - _snap_loss(fit, cfgs, bm, E_ref, F_ref)).item() / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 * max(abs(g[k]), 1e-3 * scale), (k, fd, g[k])
    for c in cfgs:
        c.close()


def test_snap_adjoint_from_kept_phases_is_bit_identical():
    """On one force pass and the same dL/dF, the adjoint reading the U_tot and
    Z that the force pass kept gives the bits of one that recomputes them
    (two force passes would not do: the pair forces reach j through FP64
    atomics, so forces, and a loss gradient built from them, can differ in
    the last bit from pass to pass).  After the positions move, the kept copy
    is stale and the adjoint recomputes."""
    fit, cfgs, ncoef, E_ref, F_ref = _snap_setup(3)
    beta = torch.tensor(fit.synthetic_beta(11, ncoef))
    rng = np.random.default_rng(3)
    for c in cfgs:
        gF = rng.normal(size=(c.n, 3))
        c.ctx.snap_keep_for_adjoint(True)
        with torch.no_grad():
            fit.SnapEnergyForces.apply(beta, [c])  # the force pass keeps U_tot and Z
        g_kept = c.adjoint(gF, 0.5, ncoef)
        g_again = c.adjoint(gF, 0.5, ncoef)
        c.ctx.snap_keep_for_adjoint(False)
        g_fresh = c.adjoint(gF, 0.5, ncoef)
        np.testing.assert_array_equal(g_kept, g_fresh)
        np.testing.assert_array_equal(g_again, g_fresh)
    c = cfgs[0]
    n = c.n
    gF = rng.normal(size=(n, 3))
    c.ctx.snap_keep_for_adjoint(True)
    with torch.no_grad():
        fit.SnapEnergyForces.apply(beta, [c])
    g_kept = c.adjoint(gF, 0.5, ncoef)
    c.ctx.update(0, x=c.ctx.get(0, n)["x"] + rng.uniform(-1e-3, 1e-3, (n, 3)))  # moved: the kept copy is stale
    g_moved = c.adjoint(gF, 0.5, ncoef)
    c.ctx.snap_keep_for_adjoint(False)
    g_fresh = c.adjoint(gF, 0.5, ncoef)
    np.testing.assert_array_equal(g_moved, g_fresh)
    assert not np.array_equal(g_kept, g_moved)
    for c in cfgs:
        c.close()


def test_lj_adjoint_vs_fd():
    from examinimd_gb300 import fit
    cfgs = [fit.LJConfig(x, box) for x, box in fit.lj_config_set(3)]
    E_ref, F_ref = fit.LJEnergyForces.apply(torch.tensor([1.05, 0.98], dtype=torch.float64), cfgs)
    E_ref, F_ref = E_ref.detach(), F_ref.detach()

    def loss(p):
        E, F = fit.LJEnergyForces.apply(p, cfgs)
        return fit.loss_fn(E, F, E_ref, F_ref, w_E=1e-3, w_F=1.0)

    p = torch.tensor([1.0, 1.0], dtype=torch.float64, requires_grad=True)
    loss(p).backward()
    g = p.grad.numpy().copy()
    h = 1e-6
    for k in range(2):
        with torch.no_grad():
            pp, pm = p.detach().clone(), p.detach().clone()
            pp[k] += h
            pm[k] -= h
            fd = (loss(pp) - loss(pm)).item() / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 * abs(g[k]), (k, fd, g[k])
    for c in cfgs:
        c.close()
