"""Force-matching harness over the GB300 SNAP and LJ adjoints.

A fit of SNAP's linear coefficients beta (or LJ's eps / sigma) to target
energies and forces.  The loss

    L = w_E * sum_c (E_c - E*_c)^2 / n_cfg + w_F * sum_c |F_c - F*_c|^2 / (3 N)

is a plain torch expression.  The energies and forces come from
`SnapEnergyForces` / `LJEnergyForces`, torch.autograd.Functions:

- forward runs the FP64 force and energy of every configuration through the C ABI;
- backward hands dL/dE and dL/dF to `emd_snap_adjoint` / `emd_lj_adjoint`, which return dL/dbeta
  (or dL/deps, dL/dsigma) in one pass per configuration.

Each configuration lives on its own `Context`: a periodic orthorhombic box,
one atom type, the neighbour list built once, with skin 0 and no MD.  Atom
order is the caller's: forces are returned, and dL/dF accepted, in the order
the positions were given.

This module is the only place torch autograd meets the library.  The
simulation path does not use it.
"""
from __future__ import annotations

from concurrent.futures import ThreadPoolExecutor

import numpy as np
import torch

from ._lib import EMD_NEIGH_CSR, EMD_PREC_FP64, Context

# ---------------------------------------------------------------- configurations


def lattice(style: str, a: float, n: int) -> np.ndarray:
    """Cubic lattice positions (bcc or fcc), n x n x n cells of side a."""
    basis = {"bcc": [(0, 0, 0), (0.5, 0.5, 0.5)],
             "fcc": [(0, 0, 0), (0.5, 0.5, 0), (0.5, 0, 0.5), (0, 0.5, 0.5)]}[style]
    g = np.stack(np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij"), -1).reshape(-1, 3)
    return ((g[:, None, :] + np.asarray(basis)[None]) * a).reshape(-1, 3)


def perturbed(style: str, a: float, n: int, rng: np.random.Generator, sigma: float, strain: float):
    """Lattice with Gaussian displacements (std `sigma`) and a random diagonal
    strain in [-strain, +strain] per axis; returns (positions in [0, L), box L)."""
    e = 1.0 + rng.uniform(-strain, strain, size=3)
    box = n * a * e
    x = lattice(style, a, n) * e + rng.normal(0.0, sigma, size=(2 if style == "bcc" else 4) * n ** 3 * 3).reshape(-1, 3)
    return np.mod(x, box), box


def snap_config_set(n_cfg=64, seed=20261205, a=3.1803, sigma=0.05, strain=0.02):
    """bcc tungsten configurations of uneven size: cells n^3 for n = 2..8 in turn
    (16 to 1,024 atoms), seeded displacements and strains."""
    rng = np.random.default_rng(seed)
    return [perturbed("bcc", a, 2 + (k % 7), rng, sigma, strain) for k in range(n_cfg)]


def lj_config_set(n_cfg=16, seed=20261206, rho=0.8442, sigma=0.05, strain=0.02):
    """fcc LJ configurations, cells n^3 for n = 5..10 in turn (500 to 4,000 atoms)."""
    rng = np.random.default_rng(seed)
    a = (4.0 / rho) ** (1.0 / 3.0)
    return [perturbed("fcc", a, 5 + (k % 6), rng, sigma, strain) for k in range(n_cfg)]


# ---------------------------------------------------------------- one configuration


class _Config:
    """A configuration on its own context: binning, halo and full list built once."""

    def __init__(self, x, box, cut, newton, device=0):
        self.n = len(x)
        self.box = np.asarray(box, float)
        if np.any(self.box <= cut):
            raise ValueError(f"box {self.box} not larger than the cutoff {cut} on every axis")
        self.ctx = Context(device)
        self.newton = newton
        c = self.ctx
        c.system_init([1.0], 1.0, 1.0, 0.001, self.box)
        c.set_local(np.asarray(x, float), np.zeros(self.n, np.int32), np.arange(1, self.n + 1, dtype=np.int32))
        self.cut = cut
        self._built = False

    def build(self):
        c, cut = self.ctx, self.cut
        c.comm_init(cut)
        c.neigh_init(EMD_NEIGH_CSR, cut, self.newton)
        c.comm_exchange()
        c.binning_create(cut, cut, cut, 1, True, False, True)
        c.comm_exchange_halo()
        c.binning_create(cut, cut, cut, 1, True, True, False)
        c.neigh_create(False)
        # the context's atom order (binning sorts) -> the caller's (ids 1..n)
        self.order = c.get(0, self.n, fields=("id",))["id"] - 1
        self._built = True

    def forces(self):
        """Forces on the owned atoms, in the caller's order."""
        c = self.ctx
        c.zero_forces()
        self._compute()
        if self.newton:
            c.comm_update_force()
        f = c.get(0, self.n, fields=("f",))["f"]
        out = np.empty_like(f)
        out[self.order] = f
        return out

    def to_ctx_order(self, g):
        return np.ascontiguousarray(np.asarray(g, float)[self.order])

    def close(self):
        self.ctx.close()


class SnapConfig(_Config):
    """FP64 SNAP on one configuration (one element, newton on)."""

    def __init__(self, x, box, params: dict, radius=0.5, weight=1.0, device=0):
        self.params = params
        self.radius, self.weight = radius, weight
        super().__init__(x, box, 2.0 * radius * float(params["rcutfac"]), True, device)

    def set_beta(self, beta):
        if self._built:  # tables and list in place: only the coefficients change
            self.ctx.snap_set_beta(np.asarray(beta, float)[None, :])
            return
        p = self.params
        self.ctx.snap_init(int(p["twojmax"]), float(p.get("rfac0", 0.99363)), float(p.get("rmin0", 0.0)),
                           int(p.get("switchflag", 1)), float(p["rcutfac"]), [self.radius], [self.weight],
                           np.asarray(beta, float)[None, :], [0], precision=EMD_PREC_FP64)
        # the forward pass keeps U_tot and Z for the adjoint of the backward pass
        self.ctx.snap_keep_for_adjoint(True)
        self.build()

    def _compute(self):
        # the energy of this configuration from the same FP64 pass
        self.ctx.snap_request_energy()
        self.ctx.snap_compute()

    def energy(self):
        e = self.ctx.snap_force_energy()
        return self.ctx.snap_energy() if e is None else e

    def adjoint(self, dL_dF, dL_dE, ncoeffall):
        return self.ctx.snap_adjoint(self.to_ctx_order(dL_dF), dL_dE, 1, ncoeffall)[0]


class LJConfig(_Config):
    """FP64 LJ (one type, cutoff fixed) on one configuration (full list)."""

    def __init__(self, x, box, cut=2.5, device=0):
        super().__init__(x, box, cut, False, device)

    def set_params(self, eps, sigma):
        lj1 = np.array([48.0 * eps * sigma ** 12])
        lj2 = np.array([24.0 * eps * sigma ** 6])
        self.ctx.lj_init(lj1, lj2, np.array([self.cut ** 2]), half=False, precision=EMD_PREC_FP64)
        if not self._built:
            self.build()

    def _compute(self):
        self.ctx.lj_compute()

    def energy(self):
        return self.ctx.lj_energy()

    def adjoint(self, dL_dF, dL_dE):
        return self.ctx.lj_adjoint(self.to_ctx_order(dL_dF), dL_dE)


# ---------------------------------------------------------------- autograd functions

# Configurations are small (tens to thousands of atoms), so one alone fills a
# few SMs.  Each lives on its own context and stream; running their calls from
# a pool of host threads (the C calls release the GIL) keeps many of them on
# the GPU at once.  Results are gathered in configuration order.
_POOL = ThreadPoolExecutor(max_workers=16)


def _each(fn, items):
    return list(_POOL.map(fn, items))



class SnapEnergyForces(torch.autograd.Function):
    """beta (ncoeffall,) -> (E (n_cfg,), F (sum N, 3)) over SnapConfigs."""

    @staticmethod
    def forward(ctx, beta, configs):
        b = beta.detach().cpu().numpy().astype(np.float64)

        def one(cfg):
            cfg.set_beta(b)
            return cfg.forces(), cfg.energy()

        res = _each(one, configs)
        fs, es = [r[0] for r in res], [r[1] for r in res]
        ctx.configs = configs
        ctx.ncoeffall = b.shape[0]
        return (torch.tensor(es, dtype=torch.float64), torch.tensor(np.concatenate(fs), dtype=torch.float64))

    @staticmethod
    def backward(ctx, gE, gF):
        gE = gE.detach().cpu().numpy()
        gF = gF.detach().cpu().numpy()
        offs = np.cumsum([0] + [cfg.n for cfg in ctx.configs])
        parts = _each(lambda k: ctx.configs[k].adjoint(gF[offs[k]:offs[k + 1]], float(gE[k]), ctx.ncoeffall),
                      range(len(ctx.configs)))
        grad = np.zeros(ctx.ncoeffall)
        for g in parts:  # summed in configuration order
            grad += g
        return torch.tensor(grad, dtype=torch.float64), None


class LJEnergyForces(torch.autograd.Function):
    """(eps, sigma) -> (E (n_cfg,), F (sum N, 3)) over LJConfigs."""

    @staticmethod
    def forward(ctx, params, configs):
        eps, sigma = (float(v) for v in params.detach().cpu().numpy())

        def one(cfg):
            cfg.set_params(eps, sigma)
            return cfg.forces(), cfg.energy()

        res = _each(one, configs)
        fs, es = [r[0] for r in res], [r[1] for r in res]
        ctx.configs = configs
        return (torch.tensor(es, dtype=torch.float64), torch.tensor(np.concatenate(fs), dtype=torch.float64))

    @staticmethod
    def backward(ctx, gE, gF):
        gE = gE.detach().cpu().numpy()
        gF = gF.detach().cpu().numpy()
        offs = np.cumsum([0] + [cfg.n for cfg in ctx.configs])
        parts = _each(lambda k: ctx.configs[k].adjoint(gF[offs[k]:offs[k + 1]], float(gE[k])),
                      range(len(ctx.configs)))
        grad = np.zeros(2)
        for g in parts:  # summed in configuration order
            grad += g
        return torch.tensor(grad, dtype=torch.float64), None


def loss_fn(E, F, E_ref, F_ref, w_E=1.0, w_F=1.0):
    """Weighted energy + force mean squared error (torch, differentiable)."""
    n_cfg, n_atoms = E.shape[0], F.shape[0]
    return w_E * torch.sum((E - E_ref) ** 2) / n_cfg + w_F * torch.sum((F - F_ref) ** 2) / (3 * n_atoms)


def synthetic_beta(seed: int, ncoeffall: int, beta0=-8.0, scale=0.1) -> np.ndarray:
    """beta_0 fixed, beta_1.. ~ N(0, scale) from `seed`."""
    return np.concatenate([[beta0], np.random.default_rng(seed).normal(0.0, scale, ncoeffall - 1)])


W_PARAMS = {"rcutfac": "4.73442", "twojmax": "8", "rfac0": "0.99363", "rmin0": "0", "switchflag": "1"}


def ncoeffall_for(twojmax: int) -> int:
    """1 + the number of bispectrum components with j >= j1 >= j2 (diagonalstyle 3)."""
    n = 0
    for j1 in range(twojmax + 1):
        for j2 in range(j1 + 1):
            for j in range(abs(j1 - j2), min(twojmax, j1 + j2) + 1, 2):
                if j >= j1:
                    n += 1
    return n + 1


__all__ = ["SnapConfig", "LJConfig", "SnapEnergyForces", "LJEnergyForces", "loss_fn", "snap_config_set",
           "lj_config_set", "synthetic_beta", "W_PARAMS", "ncoeffall_for", "lattice", "perturbed"]
