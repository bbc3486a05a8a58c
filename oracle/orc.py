"""ctypes bindings for the CPU oracle -- TEST INFRASTRUCTURE ONLY.

`Oracle` exposes the same methods as examinimd_gb300.Context (orc_* for
emd_*), so a test can run the same call sequence on both and compare.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import build as _build

_P, _I, _D = C.c_void_p, C.c_int, C.c_double
_DP, _IP, _LLP = C.POINTER(C.c_double), C.POINTER(C.c_int), C.POINTER(C.c_longlong)
_lib = None

_SIGS = {
    "orc_create": ([], _P), "orc_destroy": ([_P], None), "orc_last_error": ([_P], C.c_char_p),
    "orc_set_threads": ([_P, _I], None),
    "orc_system_init": ([_P, _I, _DP, _D, _D, _D, _DP, _DP, _DP], _I),
    "orc_system_set_local": ([_P, _I, _DP, _DP, _DP, _IP, _IP, _DP], _I),
    "orc_system_get": ([_P, _I, _I, _DP, _DP, _DP, _IP, _IP, _DP], _I),
    "orc_system_info": ([_P, _IP, _IP], _I), "orc_zero_forces": ([_P], _I),
    "orc_create_lattice": ([_P, _I, _D, _DP, _I, _I, _I, _D, _I], _I),
    "orc_nve_initial": ([_P], _I), "orc_nve_final": ([_P], _I),
    "orc_comm_init": ([_P, _D], _I), "orc_comm_exchange": ([_P], _I),
    "orc_comm_exchange_halo": ([_P, _IP], _I), "orc_comm_update_halo": ([_P], _I),
    "orc_comm_update_force": ([_P], _I), "orc_comm_get_ghosts": ([_P, _IP, _IP], _I),
    "orc_binning_create": ([_P, _D, _D, _D, _I, _I, _I, _I, _IP], _I),
    "orc_binning_get": ([_P, _IP, _IP, _IP, _DP], _I),
    "orc_neigh_init": ([_P, _I, _D, _I], _I), "orc_neigh_create": ([_P, _I, _LLP], _I),
    "orc_neigh_get": ([_P, _IP, _IP], _I), "orc_neigh_maxneighs": ([_P, _IP], _I),
    "orc_lj_init": ([_P, _I, _DP, _DP, _DP, _I], _I), "orc_lj_compute": ([_P], _I),
    "orc_lj_energy": ([_P, _DP], _I), "orc_lj_energy_compensated": ([_P, _DP], _I),
    "orc_snap_init": ([_P, _I, _D, _D, _I, _D, _I, _DP, _DP, _DP, _I, _I, _IP], _I),
    "orc_snap_compute": ([_P], _I), "orc_snap_energy": ([_P, _DP], _I),
    "orc_snap_bispectrum": ([_P, _DP], _I), "orc_snap_ncoeff": ([_P, _IP], _I),
    "orc_thermo_mv2": ([_P, _DP], _I),
}


def load():
    global _lib
    if _lib is None:
        lib = C.CDLL(_build.build_oracle())
        for k, (a, r) in _SIGS.items():
            fn = getattr(lib, k)
            fn.argtypes = a
            fn.restype = r
        _lib = lib
    return _lib


def _dp(a):
    return None if a is None else a.ctypes.data_as(_DP)


def _ip(a):
    return None if a is None else a.ctypes.data_as(_IP)


def _f64(a, shape=None):
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a if shape is None else a.reshape(shape)


def _i32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.int32)


class Oracle:
    def __init__(self, threads: int = 1):
        self.lib = load()
        self.h = _P(self.lib.orc_create())
        self.lib.orc_set_threads(self.h, threads)

    def __del__(self):
        try:
            if self.h:
                self.lib.orc_destroy(self.h)
                self.h = None
        except Exception:
            pass

    def _ok(self, st, what):
        if st != 0:
            raise RuntimeError(f"{what}: {self.lib.orc_last_error(self.h).decode()}")

    def system_init(self, mass, boltz, mvv2e, dt, domain, sub_lo=(0, 0, 0), sub_hi=None):
        mass = _f64(mass)
        dom, lo = _f64(domain), _f64(sub_lo)
        hi = _f64(domain if sub_hi is None else sub_hi)
        self._ok(self.lib.orc_system_init(self.h, len(mass), _dp(mass), boltz, mvv2e, dt, _dp(dom), _dp(lo), _dp(hi)),
                 "orc_system_init")

    def create_lattice(self, style, a, nx, ny, nz, t_target, seed, offset=(0.0, 0.0, 0.0)):
        off = _f64(offset)
        self._ok(self.lib.orc_create_lattice(self.h, style, a, _dp(off), nx, ny, nz, t_target, seed),
                 "orc_create_lattice")

    def set_local(self, x, type_, id_, v=None, f=None, q=None):
        x = _f64(x, (-1, 3))
        self._ok(self.lib.orc_system_set_local(self.h, x.shape[0], _dp(x), _dp(_f64(v, (-1, 3))),
                                               _dp(_f64(f, (-1, 3))), _ip(_i32(type_)), _ip(_i32(id_)), _dp(_f64(q))),
                 "orc_system_set_local")

    def info(self):
        a, b = _I(), _I()
        self._ok(self.lib.orc_system_info(self.h, C.byref(a), C.byref(b)), "orc_system_info")
        return a.value, b.value, a.value + b.value

    def get(self, first=0, count=None, fields=("x", "v", "f", "type", "id", "q")):
        nl, ng, _ = self.info()
        if count is None:
            count = nl - first
        x = np.empty((count, 3)) if "x" in fields else None
        v = np.empty((count, 3)) if "v" in fields else None
        f = np.empty((count, 3)) if "f" in fields else None
        t = np.empty(count, np.int32) if "type" in fields else None
        i = np.empty(count, np.int32) if "id" in fields else None
        q = np.empty(count) if "q" in fields else None
        self._ok(self.lib.orc_system_get(self.h, first, count, _dp(x), _dp(v), _dp(f), _ip(t), _ip(i), _dp(q)),
                 "orc_system_get")
        return {k: a for k, a in (("x", x), ("v", v), ("f", f), ("type", t), ("id", i), ("q", q)) if a is not None}

    def zero_forces(self):
        self._ok(self.lib.orc_zero_forces(self.h), "orc_zero_forces")

    def nve_initial(self):
        self._ok(self.lib.orc_nve_initial(self.h), "orc_nve_initial")

    def nve_final(self):
        self._ok(self.lib.orc_nve_final(self.h), "orc_nve_final")

    def comm_init(self, depth):
        self._ok(self.lib.orc_comm_init(self.h, depth), "orc_comm_init")

    def comm_exchange(self):
        self._ok(self.lib.orc_comm_exchange(self.h), "orc_comm_exchange")

    def comm_exchange_halo(self):
        n = _I()
        self._ok(self.lib.orc_comm_exchange_halo(self.h, C.byref(n)), "orc_comm_exchange_halo")
        return n.value

    def comm_update_halo(self):
        self._ok(self.lib.orc_comm_update_halo(self.h), "orc_comm_update_halo")

    def comm_update_force(self):
        self._ok(self.lib.orc_comm_update_force(self.h), "orc_comm_update_force")

    def comm_ghosts(self):
        ng = (C.c_int * 6)()
        self._ok(self.lib.orc_comm_get_ghosts(self.h, ng, None), "orc_comm_get_ghosts")
        counts = np.array(list(ng), np.int32)
        pack = np.empty(max(int(counts.sum()), 1), np.int32)
        self._ok(self.lib.orc_comm_get_ghosts(self.h, ng, _ip(pack)), "orc_comm_get_ghosts")
        return counts, pack[:int(counts.sum())]

    def binning_create(self, dx, dy, dz, halo=1, do_local=True, do_ghost=False, sort=False):
        nb = (C.c_int * 3)()
        self._ok(self.lib.orc_binning_create(self.h, dx, dy, dz, halo, int(do_local), int(do_ghost), int(sort), nb),
                 "orc_binning_create")
        return tuple(nb)

    def binning_get(self, nbins, count):
        bc, bo = np.empty(nbins, np.int32), np.empty(nbins, np.int32)
        perm, b = np.empty(max(count, 1), np.int32), np.empty(6)
        self._ok(self.lib.orc_binning_get(self.h, _ip(bc), _ip(bo), _ip(perm), _dp(b)), "orc_binning_get")
        return bc, bo, perm[:count], b

    def neigh_init(self, kind, cut, newton=False):
        self._ok(self.lib.orc_neigh_init(self.h, kind, cut, int(newton)), "orc_neigh_init")

    def neigh_create(self, half=False):
        t = C.c_longlong()
        self._ok(self.lib.orc_neigh_create(self.h, int(half), C.byref(t)), "orc_neigh_create")
        return t.value

    def neigh_get(self, total=None):
        """Row lengths and entries (every entry is written: without `total`
        the lengths are read first to size the buffer)."""
        nl, _, _ = self.info()
        num = np.empty(max(nl, 1), np.int32)
        if total is None:
            self._ok(self.lib.orc_neigh_get(self.h, _ip(num), None), "orc_neigh_get")
            total = int(num[:nl].sum())
        ent = np.empty(max(total, 1), np.int32)
        self._ok(self.lib.orc_neigh_get(self.h, _ip(num), _ip(ent)), "orc_neigh_get")
        return num[:nl], ent[:total]

    def neigh_maxneighs(self):
        m = _I()
        self._ok(self.lib.orc_neigh_maxneighs(self.h, C.byref(m)), "orc_neigh_maxneighs")
        return m.value

    def lj_init(self, lj1, lj2, cutsq, half=False, precision=0):
        lj1, lj2, cutsq = _f64(lj1), _f64(lj2), _f64(cutsq)
        nt = int(round(np.sqrt(lj1.size)))
        self._ok(self.lib.orc_lj_init(self.h, nt, _dp(lj1), _dp(lj2), _dp(cutsq), int(half)), "orc_lj_init")

    def lj_compute(self):
        self._ok(self.lib.orc_lj_compute(self.h), "orc_lj_compute")

    def lj_energy(self):
        e = _D()
        self._ok(self.lib.orc_lj_energy(self.h, C.byref(e)), "orc_lj_energy")
        return e.value

    def lj_energy_compensated(self):
        """The reference's pair terms summed with compensation (no serial-sum rounding)."""
        e = _D()
        self._ok(self.lib.orc_lj_energy_compensated(self.h, C.byref(e)), "orc_lj_energy_compensated")
        return e.value

    def snap_init(self, twojmax, rfac0, rmin0, switchflag, rcutfac, radelem, wjelem, beta, type_map, precision=0):
        radelem, wjelem = _f64(radelem), _f64(wjelem)
        beta = _f64(beta, (len(radelem), -1))
        tmap = _i32(type_map)
        self._ok(self.lib.orc_snap_init(self.h, twojmax, rfac0, rmin0, switchflag, rcutfac, len(radelem),
                                        _dp(radelem), _dp(wjelem), _dp(beta), beta.shape[1], len(tmap), _ip(tmap)),
                 "orc_snap_init")

    def snap_compute(self):
        self._ok(self.lib.orc_snap_compute(self.h), "orc_snap_compute")

    def snap_energy(self):
        e = _D()
        self._ok(self.lib.orc_snap_energy(self.h, C.byref(e)), "orc_snap_energy")
        return e.value

    def snap_bispectrum(self):
        nl, _, _ = self.info()
        n = _I()
        self._ok(self.lib.orc_snap_ncoeff(self.h, C.byref(n)), "orc_snap_ncoeff")
        b = np.empty((nl, n.value))
        self._ok(self.lib.orc_snap_bispectrum(self.h, _dp(b)), "orc_snap_bispectrum")
        return b

    def thermo_mv2(self):
        e = _D()
        self._ok(self.lib.orc_thermo_mv2(self.h, C.byref(e)), "orc_thermo_mv2")
        return e.value
