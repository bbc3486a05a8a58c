"""ctypes bindings for libemd_gb300.so (include/emd_gpu.h, include/emd_driver.h)."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
EMD_PREC_FP64, EMD_PREC_MIXED = 0, 1
# emd_status codes (include/emd_gpu.h); a latched device status word holds bit (1 << code)
(EMD_OK, EMD_ERR_OVERFLOW_GHOST, EMD_ERR_OVERFLOW_NEIGH, EMD_ERR_TIMEOUT, EMD_ERR_BOUNDS, EMD_ERR_CUDA, EMD_ERR_ARG,
 EMD_ERR_STATE, EMD_ERR_NOMEM) = range(9)
EMD_NEIGH_CSR, EMD_NEIGH_2D = 0, 1
EMD_LJ_ENERGY_NOALLOC_MAX_LOCAL = 4194304  # include/emd_gpu.h

_lib = None


class EmdError(RuntimeError):
    pass


def library_path() -> str:
    return os.path.join(HERE, "libemd_gb300.so")


_P = C.c_void_p
_I = C.c_int
_D = C.c_double
_DP = C.POINTER(C.c_double)
_IP = C.POINTER(C.c_int)
_LLP = C.POINTER(C.c_longlong)

_SIGS = {
    "emd_abi_version": ([], _I),
    "emd_create": ([C.POINTER(_P), _I], _I),
    "emd_destroy": ([_P], None),
    "emd_status_string": ([_I], C.c_char_p),
    "emd_last_error": ([_P], C.c_char_p),
    "emd_stream": ([_P], _P),
    "emd_synchronize": ([_P], _I),
    "emd_get_status": ([_P, C.POINTER(C.c_uint)], _I),
    "emd_device_allocations": ([C.POINTER(C.c_ulonglong)], _I),
    "emd_system_init": ([_P, _I, _DP, _D, _D, _D, _DP, _DP, _DP], _I),
    "emd_system_grow": ([_P, _I], _I),
    "emd_system_set_local": ([_P, _I, _DP, _DP, _DP, _IP, _IP, _DP], _I),
    "emd_system_update": ([_P, _I, _I, _DP, _DP, _DP], _I),
    "emd_system_get": ([_P, _I, _I, _DP, _DP, _DP, _IP, _IP, _DP], _I),
    "emd_system_info": ([_P, _IP, _IP, _IP], _I),
    "emd_system_download": ([_P, _I, _DP], _I),
    "emd_system_download_wait": ([_P], _I),
    "emd_system_stage": ([_P, _I, _DP], _I),
    "emd_system_commit": ([_P], _I),
    "emd_system_download_range": ([_P, _I, _DP, _I, _I], _I),
    "emd_system_stage_range": ([_P, _I, _DP, _I, _I], _I),
    "emd_system_commit_range": ([_P, _I, _I], _I),
    "emd_zero_forces": ([_P], _I),
    "emd_nve_initial": ([_P], _I),
    "emd_nve_final": ([_P], _I),
    "emd_nve_initial_range": ([_P, _I, _I], _I),
    "emd_comm_init": ([_P, _D], _I),
    "emd_comm_exchange": ([_P], _I),
    "emd_comm_exchange_halo": ([_P, _IP], _I),
    "emd_comm_update_halo": ([_P], _I),
    "emd_comm_update_force": ([_P], _I),
    "emd_comm_get_ghosts": ([_P, _IP, _IP], _I),
    "emd_binning_create": ([_P, _D, _D, _D, _I, _I, _I, _I, _IP], _I),
    "emd_binning_get": ([_P, _IP, _IP, _IP, _DP], _I),
    "emd_neigh_init": ([_P, _I, _D, _I], _I),
    "emd_neigh_create": ([_P, _I, _LLP], _I),
    "emd_neigh_get": ([_P, _IP, _IP], _I),
    "emd_neigh_maxneighs": ([_P, _IP], _I),
    "emd_lj_init": ([_P, _I, _DP, _DP, _DP, _I, _I], _I),
    "emd_lj_compute": ([_P], _I),
    "emd_lj_energy": ([_P, _DP], _I),
    "emd_lj_energy_noalloc": ([_P, _DP], _I),
    "emd_lj_request_energy": ([_P], _I),
    "emd_snap_request_energy": ([_P], _I),
    "emd_snap_force_energy": ([_P, _DP, _IP], _I),
    "emd_lj_force_energy": ([_P, _DP, _IP], _I),
    "emd_lj_energy_mixed": ([_P, _DP, _IP], _I),
    "emd_lj_adjoint": ([_P, _DP, _D, _DP], _I),
    "emd_batch_create": ([C.POINTER(_P), _I, _I, _IP, _DP, _DP, _DP, _D, _D, _D, _D, _D, _D, _I, _I, _D], _I),
    "emd_batch_destroy": ([_P], None),
    "emd_batch_last_error": ([_P], C.c_char_p),
    "emd_batch_run": ([_P, _I], _I),
    "emd_batch_set_shape": ([_P, _I, _I], _I),
    "emd_batch_tune": ([_P, _I, _IP, _IP], _I),
    "emd_batch_get": ([_P, _DP, _DP, _DP], _I),
    "emd_batch_thermo": ([_P, _DP, _DP], _I),
    "emd_batch_info": ([_P, _LLP, _IP, _IP, _LLP], _I),
    "emd_batch_stream": ([_P], _P),
    "emd_snap_adjoint": ([_P, _DP, _D, _DP], _I),
    "emd_snap_init": ([_P, _I, _D, _D, _I, _D, _I, _DP, _DP, _DP, _I, _I, _IP, _I], _I),
    "emd_snap_info": ([_P, _IP, _IP], _I),
    "emd_snap_keep_for_adjoint": ([_P, _I], _I),
    "emd_snap_set_beta": ([_P, _DP], _I),
    "emd_snap_compute": ([_P], _I),
    "emd_snap_energy": ([_P, _DP], _I),
    "emd_snap_ncoeff": ([_P, _IP], _I),
    "emd_thermo_mv2": ([_P, _DP], _I),
    "emd_timing_enable": ([_P, _I], _I),
    "emd_timing_only": ([_P, C.c_char_p], _I),
    "emd_timing_reset": ([_P], _I),
    "emd_timing_report": ([_P, C.c_char_p, _I], _I),
    "emd_timing_get": ([_P, C.c_char_p, _DP, _LLP], _I),
    "emd_md_create": ([_I, C.POINTER(C.c_char_p), C.c_char_p, _I], _P),
    "emd_md_run": ([_P, _I], _I),
    "emd_md_run_host": ([_P, _I, _DP, _DP, _DP], _I),
    "emd_md_destroy": ([_P], None),
    "emd_md_error": ([_P], C.c_char_p),
    "emd_md_ctx": ([_P], _P),
    "emd_md_info": ([_P, _IP, _IP, _IP, _IP, _IP], _I),
    "emd_md_thermo": ([_P, _DP, _DP, _DP], _I),
    "emd_md_compute_thermo": ([_P, _DP, _DP, _DP], _I),
    "emd_md_timers": ([_P, _DP], _I),
}


def load_library(path: str | None = None):
    """Loads libemd_gb300.so; raises if it has not been built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or library_path()
    if not os.path.exists(p):
        raise EmdError(f"{p} not found: build it with `python -m examinimd_gb300.build` (no CPU fallback exists)")
    lib = C.CDLL(p)
    for name, (args, res) in _SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    if path is None:
        _lib = lib
    return lib


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


def device_allocations() -> int:
    """Device allocations the library has made in this process (emd_device_allocations)."""
    n = C.c_ulonglong()
    if load_library().emd_device_allocations(C.byref(n)) != 0:
        raise EmdError("emd_device_allocations failed")
    return n.value


class Context:
    """One emd_ctx: device-resident particle system and module state."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        h = _P()
        st = self.lib.emd_create(C.byref(h), device)
        if st != 0:
            raise EmdError(f"emd_create failed: {self.lib.emd_status_string(st).decode()}")
        self.h = h

    def close(self):
        if self.h:
            self.lib.emd_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ok(self, st, what):
        if st != 0:
            msg = self.lib.emd_last_error(self.h).decode()
            raise EmdError(f"{what}: {self.lib.emd_status_string(st).decode()} ({msg})")

    @property
    def stream(self) -> int:
        return int(self.lib.emd_stream(self.h) or 0)

    def synchronize(self):
        self._ok(self.lib.emd_synchronize(self.h), "emd_synchronize")

    def status(self) -> int:
        f = C.c_uint()
        self._ok(self.lib.emd_get_status(self.h, C.byref(f)), "emd_get_status")
        return f.value

    # ---- System
    def system_init(self, mass, boltz, mvv2e, dt, domain, sub_lo=(0, 0, 0), sub_hi=None):
        mass = _f64(mass)
        dom = _f64(domain)
        lo = _f64(sub_lo)
        hi = _f64(domain if sub_hi is None else sub_hi)
        if dom.size != 3 or lo.size != 3 or hi.size != 3:
            raise EmdError("system_init: domain, sub_lo and sub_hi need three components each")
        self._ok(self.lib.emd_system_init(self.h, len(mass), _dp(mass), boltz, mvv2e, dt, _dp(dom), _dp(lo), _dp(hi)),
                 "emd_system_init")

    def set_local(self, x, type_, id_, v=None, f=None, q=None):
        x = _f64(x, (-1, 3))
        n = x.shape[0]
        v, f, q = _f64(v, (-1, 3)), _f64(f, (-1, 3)), _f64(q)
        t, i = _i32(type_), _i32(id_)
        # the library reads n rows of every array it is given
        for name, a, rows in (("v", v, n), ("f", f, n), ("q", q, n), ("type", t, n), ("id", i, n)):
            if a is not None and a.shape[0] != rows:
                raise EmdError(f"set_local: {name} must have {rows} rows like x")
        self._ok(self.lib.emd_system_set_local(self.h, n, _dp(x), _dp(v), _dp(f), _ip(t), _ip(i), _dp(q)),
                 "emd_system_set_local")

    def info(self):
        a, b, c = _I(), _I(), _I()
        self._ok(self.lib.emd_system_info(self.h, C.byref(a), C.byref(b), C.byref(c)), "emd_system_info")
        return a.value, b.value, c.value

    def get(self, first=0, count=None, fields=("x", "v", "f", "type", "id", "q")):
        nl, ng, _ = self.info()
        if count is None:
            count = nl - first
        out = {}
        x = np.empty((count, 3)) if "x" in fields else None
        v = np.empty((count, 3)) if "v" in fields else None
        f = np.empty((count, 3)) if "f" in fields else None
        t = np.empty(count, np.int32) if "type" in fields else None
        i = np.empty(count, np.int32) if "id" in fields else None
        q = np.empty(count) if "q" in fields else None
        self._ok(self.lib.emd_system_get(self.h, first, count, _dp(x), _dp(v), _dp(f), _ip(t), _ip(i), _dp(q)),
                 "emd_system_get")
        for k, a in (("x", x), ("v", v), ("f", f), ("type", t), ("id", i), ("q", q)):
            if a is not None:
                out[k] = a
        return out

    def update(self, first=0, x=None, v=None, f=None):
        """emd_system_update: overwrites rows [first, first + len) of the owned
        particles' x, v, f (None = unchanged)."""
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (x, v, f)]
        n = next((a.shape[0] for a in arrs if a is not None), 0)
        if any(a is not None and a.shape != (n, 3) for a in arrs):
            raise EmdError(f"update: x, v, f must all have shape ({n}, 3)")
        self._ok(self.lib.emd_system_update(self.h, first, n, *[_dp(a) for a in arrs]), "emd_system_update")

    def stage(self, field, arr):
        """emd_system_stage: queues the upload of x (0), v (1) or f (2) of the
        owned particles from ``arr`` (N_local x 3 float64, C order, kept alive
        and unwritten until a later synchronisation); applied by commit()."""
        if not (isinstance(arr, np.ndarray) and arr.dtype == np.float64 and arr.flags.c_contiguous):
            raise TypeError("stage: a C-contiguous float64 array is required")
        n = self.info()[0]
        if arr.shape != (n, 3):
            raise EmdError(f"stage: the array must hold the {n} owned rows, shape ({n}, 3)")
        self._ok(self.lib.emd_system_stage(self.h, field, _dp(arr)), "emd_system_stage")

    def commit(self):
        """emd_system_commit: moves every staged field into place."""
        self._ok(self.lib.emd_system_commit(self.h), "emd_system_commit")

    def stage_range(self, field, arr, first):
        """emd_system_stage_range: queues the upload of rows [first, first +
        len(arr)) of x (0), v (1) or f (2) from ``arr`` (kept alive and
        unwritten until a later synchronisation)."""
        if not (isinstance(arr, np.ndarray) and arr.dtype == np.float64 and arr.flags.c_contiguous
                and arr.ndim == 2 and arr.shape[1] == 3):
            raise TypeError("stage_range: a C-contiguous float64 array of shape (rows, 3) is required")
        self._ok(self.lib.emd_system_stage_range(self.h, field, _dp(arr), first, arr.shape[0]),
                 "emd_system_stage_range")

    def commit_range(self, first, count):
        """emd_system_commit_range: moves the rows staged inside [first,
        first + count) into place."""
        self._ok(self.lib.emd_system_commit_range(self.h, first, count), "emd_system_commit_range")

    def zero_forces(self):
        self._ok(self.lib.emd_zero_forces(self.h), "emd_zero_forces")

    # ---- modules
    def nve_initial(self):
        self._ok(self.lib.emd_nve_initial(self.h), "emd_nve_initial")

    def nve_final(self):
        self._ok(self.lib.emd_nve_final(self.h), "emd_nve_final")

    def nve_initial_range(self, first, count):
        self._ok(self.lib.emd_nve_initial_range(self.h, first, count), "emd_nve_initial_range")

    def comm_init(self, depth):
        self._ok(self.lib.emd_comm_init(self.h, depth), "emd_comm_init")

    def comm_exchange(self):
        self._ok(self.lib.emd_comm_exchange(self.h), "emd_comm_exchange")

    def comm_exchange_halo(self) -> int:
        n = _I()
        self._ok(self.lib.emd_comm_exchange_halo(self.h, C.byref(n)), "emd_comm_exchange_halo")
        return n.value

    def comm_update_halo(self):
        self._ok(self.lib.emd_comm_update_halo(self.h), "emd_comm_update_halo")

    def comm_update_force(self):
        self._ok(self.lib.emd_comm_update_force(self.h), "emd_comm_update_force")

    def comm_ghosts(self):
        ng = (C.c_int * 6)()
        self._ok(self.lib.emd_comm_get_ghosts(self.h, ng, None), "emd_comm_get_ghosts")
        counts = np.array(list(ng), np.int32)
        pack = np.empty(int(counts.sum()), np.int32)
        self._ok(self.lib.emd_comm_get_ghosts(self.h, ng, _ip(pack)), "emd_comm_get_ghosts")
        return counts, pack

    def binning_create(self, dx, dy, dz, halo=1, do_local=True, do_ghost=False, sort=False):
        nb = (C.c_int * 3)()
        self._ok(self.lib.emd_binning_create(self.h, dx, dy, dz, halo, int(do_local), int(do_ghost), int(sort), nb),
                 "emd_binning_create")
        return tuple(nb)

    def binning_get(self, nbins: int, count: int):
        bc = np.empty(nbins, np.int32)
        bo = np.empty(nbins, np.int32)
        perm = np.empty(max(count, 1), np.int32)
        b = np.empty(6)
        self._ok(self.lib.emd_binning_get(self.h, _ip(bc), _ip(bo), _ip(perm), _dp(b)), "emd_binning_get")
        return bc, bo, perm[:count], b

    def neigh_init(self, kind, cut, newton=False):
        self._ok(self.lib.emd_neigh_init(self.h, kind, cut, int(newton)), "emd_neigh_init")

    def neigh_create(self, half=False) -> int:
        t = C.c_longlong()
        self._ok(self.lib.emd_neigh_create(self.h, int(half), C.byref(t)), "emd_neigh_create")
        return t.value

    def neigh_get(self, total: int | None = None):
        """Row lengths and entries.  The library writes every entry, so
        without `total` the lengths are fetched first to size the buffer."""
        nl, _, _ = self.info()
        num = np.empty(max(nl, 1), np.int32)
        if total is None:
            self._ok(self.lib.emd_neigh_get(self.h, _ip(num), None), "emd_neigh_get")
            total = int(num[:nl].sum())
        ent = np.empty(max(total, 1), np.int32)
        self._ok(self.lib.emd_neigh_get(self.h, _ip(num), _ip(ent)), "emd_neigh_get")
        return num[:nl], ent[:total]

    def neigh_maxneighs(self) -> int:
        m = _I()
        self._ok(self.lib.emd_neigh_maxneighs(self.h, C.byref(m)), "emd_neigh_maxneighs")
        return m.value

    def lj_init(self, lj1, lj2, cutsq, half=False, precision=EMD_PREC_FP64):
        lj1, lj2, cutsq = _f64(lj1), _f64(lj2), _f64(cutsq)
        nt = int(round(np.sqrt(lj1.size)))
        if nt * nt != lj1.size or lj2.size != lj1.size or cutsq.size != lj1.size:
            raise EmdError("lj_init: lj1, lj2 and cutsq must be ntypes x ntypes tables")
        self._ok(self.lib.emd_lj_init(self.h, nt, _dp(lj1), _dp(lj2), _dp(cutsq), int(half), precision),
                 "emd_lj_init")

    def lj_compute(self):
        self._ok(self.lib.emd_lj_compute(self.h), "emd_lj_compute")

    def lj_energy(self) -> float:
        e = _D()
        self._ok(self.lib.emd_lj_energy(self.h, C.byref(e)), "emd_lj_energy")
        return e.value

    def lj_adjoint(self, dL_dF, dL_dE: float):
        """(dL/deps, dL/dsigma) for dL/dF (N_local x 3, current order) and dL/dE."""
        g = self._owned_rows(dL_dF, "lj_adjoint")
        out = np.zeros(2)
        self._ok(self.lib.emd_lj_adjoint(self.h, _dp(g), float(dL_dE), _dp(out)), "emd_lj_adjoint")
        return out

    def _owned_rows(self, a, what):
        """``a`` as a C-ordered float64 array of the N_local x 3 rows the library reads."""
        g = _f64(a, (-1, 3))
        n = self.info()[0]
        if g.shape[0] != n:
            raise EmdError(f"{what}: {n} rows of 3 expected, got {g.shape[0]}")
        return g

    def snap_adjoint(self, dL_dF, dL_dE: float, nelem: int, ncoeffall: int):
        """dL/dbeta (nelem x ncoeffall) for dL/dF (N_local x 3, current order) and dL/dE."""
        g = self._owned_rows(dL_dF, "snap_adjoint")
        if (nelem, ncoeffall) != self.snap_info():
            raise EmdError(f"snap_adjoint: the SNAP force has coefficients of shape {self.snap_info()}")
        out = np.zeros((nelem, ncoeffall))
        self._ok(self.lib.emd_snap_adjoint(self.h, _dp(g), float(dL_dE), _dp(out)), "emd_snap_adjoint")
        return out

    def lj_request_energy(self):
        """The next lj_compute (mixed form, one type pair) also computes the energy (emd_lj_request_energy)."""
        self._ok(self.lib.emd_lj_request_energy(self.h), "emd_lj_request_energy")

    def lj_force_energy(self):
        """The energy computed by the last lj_compute, or None (emd_lj_force_energy)."""
        e, ok = _D(), _I()
        self._ok(self.lib.emd_lj_force_energy(self.h, C.byref(e), C.byref(ok)), "emd_lj_force_energy")
        return e.value if ok.value else None

    def lj_energy_mixed(self):
        """The mixed form's energy kernel alone, or None where it does not apply (emd_lj_energy_mixed)."""
        e, ok = _D(), _I()
        self._ok(self.lib.emd_lj_energy_mixed(self.h, C.byref(e), C.byref(ok)), "emd_lj_energy_mixed")
        return e.value if ok.value else None

    def snap_request_energy(self):
        """The next snap_compute (FP64 form) also sums the energy (emd_snap_request_energy)."""
        self._ok(self.lib.emd_snap_request_energy(self.h), "emd_snap_request_energy")

    def snap_force_energy(self):
        """The energy summed by the last snap_compute, or None (emd_snap_force_energy)."""
        e, ok = _D(), _I()
        self._ok(self.lib.emd_snap_force_energy(self.h, C.byref(e), C.byref(ok)), "emd_snap_force_energy")
        return e.value if ok.value else None

    def lj_energy_noalloc(self) -> float:
        """emd_lj_energy_noalloc: the same energy, no device allocation."""
        e = _D()
        self._ok(self.lib.emd_lj_energy_noalloc(self.h, C.byref(e)), "emd_lj_energy_noalloc")
        return e.value

    def snap_init(self, twojmax, rfac0, rmin0, switchflag, rcutfac, radelem, wjelem, beta, type_map,
                  precision=EMD_PREC_FP64):
        radelem, wjelem = _f64(radelem), _f64(wjelem)
        beta = _f64(beta, (len(radelem), -1))
        tmap = _i32(type_map)
        if wjelem.size != radelem.size:
            raise EmdError("snap_init: one weight per element radius")
        self._ok(self.lib.emd_snap_init(self.h, twojmax, rfac0, rmin0, switchflag, rcutfac, len(radelem),
                                        _dp(radelem), _dp(wjelem), _dp(beta), beta.shape[1], len(tmap), _ip(tmap),
                                        precision), "emd_snap_init")

    def snap_keep_for_adjoint(self, on=True):
        """emd_snap_keep_for_adjoint: FP64 force passes keep U_tot and Z for
        the adjoint that follows on the same positions (bit-identical
        gradients, the adjoint's phases B and C skipped)."""
        self._ok(self.lib.emd_snap_keep_for_adjoint(self.h, int(bool(on))), "emd_snap_keep_for_adjoint")

    def snap_info(self):
        """(nelem, ncoeffall) of the initialised SNAP force (emd_snap_info)."""
        a, b = _I(), _I()
        self._ok(self.lib.emd_snap_info(self.h, C.byref(a), C.byref(b)), "emd_snap_info")
        return a.value, b.value

    def snap_set_beta(self, beta):
        """emd_snap_set_beta: new linear coefficients (nelem x ncoeffall), same tables."""
        b = np.ascontiguousarray(beta, dtype=np.float64)
        if b.shape != self.snap_info():
            raise EmdError(f"snap_set_beta: coefficients of shape {self.snap_info()} expected")
        self._ok(self.lib.emd_snap_set_beta(self.h, _dp(b)), "emd_snap_set_beta")

    def snap_compute(self):
        self._ok(self.lib.emd_snap_compute(self.h), "emd_snap_compute")

    def snap_energy(self) -> float:
        e = _D()
        self._ok(self.lib.emd_snap_energy(self.h, C.byref(e)), "emd_snap_energy")
        return e.value

    def thermo_mv2(self) -> float:
        e = _D()
        self._ok(self.lib.emd_thermo_mv2(self.h, C.byref(e)), "emd_thermo_mv2")
        return e.value

    def timing(self, on=True):
        self._ok(self.lib.emd_timing_enable(self.h, int(on)), "emd_timing_enable")

    def timing_only(self, kernels=None):
        """Events only for these kernel names (a list or comma-separated string; None: all)."""
        if kernels is not None and not isinstance(kernels, str):
            kernels = ",".join(kernels)
        arg = kernels.encode() if kernels else None
        self._ok(self.lib.emd_timing_only(self.h, arg), "emd_timing_only")

    def timing_reset(self):
        self._ok(self.lib.emd_timing_reset(self.h), "emd_timing_reset")

    def timing_report(self) -> dict:
        buf = C.create_string_buffer(65536)
        self._ok(self.lib.emd_timing_report(self.h, buf, len(buf)), "emd_timing_report")
        out = {}
        for line in buf.value.decode().splitlines():
            name, ms, n = line.split()
            out[name] = (float(ms), int(n))
        return out


class MD:
    """The ExaMiniMD driver on the GB300 modules (emd_driver.h)."""

    def __init__(self, args: list[str]):
        self.lib = load_library()
        argv = ["emd_gb300"] + list(args)
        arr = (C.c_char_p * len(argv))(*[a.encode() for a in argv])
        err = C.create_string_buffer(4096)
        h = self.lib.emd_md_create(len(argv), arr, err, len(err))
        if not h:
            raise EmdError(f"emd_md_create: {err.value.decode()}")
        self.h = h
        self.ctx = Context.__new__(Context)
        self.ctx.lib = self.lib
        self.ctx.h = _P(self.lib.emd_md_ctx(h))

    def close(self):
        if getattr(self, "h", None):
            self.ctx.h = None
            self.lib.emd_md_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ok(self, st, what):
        if st != 0:
            raise EmdError(f"{what}: {self.lib.emd_md_error(self.h).decode()}")

    def run(self, nsteps: int = -1):
        self._ok(self.lib.emd_md_run(self.h, nsteps), "emd_md_run")

    def run_host(self, nsteps: int, x, v, f):
        """run(nsteps) with the owned particles' x, v, f in host arrays
        (float64, C-contiguous, N_local x 3, updated in place): uploaded before
        every step and read back after it (emd_md_run_host)."""
        n = self.info()["N_local"]
        for a in (x, v, f):
            if a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"] or a.shape != (n, 3):
                raise EmdError(f"run_host: arrays must be float64, C-contiguous, shape ({n}, 3)")
        self._ok(self.lib.emd_md_run_host(self.h, nsteps, _dp(x), _dp(v), _dp(f)), "emd_md_run_host")

    def info(self) -> dict:
        v = [_I() for _ in range(5)]
        self._ok(self.lib.emd_md_info(self.h, *[C.byref(x) for x in v]), "emd_md_info")
        return dict(zip(("N", "N_local", "N_ghost", "deck_nsteps", "steps_done"), [x.value for x in v]))

    def thermo(self, recompute=False):
        v = [_D() for _ in range(3)]
        fn = self.lib.emd_md_compute_thermo if recompute else self.lib.emd_md_thermo
        self._ok(fn(self.h, *[C.byref(x) for x in v]), "emd_md_thermo")
        return tuple(x.value for x in v)

    def timers(self):
        out = np.zeros(5)
        self._ok(self.lib.emd_md_timers(self.h, _dp(out)), "emd_md_timers")
        return dict(zip(("force", "neigh", "comm", "other", "total"), out.tolist()))


class Batch:
    """A batched LJ ensemble (emd_batch.h): independent periodic systems of
    uneven size advanced together in the mixed-precision form."""

    def __init__(self, natoms, boxes, x, v, mass=1.0, dt=0.005, eps=1.0, sigma=1.0, cut=2.5, skin=0.3, every=20,
                 max_neigh=128, ghost_factor=1.5, device=0):
        self.lib = load_library()
        self.h = None
        natoms = _i32(natoms)
        boxes = _f64(boxes, (-1, 3))
        x, v = _f64(x, (-1, 3)), _f64(v, (-1, 3))
        if x.shape[0] != int(natoms.sum()) or v.shape != x.shape or boxes.shape[0] != natoms.shape[0]:
            raise EmdError("Batch: natoms, boxes, x and v do not agree")
        h = _P()
        st = self.lib.emd_batch_create(C.byref(h), device, len(natoms), _ip(natoms), _dp(boxes), _dp(x), _dp(v),
                                       mass, dt, eps, sigma, cut, skin, every, max_neigh, ghost_factor)
        if st != 0:
            raise EmdError(f"emd_batch_create: {self.lib.emd_status_string(st).decode()} (see stderr)")
        self.h = h
        self.nsys = len(natoms)
        self.natoms = natoms
        self.n = int(natoms.sum())

    def _ok(self, st, what):
        if st != 0:
            raise EmdError(f"{what}: {self.lib.emd_status_string(st).decode()} "
                           f"({self.lib.emd_batch_last_error(self.h).decode()})")

    def close(self):
        if self.h:
            self.lib.emd_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        return self.lib.emd_batch_stream(self.h) or 0

    def run(self, nsteps: int):
        self._ok(self.lib.emd_batch_run(self.h, nsteps), "emd_batch_run")

    def set_shape(self, threads: int, steps_per_launch: int):
        self._ok(self.lib.emd_batch_set_shape(self.h, threads, steps_per_launch), "emd_batch_set_shape")

    def tune(self, trial_steps: int):
        t, s = _I(), _I()
        self._ok(self.lib.emd_batch_tune(self.h, trial_steps, C.byref(t), C.byref(s)), "emd_batch_tune")
        return t.value, s.value

    def get(self):
        x, v, f = (np.empty((self.n, 3)) for _ in range(3))
        self._ok(self.lib.emd_batch_get(self.h, _dp(x), _dp(v), _dp(f)), "emd_batch_get")
        return x, v, f

    def thermo(self):
        """Per system (sum m v^2, shifted LJ potential energy)."""
        a, b = np.empty(self.nsys), np.empty(self.nsys)
        self._ok(self.lib.emd_batch_thermo(self.h, _dp(a), _dp(b)), "emd_batch_thermo")
        return a, b

    def info(self) -> dict:
        at, th, sp, sd = C.c_longlong(), _I(), _I(), C.c_longlong()
        self._ok(self.lib.emd_batch_info(self.h, C.byref(at), C.byref(th), C.byref(sp), C.byref(sd)),
                 "emd_batch_info")
        return {"atoms": at.value, "threads": th.value, "steps_per_launch": sp.value, "steps_done": sd.value}
