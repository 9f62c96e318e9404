"""ctypes wrapper around the CPU oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by bench.py's CPU-baseline / reference legs, never by the product.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

GR, GO, PKJ, IO = 0, 1, 2, 3
H_MAX = 0.125


class Desc(C.Structure):
    _fields_ = [
        ("type", C.c_int), ("nx", C.c_int), ("ny", C.c_int), ("ncomp", C.c_int),
        ("rows", C.POINTER(C.c_double)), ("gj_pairs", C.POINTER(C.c_int)),
        ("n_gj_pairs", C.c_int), ("jitter", C.POINTER(C.c_double)),
        ("stim_comp", C.POINTER(C.c_int)), ("stim_amp", C.POINTER(C.c_double)),
        ("stim_t0", C.POINTER(C.c_double)), ("stim_t1", C.POINTER(C.c_double)),
        ("io_gap_g", C.POINTER(C.c_double)),
        ("tol", C.c_double), ("hmin", C.c_double),
        ("io_gap", C.c_int), ("go_gj", C.c_int), ("pkj_gj", C.c_int),
        ("canon", C.c_int), ("cond_scale", C.POINTER(C.c_double)), ("cond_scale_ch", C.POINTER(C.c_double)),
    ]


def build(out_dir: str | None = None) -> str:
    out = out_dir or _HERE
    subprocess.run(["make", "-s", "-C", _HERE, f"OUT={out}"], check=True)
    return os.path.join(out, "liboracle.so")


def lib() -> C.CDLL:
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        P = C.c_void_p
        L.orc_create.restype = P
        L.orc_create.argtypes = [C.POINTER(Desc)]
        L.orc_destroy.argtypes = [P]
        L.orc_init.argtypes = [P]
        L.orc_advance.argtypes = [P, C.c_double]
        for f in ("orc_vnew", "orc_elem_v", "orc_b", "orc_ca", "orc_cm", "orc_area",
                  "orc_shell", "orc_rev_ca2", "orc_val"):
            getattr(L, f).restype = C.POINTER(C.c_double)
            getattr(L, f).argtypes = [P]
        for f in ("orc_ion", "orc_cond"):
            getattr(L, f).restype = C.POINTER(C.c_double)
            getattr(L, f).argtypes = [P, C.c_int]
        for f in ("orc_row", "orc_col"):
            getattr(L, f).restype = C.POINTER(C.c_int)
            getattr(L, f).argtypes = [P]
        for f in ("orc_nc", "orc_n", "orc_nnz", "orc_ncond", "orc_nion"):
            getattr(L, f).restype = C.c_int
            getattr(L, f).argtypes = [P]
        L.orc_ctl.argtypes = [P, C.POINTER(C.c_double)]
        L.orc_stats.argtypes = [P, C.POINTER(C.c_longlong)]
        L.orc_pivot_swaps.restype = C.c_longlong
        L.orc_net_create.restype = P
        L.orc_net_add_system.argtypes = [P, P]
        L.orc_net_add_synapses.argtypes = [P, C.c_int, C.c_int] + [C.POINTER(C.c_int)] * 4 + [
            C.POINTER(C.c_double), C.c_double, C.c_double, C.c_double, C.c_double, C.c_ulonglong]
        L.orc_net_set_delays.argtypes = [P, C.c_int, C.c_int, C.POINTER(C.c_int)]
        L.orc_net_build.argtypes = [P]
        L.orc_net_advance.argtypes = [P, C.c_double]
        L.orc_net_nsyn.argtypes = [P]
        L.orc_net_syn.argtypes = [P, C.c_int]
        L.orc_net_syn.restype = C.POINTER(C.c_double)
        L.orc_net_destroy.argtypes = [P]
        for f in ("orc_cm_exp", "orc_cm_log"):
            getattr(L, f).restype = C.c_double
            getattr(L, f).argtypes = [C.c_double]
        L.orc_cm_pow.restype = C.c_double
        L.orc_cm_pow.argtypes = [C.c_double, C.c_double]
        L.orc_cm_cbrt.restype = C.c_double
        L.orc_cm_cbrt.argtypes = [C.c_double]
        L.orc_ion_update.argtypes = [P, C.POINTER(C.c_double), C.c_double]
        L.orc_update_b.argtypes = [P, C.POINTER(C.c_double)]
        L.orc_set_elem_v.argtypes = [P, C.POINTER(C.c_double)]
        L.orc_set_ion.argtypes = [P, C.c_int, C.POINTER(C.c_double)]
        L.orc_set_ca.argtypes = [P, C.POINTER(C.c_double)]
        L.orc_draw_jitter.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_double)]
        _LIB = L
    return _LIB


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def draw_jitter(cell_type: int, n: int) -> np.ndarray:
    """Per-cell V0 jitter from libc rand() (caller seeds with srand)."""
    out = np.zeros(n, dtype=np.float64)
    lib().orc_draw_jitter(cell_type, n, _dp(out))
    return out


def cm_exp(x: float) -> float:
    return lib().orc_cm_exp(x)


def cm_log(x: float) -> float:
    return lib().orc_cm_log(x)


def cm_pow(x: float, y: float) -> float:
    return lib().orc_cm_pow(x, y)


def pivot_swaps() -> int:
    """Row swaps taken by the Na / KAHP Markov solvers in this process."""
    return int(lib().orc_pivot_swaps())


def libc_srand(seed: int) -> None:
    C.CDLL(None).srand(C.c_uint(seed))


class System:
    """One RKC system of the oracle (all cells of one type on an nx x ny grid)."""

    def __init__(self, cell_type, nx, ny, rows, jitter, stim=None, gj_pairs=None,
                 tol=0.0, hmin=0.0, io_gap=True, go_gj=True, pkj_gj=True, io_gap_g=None,
                 canon=False, cond_scale=None, cond_scale_ch=None):
        L = lib()
        self._keep = []
        rows = np.ascontiguousarray(rows, dtype=np.float64)
        n = nx * ny
        jitter = np.ascontiguousarray(jitter, dtype=np.float64)
        assert jitter.size == n
        d = Desc()
        d.type, d.nx, d.ny, d.ncomp = cell_type, nx, ny, rows.shape[0]
        d.rows = _dp(rows)
        d.jitter = _dp(jitter)
        self._keep += [rows, jitter]
        if gj_pairs is not None:
            g = np.ascontiguousarray(gj_pairs, dtype=np.int32).reshape(-1)
            d.gj_pairs, d.n_gj_pairs = _ip(g), g.size // 2
            self._keep.append(g)
        if stim is not None:
            comp, amp, t0, t1 = stim
            comp = np.ascontiguousarray(np.broadcast_to(comp, n), dtype=np.int32)
            amp, t0, t1 = (np.ascontiguousarray(np.broadcast_to(a, n), dtype=np.float64)
                           for a in (amp, t0, t1))
            d.stim_comp, d.stim_amp, d.stim_t0, d.stim_t1 = _ip(comp), _dp(amp), _dp(t0), _dp(t1)
            self._keep += [comp, amp, t0, t1]
        if io_gap_g is not None:
            gg = np.ascontiguousarray(io_gap_g, dtype=np.float64)
            d.io_gap_g = _dp(gg)
            self._keep.append(gg)
        d.tol, d.hmin = tol, hmin
        d.io_gap, d.go_gj, d.pkj_gj = int(io_gap), int(go_gj), int(pkj_gj)
        d.canon = int(canon)
        if cond_scale is not None:
            cs = np.ascontiguousarray(np.broadcast_to(cond_scale, n), dtype=np.float64)
            d.cond_scale = _dp(cs)
            self._keep.append(cs)
        if cond_scale_ch is not None:
            cc = np.ascontiguousarray(cond_scale_ch, dtype=np.float64).reshape(-1)
            d.cond_scale_ch = _dp(cc)
            self._keep.append(cc)
        self.h = L.orc_create(C.byref(d))
        if not self.h:
            raise RuntimeError("orc_create failed")
        self.type, self.n, self.ncomp = cell_type, n, rows.shape[0]
        self.nc = L.orc_nc(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def _arr(self, ptr, n=None):
        n = self.nc if n is None else n
        return np.ctypeslib.as_array(ptr, shape=(n,)).copy()

    def init(self) -> int:
        return lib().orc_init(self.h)

    def advance(self, t: float) -> int:
        return lib().orc_advance(self.h, t)

    def vnew(self):
        return self._arr(lib().orc_vnew(self.h))

    def elem_v(self):
        return self._arr(lib().orc_elem_v(self.h))

    def b(self):
        return self._arr(lib().orc_b(self.h))

    def ca(self):
        return self._arr(lib().orc_ca(self.h))

    def ion(self, k):
        return self._arr(lib().orc_ion(self.h, k))

    def cm(self):
        return self._arr(lib().orc_cm(self.h))

    def area(self):
        return self._arr(lib().orc_area(self.h))

    def shell(self):
        return self._arr(lib().orc_shell(self.h))

    def rev_ca2(self):
        return self._arr(lib().orc_rev_ca2(self.h))

    def cond(self, k):
        return self._arr(lib().orc_cond(self.h, k))

    def ncond(self):
        return lib().orc_ncond(self.h)

    def nion(self):
        return lib().orc_nion(self.h)

    def csr(self):
        L = lib()
        nnz = L.orc_nnz(self.h)
        row = np.ctypeslib.as_array(L.orc_row(self.h), shape=(self.nc + 1,)).copy()
        col = np.ctypeslib.as_array(L.orc_col(self.h), shape=(nnz,)).copy()
        val = np.ctypeslib.as_array(L.orc_val(self.h), shape=(nnz,)).copy()
        return row, col, val

    def ctl(self):
        out = np.zeros(8, dtype=np.float64)
        lib().orc_ctl(self.h, _dp(out))
        return dict(zip(["absh", "sprad", "naccpt", "errold", "hold", "lt", "tend", "sum_dt"], out))

    def stats(self):
        out = np.zeros(6, dtype=np.int64)
        lib().orc_stats(self.h, out.ctypes.data_as(C.POINTER(C.c_longlong)))
        return dict(zip(["steps", "rejects", "stages", "rho_calls", "ion_updates", "rho_iters"],
                        out.tolist()))

    def ion_update(self, vnew, dt):
        v = np.ascontiguousarray(vnew, dtype=np.float64)
        lib().orc_ion_update(self.h, _dp(v), dt)

    def update_b(self, vy):
        v = np.ascontiguousarray(vy, dtype=np.float64)
        lib().orc_update_b(self.h, _dp(v))

    def set_elem_v(self, v):
        v = np.ascontiguousarray(v, dtype=np.float64)
        lib().orc_set_elem_v(self.h, _dp(v))

    def set_ion(self, k, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        lib().orc_set_ion(self.h, k, _dp(x))

    def set_ca(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        lib().orc_set_ca(self.h, _dp(x))


class Network:
    """Oracle network mode: Systems advanced together with the reference's
    chemical synapses (kinds 0..3: MF->GrC, GrC->GoC, GoC->GrC, GrC->PC).
    Systems advance in the order added.  Test infrastructure."""

    def __init__(self):
        self.h = lib().orc_net_create()
        self.systems = []
        self._keep = []

    def add_system(self, s) -> int:
        self.systems.append(s)
        return lib().orc_net_add_system(self.h, s.h)

    def add_synapses(self, kind, post_system, post_comp, weight, pre_system=None, pre_comp=None,
                     rates=(0.0, 0.0, 0.0, 0.0), seed=0, delay=None) -> int:
        post_system = np.ascontiguousarray(post_system, dtype=np.int32)
        n = post_system.size
        post_comp = np.ascontiguousarray(np.broadcast_to(post_comp, n), dtype=np.int32)
        weight = np.ascontiguousarray(np.broadcast_to(weight, n), dtype=np.float64)
        pre_system = np.ascontiguousarray(np.broadcast_to(-1 if pre_system is None else pre_system, n), dtype=np.int32)
        pre_comp = np.ascontiguousarray(np.broadcast_to(0 if pre_comp is None else pre_comp, n), dtype=np.int32)
        self._keep.append((post_system, post_comp, weight, pre_system, pre_comp))
        first = lib().orc_net_add_synapses(self.h, kind, n, _ip(pre_system), _ip(pre_comp), _ip(post_system),
                                           _ip(post_comp), _dp(weight), *rates, seed)
        if delay is not None:
            d = np.ascontiguousarray(np.broadcast_to(delay, n), dtype=np.int32)
            if lib().orc_net_set_delays(self.h, first, n, _ip(d)) != 0:
                raise ValueError("delays must be 0..63 intervals")
        return first

    def build(self):
        if lib().orc_net_build(self.h) != 0:
            raise RuntimeError("synapses onto an unsupported cell type")

    def advance(self, t: float) -> int:
        return lib().orc_net_advance(self.h, t)

    def syn(self, field: int) -> np.ndarray:
        n = lib().orc_net_nsyn(self.h)
        p = lib().orc_net_syn(self.h, field)
        return np.ctypeslib.as_array(p, shape=(n,)).copy()

    def __del__(self):
        try:
            lib().orc_net_destroy(self.h)
        except Exception:
            pass
