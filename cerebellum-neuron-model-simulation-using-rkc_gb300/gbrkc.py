"""Python binding of the gbrkc C ABI (include/gbrkc.h) over ctypes.

Thin by design: every call goes straight to libgbrkc.so; there is no Python or
CPU fallback.  If the native library is missing or no CUDA device is present
the calls raise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgbrkc.so")

GR, GO, PKJ, IO = 0, 1, 2, 3
FP64, MIXED = 0, 1
F_VNEW, F_V, F_CA, F_B, F_ION, F_REV, F_YN = 0, 1, 2, 3, 4, 5, 6
H_MAX = 0.125
STATUS_BITS = {1: "non-finite error norm", 2: "step loop bound", 4: "stage count beyond table",
               8: "unexpected idid", 32: "grid barrier gave up waiting"}


class SystemDesc(C.Structure):
    _fields_ = [
        ("cell_type", C.c_int), ("nx", C.c_int), ("ny", C.c_int), ("ncomp", C.c_int),
        ("rows", C.POINTER(C.c_double)), ("gj_pairs", C.POINTER(C.c_int)), ("n_gj_pairs", C.c_int),
        ("gap_junctions", C.c_int), ("io_gap_g", C.POINTER(C.c_double)),
        ("jitter", C.POINTER(C.c_double)), ("stim_comp", C.POINTER(C.c_int)),
        ("stim_amp", C.POINTER(C.c_double)), ("stim_t0", C.POINTER(C.c_double)),
        ("stim_t1", C.POINTER(C.c_double)), ("tol", C.c_double), ("hmin", C.c_double),
        ("cond_scale", C.POINTER(C.c_double)), ("idle", C.c_int),
        ("cond_scale_ch", C.POINTER(C.c_double)),
    ]


class SlotClass(C.Structure):
    _fields_ = [("shape", SystemDesc), ("slots", C.c_longlong), ("share", C.c_double)]


class RequestDesc(C.Structure):
    _fields_ = [
        ("class_id", C.c_int), ("n_systems", C.c_int), ("n_intervals", C.c_int),
        ("jitter", C.POINTER(C.c_double)), ("stim_comp", C.POINTER(C.c_int)),
        ("stim_amp", C.POINTER(C.c_double)), ("stim_t0", C.POINTER(C.c_double)),
        ("stim_t1", C.POINTER(C.c_double)), ("cond_scale", C.POINTER(C.c_double)),
        ("io_gap_g", C.POINTER(C.c_double)),
    ]


class ServerStats(C.Structure):
    _fields_ = [(k, C.c_longlong) for k in ("submitted", "admitted", "completed", "failed", "cancelled",
                                            "queued", "resident", "rounds")] + \
               [(k, C.c_double) for k in ("p50_ms", "p99_ms", "mean_ms", "max_ms", "busy_s", "advance_s")] + \
               [(k, C.c_longlong) for k in ("compartment_updates", "hbm_reserved", "hbm_in_use", "slots",
                                            "free_slots")] + \
               [("sim_ms", C.c_double), ("lost_spike_reads", C.c_longlong)]


REQ_QUEUED, REQ_RESIDENT, REQ_DONE, REQ_FAILED = 0, 1, 2, 3


class ResetDesc(C.Structure):
    _fields_ = [
        ("jitter", C.POINTER(C.c_double)), ("stim_comp", C.POINTER(C.c_int)),
        ("stim_amp", C.POINTER(C.c_double)), ("stim_t0", C.POINTER(C.c_double)),
        ("stim_t1", C.POINTER(C.c_double)), ("cond_scale", C.POINTER(C.c_double)),
        ("io_gap_g", C.POINTER(C.c_double)), ("n_intervals", C.c_int),
        ("cond_scale_ch", C.POINTER(C.c_double)),
    ]


class SynapseDesc(C.Structure):
    _fields_ = [
        ("kind", C.c_int), ("n", C.c_int),
        ("pre_system", C.POINTER(C.c_int)), ("pre_comp", C.POINTER(C.c_int)),
        ("post_system", C.POINTER(C.c_int)), ("post_comp", C.POINTER(C.c_int)),
        ("weight", C.POINTER(C.c_double)),
        ("rate_base", C.c_double), ("rate_stim", C.c_double), ("stim_t0", C.c_double), ("stim_t1", C.c_double),
        ("seed", C.c_ulonglong), ("delay", C.POINTER(C.c_int)),
    ]


SYN_MFGR, SYN_GRGO, SYN_GOGR, SYN_GRPKJ = 0, 1, 2, 3
SYNF_VAL, SYNF_S0, SYNF_S1, SYNF_S2, SYNF_OLD_V = 0, 1, 2, 3, 4

_LIB = None


def lib() -> C.CDLL:
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} not built: run __graft_entry__.build() (no fallback exists)")
        L = C.CDLL(LIB_PATH)
        P = C.c_void_p
        L.gbrkc_engine_create.argtypes = [C.c_int, C.POINTER(P)]
        L.gbrkc_engine_destroy.argtypes = [P]
        L.gbrkc_add_system.argtypes = [P, C.POINTER(SystemDesc), C.POINTER(C.c_int)]
        L.gbrkc_build.argtypes = [P]
        L.gbrkc_advance.argtypes = [P, C.c_double, C.c_int]
        L.gbrkc_advance_noalloc.argtypes = [P, C.c_double, C.c_int]
        L.gbrkc_add_synapses.argtypes = [P, C.POINTER(SynapseDesc), C.POINTER(C.c_int)]
        L.gbrkc_read_synapses.argtypes = [P, C.c_int, C.POINTER(C.c_double), C.c_long]
        L.gbrkc_read.argtypes = [P, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double), C.c_long]
        L.gbrkc_system_ctl.argtypes = [P, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_longlong),
                                       C.POINTER(C.c_int)]
        L.gbrkc_system_nc.argtypes = [P, C.c_int]
        L.gbrkc_record_soma.argtypes = [P, C.c_int]
        L.gbrkc_read_soma.argtypes = [P, C.c_int, C.c_int, C.POINTER(C.c_double)]
        L.gbrkc_total_compartments.argtypes = [P]
        L.gbrkc_total_compartments.restype = C.c_long
        L.gbrkc_last_error.restype = C.c_char_p
        L.gbrkc_set_stim.argtypes = [P, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double),
                                     C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.gbrkc_last_advance_ms.argtypes = [P]
        L.gbrkc_last_advance_ms.restype = C.c_float
        L.gbrkc_last_kernel_ms.argtypes = [P, C.c_int]
        L.gbrkc_last_kernel_ms.restype = C.c_float
        L.gbrkc_type_cells.argtypes = [P, C.c_int]
        L.gbrkc_set_stim_type.argtypes = [P, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double),
                                          C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.gbrkc_read_soma_type.argtypes = [P, C.c_int, C.c_int, C.POINTER(C.c_double)]
        L.gbrkc_rewind_soma.argtypes = [P]
        L.gbrkc_record_width.argtypes = [P, C.c_int, C.c_int]
        L.gbrkc_retired_systems.argtypes = [P]
        L.gbrkc_autotune.argtypes = [P, C.c_double, C.c_int, C.POINTER(C.c_int)]
        L.gbrkc_launch_layout.argtypes = [P, C.POINTER(C.c_int)]
        L.gbrkc_type_team.argtypes = [P, C.c_int]
        L.gbrkc_grid_shape.argtypes = [C.c_longlong, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.gbrkc_compartment_updates.argtypes = [P, C.c_int]
        L.gbrkc_compartment_updates.restype = C.c_longlong
        L.gbrkc_systems_reset.argtypes = [P, C.c_int, C.c_int, C.POINTER(ResetDesc)]
        L.gbrkc_set_budget.argtypes = [P, C.c_int, C.c_int, C.c_int]
        L.gbrkc_system_bytes.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int]
        L.gbrkc_system_bytes.restype = C.c_longlong
        L.gbrkc_run_status.argtypes = [P, C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.gbrkc_read_run.argtypes = [P, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double), C.c_long]
        L.gbrkc_record_spikes.argtypes = [P, C.c_long]
        L.gbrkc_read_spikes.argtypes = [P, C.c_int, C.c_long, C.POINTER(C.c_double), C.POINTER(C.c_int),
                                        C.POINTER(C.c_int), C.POINTER(C.c_long)]
        S = C.c_void_p
        L.gbrkc_server_create.argtypes = [C.c_int, C.c_longlong, C.c_int, C.POINTER(S)]
        L.gbrkc_server_destroy.argtypes = [S]
        L.gbrkc_server_add_class.argtypes = [S, C.POINTER(SlotClass), C.POINTER(C.c_int)]
        L.gbrkc_server_start.argtypes = [S]
        L.gbrkc_server_class_slots.argtypes = [S, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.gbrkc_request_create.argtypes = [S, C.POINTER(RequestDesc), C.POINTER(C.c_int)]
        L.gbrkc_request_advance.argtypes = [S, C.POINTER(C.c_int)]
        L.gbrkc_request_state.argtypes = [S, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double),
                                          C.POINTER(C.c_int)]
        L.gbrkc_request_read.argtypes = [S, C.c_int, C.POINTER(C.c_double), C.c_long]
        L.gbrkc_request_spikes.argtypes = [S, C.c_int, C.c_long, C.POINTER(C.c_double), C.POINTER(C.c_int),
                                           C.POINTER(C.c_long)]
        L.gbrkc_request_destroy.argtypes = [S, C.c_int]
        L.gbrkc_server_stats.argtypes = [S, C.POINTER(ServerStats)]
        L.gbrkc_server_engine.argtypes = [S]
        L.gbrkc_server_engine.restype = C.c_void_p
        L.gbrkc_server_last_error.restype = C.c_char_p
        _LIB = L
    return _LIB


class GbrkcError(RuntimeError):
    pass


def _check(rc: int) -> None:
    if rc != 0:
        raise GbrkcError(f"gbrkc error {rc}: {lib().gbrkc_last_error().decode()}")


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


class Engine:
    """A set of RKC systems advanced together on the GPU."""

    def __init__(self, precision: int = FP64):
        self.h = C.c_void_p()
        _check(lib().gbrkc_engine_create(precision, C.byref(self.h)))
        self.precision = precision
        self._keep = []
        self.ncomp = {}

    def close(self):
        if self.h:
            lib().gbrkc_engine_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_system(self, cell_type, nx, ny, rows, jitter, stim=None, gj_pairs=None, gap=True,
                   io_gap_g=None, tol=0.0, hmin=0.0, cond_scale=None, idle=False, cond_scale_ch=None) -> int:
        n = nx * ny
        rows = np.ascontiguousarray(rows, dtype=np.float64)
        jitter = np.ascontiguousarray(jitter, dtype=np.float64)
        assert jitter.size == n
        d = SystemDesc()
        d.cell_type, d.nx, d.ny, d.ncomp = cell_type, nx, ny, rows.shape[0]
        d.rows, d.jitter = _dp(rows), _dp(jitter)
        keep = [rows, jitter]
        if gj_pairs is not None:
            g = np.ascontiguousarray(gj_pairs, dtype=np.int32).reshape(-1)
            d.gj_pairs, d.n_gj_pairs = _ip(g), g.size // 2
            keep.append(g)
        d.gap_junctions = int(gap)
        if io_gap_g is not None:
            gg = np.ascontiguousarray(io_gap_g, dtype=np.float64)
            d.io_gap_g = _dp(gg)
            keep.append(gg)
        if stim is not None:
            comp, amp, t0, t1 = stim
            comp = np.ascontiguousarray(np.broadcast_to(comp, n), dtype=np.int32)
            amp, t0, t1 = (np.ascontiguousarray(np.broadcast_to(a, n), dtype=np.float64) for a in (amp, t0, t1))
            d.stim_comp, d.stim_amp, d.stim_t0, d.stim_t1 = _ip(comp), _dp(amp), _dp(t0), _dp(t1)
            keep += [comp, amp, t0, t1]
        d.tol, d.hmin = tol, hmin
        if cond_scale is not None:
            cs = np.ascontiguousarray(np.broadcast_to(cond_scale, n), dtype=np.float64)
            d.cond_scale = _dp(cs)
            keep.append(cs)
        d.idle = int(idle)
        if cond_scale_ch is not None:
            cc = np.ascontiguousarray(cond_scale_ch, dtype=np.float64).reshape(-1)
            d.cond_scale_ch = _dp(cc)
            keep.append(cc)
        sid = C.c_int()
        _check(lib().gbrkc_add_system(self.h, C.byref(d), C.byref(sid)))
        self._keep.append(keep)
        self.ncomp[sid.value] = (cell_type, n, rows.shape[0])
        return sid.value

    def reset_systems(self, first: int, n: int, jitter, stim=None, cond_scale=None, io_gap_g=None,
                      n_intervals: int = -1, cond_scale_ch=None):
        """Refill systems first .. first+n-1 (one run of one type) with new cells of the same shape."""
        jitter = np.ascontiguousarray(jitter, dtype=np.float64)
        cells = jitter.size
        d = ResetDesc()
        d.jitter = _dp(jitter)
        keep = [jitter]
        if stim is not None:
            comp, amp, t0, t1 = stim
            comp = np.ascontiguousarray(np.broadcast_to(comp, cells), dtype=np.int32)
            amp, t0, t1 = (np.ascontiguousarray(np.broadcast_to(a, cells), dtype=np.float64) for a in (amp, t0, t1))
            d.stim_comp, d.stim_amp, d.stim_t0, d.stim_t1 = _ip(comp), _dp(amp), _dp(t0), _dp(t1)
            keep += [comp, amp, t0, t1]
        if cond_scale is not None:
            cs = np.ascontiguousarray(np.broadcast_to(cond_scale, cells), dtype=np.float64)
            d.cond_scale = _dp(cs)
            keep.append(cs)
        if io_gap_g is not None:
            gg = np.ascontiguousarray(io_gap_g, dtype=np.float64)
            d.io_gap_g = _dp(gg)
            keep.append(gg)
        if cond_scale_ch is not None:
            cc = np.ascontiguousarray(cond_scale_ch, dtype=np.float64).reshape(-1)
            d.cond_scale_ch = _dp(cc)
            keep.append(cc)
        d.n_intervals = n_intervals
        _check(lib().gbrkc_systems_reset(self.h, first, n, C.byref(d)))

    def set_budget(self, first: int, n: int, n_intervals: int):
        _check(lib().gbrkc_set_budget(self.h, first, n, n_intervals))

    def run_status(self, first: int, n: int):
        """Status words and interval budgets left of systems first .. first+n-1 (one run)."""
        st = np.empty(n, np.int32)
        left = np.empty(n, np.int32)
        _check(lib().gbrkc_run_status(self.h, first, n, _ip(st), _ip(left)))
        return st, left

    def read_run(self, first: int, n: int, field: int, n_values: int) -> np.ndarray:
        out = np.empty(n_values, np.float64)
        _check(lib().gbrkc_read_run(self.h, first, n, field, _dp(out), n_values))
        return out

    def record_spikes(self, capacity: int):
        _check(lib().gbrkc_record_spikes(self.h, capacity))

    def read_spikes(self, cell_type: int, cap: int = 1 << 20):
        """Drain one type's device raster: (times, system ids, cells within system), sorted."""
        t = np.empty(max(cap, 1), np.float64)
        sy = np.empty(max(cap, 1), np.int32)
        ce = np.empty(max(cap, 1), np.int32)
        n = C.c_long()
        _check(lib().gbrkc_read_spikes(self.h, cell_type, cap, _dp(t), _ip(sy), _ip(ce), C.byref(n)))
        return t[:n.value].copy(), sy[:n.value].copy(), ce[:n.value].copy()

    def add_synapses(self, kind, post_system, post_comp, weight, pre_system=None, pre_comp=None,
                     rates=(0.0, 0.0, 0.0, 0.0), seed=0, delay=None) -> int:
        """Add one group of chemical synapses (GBRKC_SYN_*); returns the id of
        its first synapse.  rates = (base Hz, stimulus Hz, t0 ms, t1 ms) for
        mossy fibres (all 0: the reference's schedule); delay in intervals."""
        post_system = np.ascontiguousarray(post_system, dtype=np.int32)
        n = post_system.size
        post_comp = np.ascontiguousarray(np.broadcast_to(post_comp, n), dtype=np.int32)
        weight = np.ascontiguousarray(np.broadcast_to(weight, n), dtype=np.float64)
        d = SynapseDesc()
        d.kind, d.n = kind, n
        d.post_system, d.post_comp, d.weight = _ip(post_system), _ip(post_comp), _dp(weight)
        keep = [post_system, post_comp, weight]
        if pre_system is not None:
            pre_system = np.ascontiguousarray(np.broadcast_to(pre_system, n), dtype=np.int32)
            pre_comp = np.ascontiguousarray(np.broadcast_to(pre_comp, n), dtype=np.int32)
            d.pre_system, d.pre_comp = _ip(pre_system), _ip(pre_comp)
            keep += [pre_system, pre_comp]
        d.rate_base, d.rate_stim, d.stim_t0, d.stim_t1 = rates
        d.seed = seed
        if delay is not None:
            dl = np.ascontiguousarray(np.broadcast_to(delay, n), dtype=np.int32)
            d.delay = _ip(dl)
            keep.append(dl)
        first = C.c_int()
        _check(lib().gbrkc_add_synapses(self.h, C.byref(d), C.byref(first)))
        self._keep.append(keep)
        return first.value

    def read_synapses(self, field: int, n: int) -> np.ndarray:
        out = np.empty(n, dtype=np.float64)
        _check(lib().gbrkc_read_synapses(self.h, field, _dp(out), n))
        return out

    def build(self):
        _check(lib().gbrkc_build(self.h))
        self._keep = []

    def advance(self, t0: float, n_intervals: int, tolerate_retire: bool = False):
        """Advance every system.  A system whose step goes non-finite is
        retired (the others continue); that raises unless tolerate_retire."""
        rc = lib().gbrkc_advance(self.h, t0, n_intervals)
        if rc == -5 and tolerate_retire:
            return
        _check(rc)

    def advance_noalloc(self, t0: float, n_intervals: int, tolerate_stopped: bool = False):
        """advance() through gbrkc_advance_noalloc: no device or host
        allocation during the call (launch scratch in static device memory).
        Raises while any system is stopped, unless tolerate_stopped."""
        rc = lib().gbrkc_advance_noalloc(self.h, t0, n_intervals)
        if rc == -5 and tolerate_stopped:
            return
        _check(rc)

    def launch_layout(self):
        """(persistent?, CTAs per cell type) of the advance launch."""
        c = (C.c_int * 4)()
        rc = lib().gbrkc_launch_layout(self.h, c)
        if rc < 0:
            _check(rc)
        return bool(rc), list(c)

    TEAMS = {1: "mega", 2: "grid", 3: "cluster", 4: "pool"}

    def type_team(self, cell_type: int) -> str:
        """How the type's systems are integrated: "mega", "grid", "cluster",
        "pool", or "" for an empty type."""
        rc = lib().gbrkc_type_team(self.h, cell_type)
        if rc < 0:
            _check(rc)
        return self.TEAMS.get(rc, "")

    def retired(self) -> int:
        return lib().gbrkc_retired_systems(self.h)

    def autotune(self, t0: float, n_intervals: int) -> int:
        """Time the next launch with 32, 16 and 8 granule systems per warp (the
        state is restored after each) and keep the fastest; returns it."""
        lanes = C.c_int()
        _check(lib().gbrkc_autotune(self.h, t0, n_intervals, C.byref(lanes)))
        return lanes.value

    def nc(self, sid: int) -> int:
        return lib().gbrkc_system_nc(self.h, sid)

    def read(self, sid: int, field: int, k: int = 0) -> np.ndarray:
        n = self.nc(sid)
        out = np.empty(n, dtype=np.float64)
        _check(lib().gbrkc_read(self.h, sid, field, k, _dp(out), n))
        return out

    def vnew(self, sid):
        return self.read(sid, F_VNEW)

    def ctl(self, sid):
        c = np.zeros(8)
        st = np.zeros(6, dtype=np.int64)
        status = C.c_int()
        _check(lib().gbrkc_system_ctl(self.h, sid, _dp(c), st.ctypes.data_as(C.POINTER(C.c_longlong)),
                                      C.byref(status)))
        ctl = dict(zip(["absh", "sprad", "naccpt", "errold", "hold", "lt", "tend", "sum_dt"], c))
        stats = dict(zip(["steps", "rejects", "stages", "rho_calls", "ion_updates", "rho_iters"], st.tolist()))
        return ctl, stats, status.value

    def record_soma(self, n_max: int):
        _check(lib().gbrkc_record_soma(self.h, n_max))

    def read_soma(self, sid: int, n_intervals: int) -> np.ndarray:
        _, n, _ = self.ncomp[sid]
        out = np.empty((n_intervals, n), dtype=np.float64)
        _check(lib().gbrkc_read_soma(self.h, sid, n_intervals, _dp(out)))
        return out

    def total_compartments(self) -> int:
        return lib().gbrkc_total_compartments(self.h)

    def set_stim(self, sid, comp, amp, t0, t1):
        _, n, _ = self.ncomp[sid]
        comp = np.ascontiguousarray(np.broadcast_to(comp, n), dtype=np.int32)
        amp, t0, t1 = (np.ascontiguousarray(np.broadcast_to(a, n), dtype=np.float64) for a in (amp, t0, t1))
        _check(lib().gbrkc_set_stim(self.h, sid, _ip(comp), _dp(amp), _dp(t0), _dp(t1)))

    def type_cells(self, cell_type: int) -> int:
        n = lib().gbrkc_type_cells(self.h, cell_type)
        if n < 0:
            _check(n)
        return n

    def set_stim_type(self, cell_type, comp, amp, t0, t1):
        """Bulk stimulus upload from host buffers (np arrays of type_cells entries)."""
        _check(lib().gbrkc_set_stim_type(self.h, cell_type, _ip(comp), _dp(amp), _dp(t0), _dp(t1)))

    def read_soma_type(self, cell_type: int, n_intervals: int, out: np.ndarray):
        _check(lib().gbrkc_read_soma_type(self.h, cell_type, n_intervals, _dp(out)))
        return out

    def record_width(self, cell_type: int, width: int):
        _check(lib().gbrkc_record_width(self.h, cell_type, width))

    def rewind_soma(self):
        _check(lib().gbrkc_rewind_soma(self.h))

    def compartment_updates(self, cell_type: int = -1) -> int:
        n = lib().gbrkc_compartment_updates(self.h, cell_type)
        if n < 0:
            _check(int(n))
        return int(n)

    def last_advance_ms(self) -> float:
        return float(lib().gbrkc_last_advance_ms(self.h))

    def last_kernel_ms(self, cell_type: int) -> float:
        return float(lib().gbrkc_last_kernel_ms(self.h, cell_type))


def system_bytes(precision: int, cell_type: int, ncomp: int, ncell: int) -> int:
    """Device bytes one system of this shape takes (an upper estimate)."""
    b = lib().gbrkc_system_bytes(precision, cell_type, ncomp, ncell)
    if b < 0:
        _check(int(b))
    return int(b)


def grid_shape(nc: int, max_ctas: int):
    """The grid team's launch shape for a lone system of nc compartments on at
    most max_ctas CTAs: (threads per CTA, CTAs).  Host only."""
    bw, n = C.c_int(), C.c_int()
    _check(lib().gbrkc_grid_shape(nc, max_ctas, C.byref(bw), C.byref(n)))
    return bw.value, n.value


def _scheck(rc: int) -> None:
    if rc != 0:
        raise GbrkcError(f"gbrkc server error {rc}: {lib().gbrkc_server_last_error().decode()}")


class Server:
    """Request server: jobs of uneven sizes and durations advanced together in one resident arena."""

    def __init__(self, precision: int = MIXED, hbm_budget: int = 0, quantum: int = 8):
        self.h = C.c_void_p()
        _scheck(lib().gbrkc_server_create(precision, hbm_budget, quantum, C.byref(self.h)))
        self._keep = []
        self.cells = {}      # class id -> (cells per system, compartments per system)

    def close(self):
        if self.h:
            lib().gbrkc_server_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_class(self, cell_type, nx, ny, rows, slots=0, share=0.0, gj_pairs=None, gap=True, tol=0.0,
                  hmin=0.0) -> int:
        rows = np.ascontiguousarray(rows, dtype=np.float64)
        c = SlotClass()
        d = c.shape
        d.cell_type, d.nx, d.ny, d.ncomp = cell_type, nx, ny, rows.shape[0]
        d.rows = _dp(rows)
        keep = [rows]
        if gj_pairs is not None:
            g = np.ascontiguousarray(gj_pairs, dtype=np.int32).reshape(-1)
            d.gj_pairs, d.n_gj_pairs = _ip(g), g.size // 2
            keep.append(g)
        d.gap_junctions = int(gap)
        d.tol, d.hmin = tol, hmin
        c.slots, c.share = slots, share
        cid = C.c_int()
        _scheck(lib().gbrkc_server_add_class(self.h, C.byref(c), C.byref(cid)))
        self._keep.append(keep)
        self.cells[cid.value] = (nx * ny, nx * ny * rows.shape[0])
        return cid.value

    def start(self):
        _scheck(lib().gbrkc_server_start(self.h))

    def class_slots(self, cid: int):
        n, first = C.c_int(), C.c_int()
        _scheck(lib().gbrkc_server_class_slots(self.h, cid, C.byref(n), C.byref(first)))
        return n.value, first.value

    def submit(self, cid, n_systems, n_intervals, jitter, stim=None, cond_scale=None, io_gap_g=None) -> int:
        cells = n_systems * self.cells[cid][0]
        jitter = np.ascontiguousarray(jitter, dtype=np.float64)
        assert jitter.size == cells
        d = RequestDesc()
        d.class_id, d.n_systems, d.n_intervals = cid, n_systems, n_intervals
        d.jitter = _dp(jitter)
        keep = [jitter]
        if stim is not None:
            comp, amp, t0, t1 = stim
            comp = np.ascontiguousarray(np.broadcast_to(comp, cells), dtype=np.int32)
            amp, t0, t1 = (np.ascontiguousarray(np.broadcast_to(a, cells), dtype=np.float64) for a in (amp, t0, t1))
            d.stim_comp, d.stim_amp, d.stim_t0, d.stim_t1 = _ip(comp), _dp(amp), _dp(t0), _dp(t1)
            keep += [comp, amp, t0, t1]
        if cond_scale is not None:
            cs = np.ascontiguousarray(np.broadcast_to(cond_scale, cells), dtype=np.float64)
            d.cond_scale = _dp(cs)
            keep.append(cs)
        if io_gap_g is not None:
            gg = np.ascontiguousarray(io_gap_g, dtype=np.float64)
            assert gg.size == 4 * cells
            d.io_gap_g = _dp(gg)
            keep.append(gg)
        rid = C.c_int()
        _scheck(lib().gbrkc_request_create(self.h, C.byref(d), C.byref(rid)))
        return rid.value

    def advance(self) -> int:
        n = C.c_int()
        _scheck(lib().gbrkc_request_advance(self.h, C.byref(n)))
        return n.value

    def state(self, rid: int):
        st, lat, status = C.c_int(), C.c_double(), C.c_int()
        _scheck(lib().gbrkc_request_state(self.h, rid, C.byref(st), C.byref(lat), C.byref(status)))
        return st.value, lat.value, status.value

    def read(self, rid: int, n: int) -> np.ndarray:
        out = np.empty(n, np.float64)
        _scheck(lib().gbrkc_request_read(self.h, rid, _dp(out), n))
        return out

    def spikes(self, rid: int, cap: int = 1 << 20):
        t = np.empty(max(cap, 1), np.float64)
        c = np.empty(max(cap, 1), np.int32)
        n = C.c_long()
        _scheck(lib().gbrkc_request_spikes(self.h, rid, cap, _dp(t), _ip(c), C.byref(n)))
        return t[:n.value].copy(), c[:n.value].copy()

    def destroy(self, rid: int):
        _scheck(lib().gbrkc_request_destroy(self.h, rid))

    def stats(self) -> dict:
        st = ServerStats()
        _scheck(lib().gbrkc_server_stats(self.h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in ServerStats._fields_}
