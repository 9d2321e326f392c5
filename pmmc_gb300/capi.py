"""ctypes binding of the C ABI (include/pmmc_gb300.h).

The library is the in-tree ``libpmmc_gb300.so`` built by pmmc_gb300.build.
Importing this module never falls back to anything: if the library is
missing, :func:`lib` raises; if no GB300 device is present, creating a
context raises :class:`PmmcError` with PMMC_ERR_NO_DEVICE.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpmmc_gb300.so")

PMMC_OK = 0
PMMC_ERR_INVALID = 1
PMMC_ERR_NO_DEVICE = 2
PMMC_ERR_CUDA = 3
PMMC_ERR_NOMEM = 4
PMMC_ERR_TIMEOUT = 5
PMMC_ERR_BUDGET = 6
PMMC_ERR_FIXED = 7
PMMC_ERR_BUSY = 8
PMMC_ERR_NOT_FOUND = 9
PMMC_ERR_CANCELLED = 10

SCHEDULE_GPU = 0
SCHEDULE_CPU = 1
LEVEL_ARCS, LEVEL_HEATMAP, LEVEL_SMOOTH = 0, 1, 2

# Symbols the header declares (checked by the CPU tests without calling them).
HEADER_SYMBOLS = [
    "pmmc_ctx_create", "pmmc_ctx_destroy", "pmmc_status_string", "pmmc_last_error",
    "pmmc_set_seed", "pmmc_sm_count", "pmmc_default_params", "pmmc_arcs_dense_to_csr",
    "pmmc_arcs_anneal", "pmmc_smooth_anneal", "pmmc_heatmap_anneal", "pmmc_mark_arcs",
    "pmmc_arcs_batch_create", "pmmc_arcs_batch_run", "pmmc_arcs_batch_results",
    "pmmc_arcs_batch_stats", "pmmc_arcs_batch_destroy", "pmmc_arcs_batch_anneal",
    "pmmc_arcs_batch_create_ex", "pmmc_arcs_batch_trace", "pmmc_smooth_batch_anneal",
    "pmmc_heatmap_batch_anneal", "pmmc_arcs_anneal_noalloc",
    "pmmc_server_create", "pmmc_server_submit", "pmmc_server_poll", "pmmc_server_wait",
    "pmmc_server_get_stats", "pmmc_server_destroy", "pmmc_arcs_batch_classes",
    "pmmc_selftest_sqrt", "pmmc_distance_heatmap", "pmmc_distance_heatmap_device",
    "pmmc_equidistant_model", "pmmc_hcm_write", "pmmc_anchor_targets", "pmmc_stress_refine",
    "pmmc_server_cancel", "pmmc_arcs_batch_trace_chain", "pmmc_arcs_batch_chain_results",
    "pmmc_arcs_rows_to_csr", "pmmc_smooth_set_window", "pmmc_smooth_batch_anneal_packed",
    "pmmc_heatmap_set_cluster",
]

LANES_AUTO = -1  # PMMC_LANES_AUTO: the autotuner picks lanes and warps per class


class PmmcError(RuntimeError):
    def __init__(self, status: int, message: str = ""):
        self.status = status
        super().__init__(f"pmmc status {status}: {message}")


class AnnealParams(C.Structure):
    _fields_ = [
        ("max_temp", C.c_float), ("dt_temp", C.c_float), ("jump_scale", C.c_float),
        ("jump_coef", C.c_float), ("improvement", C.c_float), ("min_successes", C.c_int),
        ("milestone_steps", C.c_int), ("k_stretch", C.c_float), ("k_squeeze", C.c_float),
        ("k_angle", C.c_float), ("w_dist", C.c_float), ("w_angle", C.c_float),
        ("sphere_radius", C.c_float), ("use2d", C.c_int), ("milestone_fails", C.c_int),
        ("schedule", C.c_int), ("resync_every", C.c_int), ("max_moves", C.c_int64),
        ("arcs_extended", C.c_int), ("bond_target", C.c_float),
        ("k_stretch_bond", C.c_float), ("k_squeeze_bond", C.c_float),
        ("k_angle_ext", C.c_float),
    ]


class Result(C.Structure):
    _fields_ = [
        ("score", C.c_float), ("energy", C.c_double), ("energy_fp64", C.c_double),
        ("rel_error", C.c_double), ("moves", C.c_int64), ("accepted", C.c_int64),
        ("total_moves", C.c_int64), ("best_chain", C.c_int), ("status", C.c_int),
    ]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class ArcsProblem(C.Structure):
    _fields_ = [
        ("n", C.c_int), ("pos", C.c_void_p), ("fixed", C.c_void_p), ("row_ptr", C.c_void_p),
        ("col", C.c_void_p), ("target", C.c_void_p), ("n_loops", C.c_int),
        ("loop_i", C.c_void_p), ("loop_j", C.c_void_p), ("loop_k", C.c_void_p),
        ("loop_r0", C.c_void_p),
    ]


class HeatmapProblem(C.Structure):
    _fields_ = [
        ("n", C.c_int), ("pos", C.c_void_p), ("fixed", C.c_void_p), ("heat", C.c_void_p),
        ("diag", C.c_int), ("n_bounds", C.c_int), ("bounds", C.c_void_p),
    ]


class AnchorTargetsProblem(C.Structure):
    _fields_ = [
        ("n", C.c_int), ("active", C.c_void_p), ("arc_ptr", C.c_void_p),
        ("arc_idx", C.c_void_p), ("n_arcs", C.c_int), ("arc_start", C.c_void_p),
        ("arc_end", C.c_void_p), ("arc_score", C.c_void_p), ("n_long", C.c_int),
        ("long_start", C.c_void_p), ("long_end", C.c_void_p), ("long_score", C.c_void_p),
        ("n_anchors", C.c_int), ("anchor_start", C.c_void_p), ("anchor_end", C.c_void_p),
        ("first_cluster", C.c_int), ("freq_memo", C.c_void_p), ("count_a", C.c_float),
        ("count_scale", C.c_float), ("count_shift", C.c_float), ("count_base", C.c_float),
        ("anchor_heat", C.c_void_p), ("anchor_influence", C.c_float),
    ]


class AnchorTargetsStats(C.Structure):
    _fields_ = [("applied", C.c_int64), ("out_of_range", C.c_int64), ("inactive", C.c_int64),
                ("collision", C.c_int64), ("ms_map", C.c_float), ("ms_sort", C.c_float),
                ("ms_resolve", C.c_float), ("ms_assemble", C.c_float)]


class StressProblem(C.Structure):
    _fields_ = [
        ("n", C.c_int), ("active", C.c_void_p), ("genomic_pos", C.c_void_p), ("pos", C.c_void_p),
        ("n_arcs", C.c_int), ("arc_start", C.c_void_p), ("arc_end", C.c_void_p),
        ("arc_score", C.c_void_p), ("n_long", C.c_int), ("long_start", C.c_void_p),
        ("long_end", C.c_void_p), ("long_score", C.c_void_p), ("n_anchors", C.c_int),
        ("anchor_start", C.c_void_p), ("anchor_end", C.c_void_p), ("first_cluster", C.c_int),
    ] + [(k, C.c_float) for k in ("count_a", "count_scale", "count_shift", "count_base",
                                  "glen_base", "glen_scale", "glen_power", "k_stretch",
                                  "k_squeeze", "k_angular")]


class StressResult(C.Structure):
    _fields_ = [("iterations", C.c_int), ("stop", C.c_int), ("lr", C.c_float),
                ("total", C.c_double), ("backbone", C.c_double), ("hic", C.c_double),
                ("angular", C.c_double), ("n_pairs", C.c_int64), ("kernel_ms", C.c_double)]


class SmoothProblem(C.Structure):
    _fields_ = [
        ("n", C.c_int), ("pos", C.c_void_p), ("fixed", C.c_void_p),
        ("dist_to_next", C.c_void_p),
    ]


class BatchOpts(C.Structure):
    _fields_ = [("chains_per_unit", C.c_int), ("use_graph", C.c_int),
                ("lanes_per_chain", C.c_int), ("drawing_warp", C.c_int)]


class ServerOpts(C.Structure):
    _fields_ = [("budget_bytes", C.c_size_t), ("max_waves", C.c_int),
                ("max_wave_requests", C.c_int), ("lanes_per_chain", C.c_int)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_longlong), ("completed", C.c_longlong),
                ("rejected", C.c_longlong), ("failed", C.c_longlong),
                ("waves", C.c_longlong), ("queued", C.c_longlong),
                ("bytes_in_use", C.c_longlong), ("bytes_peak", C.c_longlong),
                ("budget_bytes", C.c_longlong), ("running_peak", C.c_int),
                ("waves_peak", C.c_int)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class MoveTrace(C.Structure):
    _fields_ = [("bead", C.c_int), ("accepted", C.c_int), ("before", C.c_float),
                ("after", C.c_float), ("dx", C.c_float), ("dy", C.c_float),
                ("dz", C.c_float), ("pad", C.c_float)]


TRACE_DTYPE = np.dtype([("bead", np.int32), ("accepted", np.int32), ("before", np.float32),
                        ("after", np.float32), ("dx", np.float32), ("dy", np.float32),
                        ("dz", np.float32), ("pad", np.float32)])

_lib = None


def lib():
    """Load libpmmc_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build it with "
                "python -c 'import __graft_entry__ as g; g.build()'")
        L = C.CDLL(LIB_PATH)
        L.pmmc_status_string.restype = C.c_char_p
        L.pmmc_last_error.restype = C.c_char_p
        L.pmmc_ctx_create.argtypes = [C.POINTER(C.c_void_p), C.c_int]
        L.pmmc_ctx_destroy.argtypes = [C.c_void_p]
        L.pmmc_last_error.argtypes = [C.c_void_p]
        L.pmmc_set_seed.argtypes = [C.c_void_p, C.c_uint64]
        L.pmmc_sm_count.argtypes = [C.c_void_p]
        L.pmmc_smooth_set_window.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int]
        L.pmmc_heatmap_set_cluster.argtypes = [C.c_void_p, C.c_int]
        L.pmmc_arcs_batch_destroy.argtypes = [C.c_void_p]
        L.pmmc_server_create.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.POINTER(C.c_void_p)]
        L.pmmc_server_submit.argtypes = [C.c_void_p, C.c_void_p, C.c_float, C.c_uint64,
                                         C.POINTER(C.c_longlong)]
        L.pmmc_server_poll.argtypes = [C.c_void_p, C.c_longlong, C.POINTER(C.c_int)]
        L.pmmc_server_wait.argtypes = [C.c_void_p, C.c_longlong, C.c_int, C.c_void_p,
                                       C.c_void_p, C.POINTER(C.c_double)]
        L.pmmc_server_get_stats.argtypes = [C.c_void_p, C.c_void_p]
        L.pmmc_server_destroy.argtypes = [C.c_void_p]
        L.pmmc_server_destroy.restype = None
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def default_params(level: int = LEVEL_ARCS, **kw) -> AnnealParams:
    p = AnnealParams()
    lib().pmmc_default_params(int(level), C.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise AttributeError(k)
        setattr(p, k, v)
    return p


def dense_to_csr(dense: np.ndarray):
    """Reference dense matrix -> (row_ptr, col, target) over both directions
    (pmmc_arcs_dense_to_csr)."""
    d = _f32(dense)
    n = d.shape[0]
    rp = np.zeros(n + 1, np.int32)
    nnz = C.c_int64()
    _check(None, lib().pmmc_arcs_dense_to_csr(n, _p(d), _p(rp), None, None, C.c_int64(0),
                                              C.byref(nnz)))
    col = np.zeros(max(nnz.value, 1), np.int32)
    tgt = np.zeros(max(nnz.value, 1), np.float32)
    _check(None, lib().pmmc_arcs_dense_to_csr(n, _p(d), _p(rp), _p(col), _p(tgt),
                                              C.c_int64(nnz.value), C.byref(nnz)))
    return rp, col[:nnz.value], tgt[:nnz.value]


def _check(ctx, status):
    if status != PMMC_OK:
        msg = lib().pmmc_status_string(status).decode()
        if ctx is not None:
            le = lib().pmmc_last_error(ctx)
            if le:
                msg += ": " + le.decode()
        raise PmmcError(status, msg)


class Context:
    """Owns a pmmc_ctx (replaces the reference's GpuResourceCache)."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        _check(None, lib().pmmc_ctx_create(C.byref(h), int(device)))
        self.h = h

    def close(self):
        if self.h:
            lib().pmmc_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, status):
        _check(self.h, status)

    def set_seed(self, seed: int):
        lib().pmmc_set_seed(self.h, C.c_uint64(int(seed) & (2**64 - 1)))

    def set_smooth_window(self, window: int = 8, window_long: int | None = None,
                          long_min_free: int = 16):
        """Smoothing kernel choice (pmmc_smooth_set_window): regions with at
        least `long_min_free` movable beads are annealed `window_long`
        proposals at a time, the others `window` at a time (0 = one move at
        a time).  window_long defaults to `window`."""
        wl = window if window_long is None else window_long
        self.check(lib().pmmc_smooth_set_window(self.h, int(window), int(wl), int(long_min_free)))

    def set_heatmap_cluster(self, ctas: int = 0):
        """Heatmap kernel choice (pmmc_heatmap_set_cluster): CTAs of the
        thread-block cluster that runs one chain (0 = by the batch)."""
        self.check(lib().pmmc_heatmap_set_cluster(self.h, int(ctas)))

    @property
    def sm_count(self) -> int:
        return lib().pmmc_sm_count(self.h)


class ArcsInput:
    """Keeps the numpy arrays of one arc problem alive behind the C struct,
    which is built once, at construction (its pointers are into this
    object's own arrays: change them in place, do not rebind them)."""

    def __init__(self, pos, row_ptr, col, target, fixed=None, loops=None):
        self.pos = _f32(pos).reshape(-1, 3)
        self.row_ptr = _i32(row_ptr)
        self.col = _i32(col) if len(col) else np.zeros(1, np.int32)
        self.target = _f32(target) if len(target) else np.zeros(1, np.float32)
        self.fixed = None if fixed is None else np.ascontiguousarray(fixed, dtype=np.uint8)
        if loops is None:
            loops = (np.zeros(0, np.int32),) * 2 + (np.zeros(0, np.float32),) * 2
        self.li, self.lj = _i32(loops[0]), _i32(loops[1])
        self.lk, self.lr = _f32(loops[2]), _f32(loops[3])
        self.n = self.pos.shape[0]
        n_l = len(self.li)
        self._struct = ArcsProblem(self.n, _p(self.pos), _p(self.fixed), _p(self.row_ptr),
                                   _p(self.col), _p(self.target), n_l,
                                   _p(self.li) if n_l else None, _p(self.lj) if n_l else None,
                                   _p(self.lk) if n_l else None, _p(self.lr) if n_l else None)

    @classmethod
    def from_dense(cls, pos, dense, fixed=None, loops=None):
        rp, col, tgt = dense_to_csr(dense)
        return cls(pos, rp, col, tgt, fixed, loops)

    def struct(self) -> ArcsProblem:
        return self._struct


class ArcsBatch:
    """Device-resident batch of arc regions (pmmc_arcs_batch_*)."""

    def __init__(self, ctx: Context, inputs, params: AnnealParams, steps, chains=1,
                 use_graph=True, stop_all=False, trace_cap=0, lanes=0, drawing_warp=False):
        self.ctx = ctx
        self.inputs = list(inputs)
        arr = (ArcsProblem * len(self.inputs))(*[x.struct() for x in self.inputs])
        self._arr = arr
        self.steps = _f32(steps)
        opts = BatchOpts(int(chains), int(bool(use_graph)), int(lanes), int(bool(drawing_warp)))
        h = C.c_void_p()
        ctx.check(lib().pmmc_arcs_batch_create_ex(
            ctx.h, len(self.inputs), arr, C.byref(params), _p(self.steps), C.byref(opts),
            int(bool(stop_all)), int(trace_cap), C.byref(h)))
        self.h = h
        self.trace_cap = trace_cap

    def run(self, stream=None):
        self.ctx.check(lib().pmmc_arcs_batch_run(self.h, C.c_void_p(stream) if stream else None))

    def results(self):
        tot = sum(x.n for x in self.inputs)
        pos = np.zeros((tot, 3), np.float32)
        res = (Result * len(self.inputs))()
        self.ctx.check(lib().pmmc_arcs_batch_results(self.h, _p(pos), res))
        out, off = [], 0
        for x in self.inputs:
            out.append(pos[off:off + x.n])
            off += x.n
        return out, [r for r in res]

    def stats(self):
        ms = C.c_double()
        mv = C.c_int64()
        lanes = C.c_int()
        self.ctx.check(lib().pmmc_arcs_batch_stats(self.h, C.byref(ms), C.byref(mv),
                                                   C.byref(lanes)))
        return ms.value, mv.value, lanes.value

    def classes(self):
        """Per shared-memory class: (lanes, chains per CTA, items, staged,
        drawing warp)."""
        cap = 64
        n = C.c_int()
        la, wa, it, nb, dw = ((C.c_int * cap)() for _ in range(5))
        self.ctx.check(lib().pmmc_arcs_batch_classes(self.h, cap, C.byref(n), la, wa, it, nb, dw))
        return [(la[k], wa[k], it[k], bool(nb[k]), bool(dw[k]))
                for k in range(min(n.value, cap))]

    def trace(self, count=None, chain=0):
        """The first `count` trace records of chain `chain` of region 0."""
        count = self.trace_cap if count is None else count
        out = np.zeros(count, TRACE_DTYPE)
        self.ctx.check(lib().pmmc_arcs_batch_trace_chain(self.h, int(chain), _p(out),
                                                         int(count)))
        return out

    def chain_results(self, unit=0):
        """The result of every chain of region `unit`, in chain order."""
        n = C.c_int()
        self.ctx.check(lib().pmmc_arcs_batch_chain_results(self.h, int(unit), 0, None,
                                                           C.byref(n)))
        res = (Result * max(n.value, 1))()
        self.ctx.check(lib().pmmc_arcs_batch_chain_results(self.h, int(unit), n.value, res,
                                                           C.byref(n)))
        return [res[k] for k in range(n.value)]

    def close(self):
        if self.h:
            lib().pmmc_arcs_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def arcs_anneal(ctx: Context, inp: ArcsInput, params: AnnealParams, step: float,
                n_chains: int = 0):
    pos = np.zeros((inp.n, 3), np.float32)
    res = Result()
    s = inp.struct()
    ctx.check(lib().pmmc_arcs_anneal(ctx.h, C.byref(s), C.byref(params), C.c_float(step),
                                     int(n_chains), _p(pos), C.byref(res)))
    return pos, res


class Server:
    """Request loop over arc-level regions (pmmc_server_*): submit from any
    thread, results come back per ticket with their latency."""

    def __init__(self, ctx: Context, params: AnnealParams, budget_bytes: int = 0,
                 max_waves: int = 0, max_wave_requests: int = 0, lanes: int = 0):
        self.ctx = ctx
        self.params = params
        opts = ServerOpts(int(budget_bytes), int(max_waves), int(max_wave_requests), int(lanes))
        h = C.c_void_p()
        ctx.check(lib().pmmc_server_create(ctx.h, C.byref(params), C.byref(opts), C.byref(h)))
        self.h = h
        self._n = {}

    def submit(self, inp: ArcsInput, step: float, seed: int) -> int:
        s = inp.struct()
        t = C.c_longlong()
        self.ctx.check(lib().pmmc_server_submit(self.h, C.byref(s), C.c_float(step),
                                                C.c_uint64(int(seed) & (2**64 - 1)),
                                                C.byref(t)))
        self._n[t.value] = inp.n
        return t.value

    def poll(self, ticket: int) -> bool:
        d = C.c_int()
        self.ctx.check(lib().pmmc_server_poll(self.h, C.c_longlong(ticket), C.byref(d)))
        return bool(d.value)

    def wait(self, ticket: int, timeout_ms: int = -1):
        """(positions, Result, latency_ms) of a finished request."""
        pos = np.zeros((self._n.get(ticket, 0), 3), np.float32)
        res = Result()
        lat = C.c_double()
        self.ctx.check(lib().pmmc_server_wait(self.h, C.c_longlong(ticket), int(timeout_ms),
                                              _p(pos), C.byref(res), C.byref(lat)))
        self._n.pop(ticket, None)
        return pos, res, lat.value

    def cancel(self, ticket: int) -> int:
        """pmmc_server_cancel: the status (0 = withdrawn while queued)."""
        return int(lib().pmmc_server_cancel(self.h, C.c_longlong(ticket)))

    def stats(self) -> dict:
        st = ServerStats()
        self.ctx.check(lib().pmmc_server_get_stats(self.h, C.byref(st)))
        return st.as_dict()

    def close(self):
        if self.h:
            lib().pmmc_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class SmoothInput:
    """One smoothing region; the C struct is built once, at construction,
    with pointers into this object's own arrays."""

    def __init__(self, pos, dist_to_next, fixed=None):
        self.pos = _f32(pos).reshape(-1, 3)
        self.dtn = _f32(dist_to_next)
        self.fixed = None if fixed is None else np.ascontiguousarray(fixed, dtype=np.uint8)
        self.n = self.pos.shape[0]
        self._struct = SmoothProblem(self.n, _p(self.pos), _p(self.fixed), _p(self.dtn))

    def struct(self) -> SmoothProblem:
        return self._struct


def smooth_batch_anneal(ctx: Context, inputs, params: AnnealParams, steps, chains=1,
                        trace_cap=0):
    inputs = list(inputs)
    arr = (SmoothProblem * len(inputs))(*[x.struct() for x in inputs])
    st = _f32(steps)
    tot = sum(x.n for x in inputs)
    pos = np.zeros((tot, 3), np.float32)
    res = (Result * len(inputs))()
    ms = C.c_double()
    tr = np.zeros(max(trace_cap, 1), TRACE_DTYPE)
    ctx.check(lib().pmmc_smooth_batch_anneal(ctx.h, len(inputs), arr, C.byref(params), _p(st),
                                             int(chains), _p(pos), res, C.byref(ms),
                                             _p(tr) if trace_cap else None, int(trace_cap)))
    out, off = [], 0
    for x in inputs:
        out.append(pos[off:off + x.n])
        off += x.n
    if trace_cap:
        return out, [r for r in res], ms.value, tr
    return out, [r for r in res], ms.value


def smooth_batch_anneal_packed(ctx: Context, bead_off, pos, dist_to_next, fixed,
                               params: AnnealParams, steps, chains=1, trace_cap=0):
    """Regions packed back to back (pmmc_smooth_batch_anneal_packed): region u
    is rows [bead_off[u], bead_off[u+1]) of pos (n x 3), dist_to_next and
    fixed.  Returns (positions n x 3 of each region's reported chain, the
    ctypes array of results, kernel ms[, trace])."""
    off = np.ascontiguousarray(bead_off, dtype=np.int64)
    n_units = len(off) - 1
    pos = _f32(pos).reshape(-1, 3)
    dtn = _f32(dist_to_next)
    fx = None if fixed is None else np.ascontiguousarray(fixed, dtype=np.uint8)
    st = _f32(steps)
    out = np.zeros_like(pos)
    res = (Result * n_units)()
    ms = C.c_double()
    tr = np.zeros(max(trace_cap, 1), TRACE_DTYPE)
    ctx.check(lib().pmmc_smooth_batch_anneal_packed(
        ctx.h, n_units, _p(off), _p(pos), _p(dtn), _p(fx), C.byref(params), _p(st), int(chains),
        _p(out), res, C.byref(ms), _p(tr) if trace_cap else None, int(trace_cap)))
    if trace_cap:
        return out, res, ms.value, tr
    return out, res, ms.value


def smooth_anneal(ctx: Context, inp: SmoothInput, params: AnnealParams, step: float,
                  n_chains: int = 0):
    pos = np.zeros((inp.n, 3), np.float32)
    res = Result()
    s = inp.struct()
    ctx.check(lib().pmmc_smooth_anneal(ctx.h, C.byref(s), C.byref(params), C.c_float(step),
                                       int(n_chains), _p(pos), C.byref(res)))
    return pos, res


class HeatmapInput:
    def __init__(self, pos, heat, diag=1, bounds=None, fixed=None):
        self.pos = _f32(pos).reshape(-1, 3)
        self.heat = _f32(heat)
        self.diag = int(diag)
        self.bounds = _i32(bounds if bounds is not None else np.zeros(0, np.int32))
        self.fixed = None if fixed is None else np.ascontiguousarray(fixed, dtype=np.uint8)
        self.n = self.pos.shape[0]

    def struct(self) -> HeatmapProblem:
        nb = len(self.bounds)
        return HeatmapProblem(self.n, _p(self.pos), _p(self.fixed), _p(self.heat), self.diag,
                              nb, _p(self.bounds) if nb else None)


def heatmap_batch_anneal(ctx: Context, inputs, params: AnnealParams, steps, trace_cap=0):
    inputs = list(inputs)
    arr = (HeatmapProblem * len(inputs))(*[x.struct() for x in inputs])
    st = _f32(steps)
    tot = sum(x.n for x in inputs)
    pos = np.zeros((tot, 3), np.float32)
    res = (Result * len(inputs))()
    ms = C.c_double()
    tr = np.zeros(max(trace_cap, 1), TRACE_DTYPE)
    ctx.check(lib().pmmc_heatmap_batch_anneal(ctx.h, len(inputs), arr, C.byref(params), _p(st),
                                              _p(pos), res, C.byref(ms),
                                              _p(tr) if trace_cap else None, int(trace_cap)))
    out, off = [], 0
    for x in inputs:
        out.append(pos[off:off + x.n])
        off += x.n
    return out, [r for r in res], ms.value, (tr if trace_cap else None)


def heatmap_anneal(ctx: Context, inp: HeatmapInput, params: AnnealParams, step: float):
    pos = np.zeros((inp.n, 3), np.float32)
    res = Result()
    s = inp.struct()
    ctx.check(lib().pmmc_heatmap_anneal(ctx.h, C.byref(s), C.byref(params), C.c_float(step),
                                        _p(pos), C.byref(res)))
    return pos, res


def distance_heatmap(ctx: Context, contact, diag: int, scale: float, power: float,
                     stretching: float):
    """pmmc_distance_heatmap: (n x n distance map, avg, clamp value, kernel ms)."""
    c = _f32(contact)
    n = c.shape[0]
    out = np.zeros((n, n), np.float32)
    avg, mx, ms = C.c_float(), C.c_float(), C.c_double()
    ctx.check(lib().pmmc_distance_heatmap(ctx.h, n, _p(c), int(diag), C.c_float(scale),
                                          C.c_float(power), C.c_float(stretching), _p(out),
                                          C.byref(avg), C.byref(mx), C.byref(ms)))
    return out, avg.value, mx.value, ms.value


def anchor_targets_arrays(t: dict) -> dict:
    """The arrays of an anchor-target problem dict (keys: active, arc_ptr,
    arc_idx, arc_start, arc_end, arc_score, long_start, long_end, long_score,
    anc_start, anc_end, first_cluster, memo, count = (a, scale, shift, base),
    heat or None, influence) as contiguous int32 / float32 arrays."""
    out = {k: _i32(t[k]) for k in ("active", "arc_ptr", "arc_idx", "arc_start", "arc_end",
                                   "arc_score", "long_start", "long_end", "long_score",
                                   "anc_start", "anc_end")}
    out["memo"] = _f32(t["memo"])
    out["heat"] = None if t.get("heat") is None else _f32(t["heat"])
    return out


def anchor_targets(ctx: Context, t: dict):
    """pmmc_anchor_targets: (row_ptr, col, target, stats dict, kernel ms).
    The stats dict holds the long-arc counters; anchor_targets_phases()
    gives the per-phase device times of the last call."""
    a = anchor_targets_arrays(t)
    n = len(a["active"])
    ca, cs, csh, cb = (float(x) for x in t["count"])
    pr = AnchorTargetsProblem(
        n, _p(a["active"]), _p(a["arc_ptr"]), _p(a["arc_idx"]), len(a["arc_start"]),
        _p(a["arc_start"]), _p(a["arc_end"]), _p(a["arc_score"]), len(a["long_start"]),
        _p(a["long_start"]), _p(a["long_end"]), _p(a["long_score"]), len(a["anc_start"]),
        _p(a["anc_start"]), _p(a["anc_end"]), int(t["first_cluster"]), _p(a["memo"]), ca, cs,
        csh, cb, _p(a["heat"]), float(t.get("influence", 0.0)))
    cap = 2 * (int(a["arc_ptr"][-1]) + len(a["long_start"]))
    row_ptr = np.zeros(n + 1, np.int32)
    col = np.zeros(max(cap, 1), np.int32)
    tgt = np.zeros(max(cap, 1), np.float32)
    nnz = C.c_int64()
    st = AnchorTargetsStats()
    ms = C.c_double()
    ctx.check(lib().pmmc_anchor_targets(ctx.h, C.byref(pr), _p(row_ptr), _p(col), _p(tgt),
                                        C.c_int64(cap), C.byref(nnz), C.byref(st),
                                        C.byref(ms)))
    k = nnz.value
    stats = {"applied": st.applied, "out_of_range": st.out_of_range, "inactive": st.inactive,
             "collision": st.collision}
    global _last_target_phases
    _last_target_phases = {"map": st.ms_map, "sort": st.ms_sort, "resolve": st.ms_resolve,
                           "assemble": st.ms_assemble}
    return row_ptr, col[:k].copy(), tgt[:k].copy(), stats, ms.value


_last_target_phases: dict = {}


def anchor_targets_phases() -> dict:
    """Device milliseconds per phase of the last anchor_targets call."""
    return dict(_last_target_phases)


def stress_arrays(t: dict) -> dict:
    """Arrays of a stress-refinement problem dict (keys: active, genomic_pos,
    pos, arc_start, arc_end, arc_score, long_start, long_end, long_score,
    anc_start, anc_end, first_cluster, count = (a, scale, shift, base),
    glen = (base, scale, power), springs = (k_stretch, k_squeeze, k_angular))."""
    out = {k: _i32(t[k]) for k in ("active", "genomic_pos", "arc_start", "arc_end",
                                   "arc_score", "long_start", "long_end", "long_score",
                                   "anc_start", "anc_end")}
    out["pos"] = _f32(t["pos"]).reshape(-1, 3)
    return out


def stress_refine(ctx: Context, t: dict, max_iter: int, lr: float):
    """pmmc_stress_refine: (order, positions n x 3 in that order, result dict)."""
    a = stress_arrays(t)
    n = len(a["active"])
    pr = StressProblem(
        n, _p(a["active"]), _p(a["genomic_pos"]), _p(a["pos"]), len(a["arc_start"]),
        _p(a["arc_start"]), _p(a["arc_end"]), _p(a["arc_score"]), len(a["long_start"]),
        _p(a["long_start"]), _p(a["long_end"]), _p(a["long_score"]), len(a["anc_start"]),
        _p(a["anc_start"]), _p(a["anc_end"]), int(t["first_cluster"]),
        *(float(x) for x in t["count"]), *(float(x) for x in t["glen"]),
        *(float(x) for x in t["springs"]))
    order = np.zeros(max(n, 1), np.int32)
    pos = np.zeros((max(n, 1), 3), np.float32)
    r = StressResult()
    ctx.check(lib().pmmc_stress_refine(ctx.h, C.byref(pr), int(max_iter), C.c_float(lr),
                                       _p(order), _p(pos), C.byref(r)))
    return order[:n], pos[:n], {k: getattr(r, k) for k, _ in StressResult._fields_}


def equidistant_model(ctx: Context, gpos, pos, first_end: int, last_start: int,
                      pos_start: int, pos_stop: int, res: int):
    """pmmc_equidistant_model: (points m x 3, kernel ms)."""
    g = _i32(gpos)
    p = _f32(pos).reshape(-1, 3)
    m = C.c_int64()
    ms = C.c_double()
    ctx.check(lib().pmmc_equidistant_model(ctx.h, len(g), _p(g), _p(p), int(first_end),
                                           int(last_start), int(pos_start), int(pos_stop),
                                           int(res), None, C.c_int64(0), C.byref(m), None))
    out = np.zeros((m.value, 3), np.float32)
    ctx.check(lib().pmmc_equidistant_model(ctx.h, len(g), _p(g), _p(p), int(first_end),
                                           int(last_start), int(pos_start), int(pos_stop),
                                           int(res), _p(out), C.c_int64(m.value), C.byref(m),
                                           C.byref(ms)))
    return out, ms.value


def hcm_write(path: str, start, end, orientation, pos, children, factors, chrs):
    """pmmc_hcm_write.  children: one list per cluster; factors: names;
    chrs: list of (name, root, arcs as rows of 7 ints)."""
    n = len(start)
    st, en = _i32(start), _i32(end)
    ori = np.frombuffer("".join(orientation).encode(), np.uint8).copy() if n else np.zeros(1, np.uint8)
    p = _f32(pos).reshape(-1, 3)
    cp = _i32(np.concatenate([[0], np.cumsum([len(c) for c in children])]) if n else [0])
    ch = _i32([x for c in children for x in c] or [0])
    fac = [f.encode() for f in factors]
    fac_arr = (C.c_char_p * max(len(fac), 1))(*fac)
    names = [c[0].encode() for c in chrs]
    names_arr = (C.c_char_p * max(len(names), 1))(*names)
    roots = _i32([c[1] for c in chrs] or [0])
    ap = _i32(np.concatenate([[0], np.cumsum([len(c[2]) for c in chrs])]) if chrs else [0])
    arcs = _i32(np.array([a for c in chrs for a in c[2]], np.int32).reshape(-1) if chrs else [0])
    if arcs.size == 0:
        arcs = np.zeros(7, np.int32)
    st_ = lib().pmmc_hcm_write(path.encode(), n, _p(st), _p(en), _p(ori), _p(p), _p(cp), _p(ch),
                               len(fac), fac_arr, len(chrs), names_arr, _p(roots), _p(ap),
                               _p(arcs))
    _check(None, st_)


def selftest_sqrt(ctx: Context, lo: int, count: int):
    """(mismatches, lowest differing bit pattern) of the kernels' square root
    against the IEEE routine on float bit patterns [lo, lo + count)."""
    bad = C.c_uint64()
    first = C.c_uint32()
    ctx.check(lib().pmmc_selftest_sqrt(ctx.h, C.c_uint32(lo), C.c_uint32(count), C.byref(bad),
                                       C.byref(first)))
    return bad.value, first.value


def mark_arcs(ctx: Context, anchors, raw):
    a = _i32(anchors).reshape(-1, 2)
    r = _i32(raw).reshape(-1, 4)
    cols = [np.ascontiguousarray(a[:, k]) for k in range(2)]
    rc = [np.ascontiguousarray(r[:, k]) for k in range(4)]
    cap = 2 * len(r) + 8
    out = np.zeros((cap, 7), np.int32)
    n_out = C.c_int()
    nm = C.c_int()
    ctx.check(lib().pmmc_mark_arcs(ctx.h, len(a), _p(cols[0]), _p(cols[1]), len(r), _p(rc[0]),
                                   _p(rc[1]), _p(rc[2]), _p(rc[3]), _p(out), cap,
                                   C.byref(n_out), C.byref(nm)))
    return out[:n_out.value].copy(), nm.value


def arcs_anneal_noalloc(prob_dev: ArcsProblem, params: AnnealParams, step: float, seed: int,
                        pos_out_dev: int, stream: int = 0) -> Result:
    """pmmc_arcs_anneal_noalloc: every pointer of prob_dev and pos_out_dev is
    a device address owned by the caller; nothing is allocated."""
    res = Result()
    st = lib().pmmc_arcs_anneal_noalloc(C.byref(prob_dev), C.byref(params), C.c_float(step),
                                        C.c_uint64(int(seed) & (2**64 - 1)),
                                        C.c_void_p(pos_out_dev), C.byref(res),
                                        C.c_void_p(stream) if stream else None)
    _check(None, st)
    return res
