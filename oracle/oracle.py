"""ctypes loader for the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import
this module; the product package never does.  Two libraries sit behind it:

* ``liboracle.so`` -- the plain-C restatement (pmmc_oracle.c) of the
  reference's CPU annealers, arc marking and HCM lines;
* ``_ref/libpmmc_ref.so`` -- the reference's own CPU code (built from its
  sources by oracle/Makefile, present only where the reference tree exists).

Arrays are numpy; positions are (n, 3) float32.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libpmmc_ref.so")

RNG_LIBC = 0
RNG_PHILOX = 1
# stopping schedules (orc_params.schedule): the reference's CPU loops, or the
# schedule of its CUDA kernels (256-move blocks, milestone_fails)
SCHEDULE_CPU = 0
SCHEDULE_GPU = 1


class OrcParams(C.Structure):
    _fields_ = [
        ("max_temp", C.c_float),
        ("dt_temp", C.c_float),
        ("jump_scale", C.c_float),
        ("jump_coef", C.c_float),
        ("improvement", C.c_float),
        ("min_successes", C.c_int),
        ("milestone_steps", C.c_int),
        ("k_stretch", C.c_float),
        ("k_squeeze", C.c_float),
        ("k_angle", C.c_float),
        ("w_dist", C.c_float),
        ("w_angle", C.c_float),
        ("sphere_radius", C.c_float),
        ("use2d", C.c_int),
        ("max_moves", C.c_int64),
        ("schedule", C.c_int),
        ("milestone_fails", C.c_int),
    ]


class OrcRng(C.Structure):
    _fields_ = [
        ("kind", C.c_int),
        ("seed", C.c_uint64),
        ("chain", C.c_uint32),
        ("move", C.c_uint64),
    ]


class OrcResult(C.Structure):
    _fields_ = [
        ("score", C.c_double),
        ("moves", C.c_int64),
        ("accepted", C.c_int64),
        ("proposals", C.c_int64),
        ("best", C.c_double),
    ]


@dataclass
class Params:
    """Annealing parameters with the reference's Settings defaults
    (src/include/Settings.hpp:479-505)."""

    max_temp: float = 20.0
    dt_temp: float = 0.99995
    jump_scale: float = 50.0
    jump_coef: float = 20.0
    improvement: float = 0.995
    min_successes: int = 5
    milestone_steps: int = 10000
    k_stretch: float = 1.0
    k_squeeze: float = 1.0
    k_angle: float = 0.1
    w_dist: float = 1.0
    w_angle: float = 1.0
    sphere_radius: float = 0.0
    use2d: int = 0
    max_moves: int = 0
    schedule: int = SCHEDULE_CPU
    milestone_fails: int = 3

    def c(self) -> OrcParams:
        return OrcParams(*[getattr(self, f[0]) for f in OrcParams._fields_])


def build() -> None:
    """Compile liboracle.so (and _ref when the reference tree exists)."""
    subprocess.run(["make", "-C", HERE, "-s"], check=True, stdout=sys.stderr)


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _u8(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.uint8)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.orc_arcs_full_score.restype = C.c_double
        L.orc_arcs_spring_score.restype = C.c_double
        L.orc_arcs_repulsion.restype = C.c_double
        L.orc_arcs_local_score.restype = C.c_double
        L.orc_heatmap_score.restype = C.c_double
        L.orc_smooth_full_score.restype = C.c_double
        L.orc_smooth_local_score.restype = C.c_double
        L.orc_u01.restype = C.c_float
        L.orc_arcs_ext_score.restype = C.c_double
        L.orc_u01.argtypes = [C.c_uint32]
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_PATH)


def ref():
    global _ref
    if _ref is None:
        if not os.path.exists(REF_PATH):
            raise FileNotFoundError(REF_PATH)
        R = C.CDLL(REF_PATH)
        R.ref_arcs_score.restype = C.c_double
        R.ref_heatmap_score.restype = C.c_double
        R.ref_smooth_score.restype = C.c_double
        R.ref_lengths_score.restype = C.c_double
        R.ref_rmsd.restype = C.c_double
        R.ref_distance_correlation.restype = C.c_double
        _ref = R
    return _ref


# ---------------------------------------------------------------------------
# Problems
# ---------------------------------------------------------------------------
@dataclass
class ArcsProblem:
    """One arc-level active region in the reference layout: positions, fixed
    flags, the dense n x n expected-distance matrix (-1 = no arc, 0 on the
    diagonal) and loop constraints (cluster_i, cluster_j, stiffness, r0)."""

    pos: np.ndarray
    exp_dist: np.ndarray
    fixed: np.ndarray | None = None
    loops_i: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    loops_j: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    loops_k: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    loops_r0: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))

    @property
    def n(self):
        return int(self.pos.shape[0])

    def loop_args(self):
        return (len(self.loops_i), _p(_i32(self.loops_i)), _p(_i32(self.loops_j)),
                _p(_f32(self.loops_k)), _p(_f32(self.loops_r0)))


def _loops(pr):
    li, lj, lk, lr = _i32(pr.loops_i), _i32(pr.loops_j), _f32(pr.loops_k), _f32(pr.loops_r0)
    return (len(li), _p(li), _p(lj), _p(lk), _p(lr)), (li, lj, lk, lr)


def arcs_full(pr: ArcsProblem, prm: Params, pos=None, repulsion=True) -> float:
    pos = _f32(pr.pos if pos is None else pos)
    ed = _f32(pr.exp_dist)
    la, keep = _loops(pr)
    f = lib().orc_arcs_full_score if repulsion else lib().orc_arcs_spring_score
    return f(pr.n, _p(pos), _p(ed), *la, C.byref(prm.c()))


def arcs_repulsion(pr: ArcsProblem, pos=None) -> float:
    pos = _f32(pr.pos if pos is None else pos)
    return lib().orc_arcs_repulsion(pr.n, _p(pos), _p(_f32(pr.exp_dist)))


def arcs_local(pr: ArcsProblem, prm: Params, moved: int, pos=None) -> float:
    pos = _f32(pr.pos if pos is None else pos)
    ed = _f32(pr.exp_dist)
    la, keep = _loops(pr)
    return lib().orc_arcs_local_score(pr.n, _p(pos), _p(ed), *la, C.byref(prm.c()),
                                      int(moved))


class Ext(C.Structure):
    """Extended arc energy (orc_ext): one bond target, the bond constants
    and the angle constant."""
    _fields_ = [("bond_target", C.c_double), ("k_stretch", C.c_float),
                ("k_squeeze", C.c_float), ("k_angle", C.c_float)]


def arcs_ext_score(n: int, pos, ext: Ext, moved: int = -1) -> float:
    return lib().orc_arcs_ext_score(int(n), _p(_f32(pos)), C.byref(ext), int(moved))


def arcs_anneal(pr: ArcsProblem, prm: Params, step: float, seed: int,
                rng=RNG_LIBC, chain=0, ext: Ext | None = None):
    pos = _f32(pr.pos).copy()
    ed = _f32(pr.exp_dist)
    fx = _u8(pr.fixed)
    la, keep = _loops(pr)
    r = OrcRng(rng, seed, chain, 0)
    res = OrcResult()
    lib().orc_arcs_anneal_ext(pr.n, _p(pos), _p(fx), _p(ed), *la, C.byref(prm.c()),
                              C.byref(ext) if ext is not None else None,
                              C.c_float(step), C.byref(r), C.byref(res))
    return pos, res


def ref_arcs_anneal(pr: ArcsProblem, prm: Params, step: float, seed: int):
    pos = _f32(pr.pos).copy()
    ed = _f32(pr.exp_dist)
    fx = _u8(pr.fixed)
    la, keep = _loops(pr)
    sc = C.c_double()
    mv = C.c_longlong()
    ref().ref_arcs_anneal(pr.n, _p(pos), _p(fx), _p(ed), *la, C.byref(prm.c()),
                          C.c_float(step), C.c_uint(seed), C.byref(sc), C.byref(mv))
    return pos, sc.value, mv.value


def ref_arcs_score(pr: ArcsProblem, prm: Params, moved: int, pos=None) -> float:
    pos = _f32(pr.pos if pos is None else pos)
    ed = _f32(pr.exp_dist)
    la, keep = _loops(pr)
    return ref().ref_arcs_score(pr.n, _p(pos), _p(ed), *la, C.byref(prm.c()), int(moved))


@dataclass
class HeatmapProblem:
    pos: np.ndarray
    heat: np.ndarray
    diag: int = 1
    bounds: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    fixed: np.ndarray | None = None

    @property
    def n(self):
        return int(self.pos.shape[0])


def heatmap_score(pr: HeatmapProblem, moved=-1, pos=None) -> float:
    pos = _f32(pr.pos if pos is None else pos)
    b = _i32(pr.bounds)
    return lib().orc_heatmap_score(pr.n, _p(pos), _p(_f32(pr.heat)), int(pr.diag),
                                   len(b), _p(b), int(moved))


def heatmap_anneal(pr: HeatmapProblem, prm: Params, step: float, seed: int,
                   rng=RNG_LIBC, incremental=False, chain=0):
    pos = _f32(pr.pos).copy()
    b = _i32(pr.bounds)
    fx = _u8(pr.fixed)
    r = OrcRng(rng, seed, chain, 0)
    res = OrcResult()
    lib().orc_heatmap_anneal(pr.n, _p(pos), _p(fx), _p(_f32(pr.heat)), int(pr.diag),
                             len(b), _p(b), C.byref(prm.c()), C.c_float(step),
                             int(bool(incremental)), C.byref(r), C.byref(res))
    return pos, res


def ref_heatmap_anneal(pr: HeatmapProblem, prm: Params, step: float, seed: int):
    pos = _f32(pr.pos).copy()
    b = _i32(pr.bounds)
    fx = _u8(pr.fixed)
    sc = C.c_double()
    mv = C.c_longlong()
    ref().ref_heatmap_anneal(pr.n, _p(pos), _p(fx), _p(_f32(pr.heat)), int(pr.diag),
                             len(b), _p(b), C.byref(prm.c()), C.c_float(step),
                             C.c_uint(seed), C.byref(sc), C.byref(mv))
    return pos, sc.value, mv.value


def ref_heatmap_score(pr: HeatmapProblem, moved=-1, pos=None) -> float:
    pos = _f32(pr.pos if pos is None else pos)
    b = _i32(pr.bounds)
    return ref().ref_heatmap_score(pr.n, _p(pos), _p(_f32(pr.heat)), int(pr.diag),
                                   len(b), _p(b), int(moved))


@dataclass
class SmoothProblem:
    pos: np.ndarray
    dist_to_next: np.ndarray
    fixed: np.ndarray | None = None

    @property
    def n(self):
        return int(self.pos.shape[0])


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def smooth_full(pr: SmoothProblem, prm: Params, pos=None) -> float:
    pos = _f32(pr.pos if pos is None else pos)
    return lib().orc_smooth_full_score(pr.n, _p(pos), _p(_f64(pr.dist_to_next)),
                                       C.byref(prm.c()))


def smooth_local(pr: SmoothProblem, prm: Params, moved: int, pos=None) -> float:
    pos = _f32(pr.pos if pos is None else pos)
    return lib().orc_smooth_local_score(pr.n, _p(pos), _p(_f64(pr.dist_to_next)),
                                        C.byref(prm.c()), int(moved))


def smooth_anneal(pr: SmoothProblem, prm: Params, step: float, seed: int,
                  rng=RNG_LIBC, chain=0):
    pos = _f32(pr.pos).copy()
    fx = _u8(pr.fixed)
    r = OrcRng(rng, seed, chain, 0)
    res = OrcResult()
    lib().orc_smooth_anneal(pr.n, _p(pos), _p(fx), _p(_f64(pr.dist_to_next)),
                            C.byref(prm.c()), C.c_float(step), C.byref(r), C.byref(res))
    return pos, res


def ref_smooth_anneal(pr: SmoothProblem, prm: Params, step: float, seed: int):
    pos = _f32(pr.pos).copy()
    fx = _u8(pr.fixed)
    sc = C.c_double()
    mv = C.c_longlong()
    ref().ref_smooth_anneal(pr.n, _p(pos), _p(fx), _p(_f64(pr.dist_to_next)),
                            C.byref(prm.c()), C.c_float(step), C.c_uint(seed),
                            C.byref(sc), C.byref(mv))
    return pos, sc.value, mv.value


def ref_smooth_score(pr: SmoothProblem, prm: Params, moved=-1, pos=None) -> float:
    pos = _f32(pr.pos if pos is None else pos)
    return ref().ref_smooth_score(pr.n, _p(pos), _p(_f64(pr.dist_to_next)),
                                  C.byref(prm.c()), int(moved))


def distance_heatmap(contact, diag: int, scale: float, power: float, stretching: float):
    """orc_distance_heatmap: (n x n distance map, avg, clamp value)."""
    c = _f32(contact)
    n = c.shape[0]
    out = np.zeros((n, n), np.float32)
    avg = C.c_float()
    mx = C.c_float()
    lib().orc_distance_heatmap(n, _p(c), int(diag), C.c_float(scale), C.c_float(power),
                               C.c_float(stretching), _p(out), C.byref(avg), C.byref(mx))
    return out, avg.value, mx.value


def ref_distance_heatmap(contact, diag: int, level: int, scale: float, power: float,
                         stretching: float):
    c = _f32(contact)
    n = c.shape[0]
    out = np.zeros((n, n), np.float32)
    ref().ref_distance_heatmap(n, _p(c), int(diag), int(level), C.c_float(scale),
                               C.c_float(power), C.c_float(stretching), _p(out))
    return out


def equidistant(gpos, pos, first_end: int, last_start: int, pos_start: int, pos_stop: int,
                res: int):
    """orc_equidistant: the interpolated points (m x 3)."""
    g = _i32(gpos)
    p = _f32(pos).reshape(-1, 3)
    m = (pos_stop - pos_start + 1) // res + 1
    out = np.zeros((max(m, 1), 3), np.float32)
    lib().orc_equidistant.restype = C.c_longlong
    k = lib().orc_equidistant(len(g), _p(g), _p(p), int(first_end), int(last_start),
                              int(pos_start), int(pos_stop), int(res), _p(out), C.c_longlong(m))
    return out[:k]


def ref_equidistant(gpos, start, end, pos, pos_start: int, pos_stop: int, res: int):
    """The reference's gpuHelper (CPU path) on one chromosome level."""
    L = C.CDLL(os.path.join(HERE, "_ref", "libpmmc_ref_hc.so"))
    g, st, en = _i32(gpos), _i32(start), _i32(end)
    p = _f32(pos).reshape(-1, 3)
    m = (pos_stop - pos_start + 1) // res + 1
    out = np.zeros((max(m, 1), 3), np.float32)
    k = L.ref_equidistant(len(g), _p(g), _p(st), _p(en), _p(p), int(pos_start), int(pos_stop),
                          int(res), _p(out), int(m))
    return out[:k]


def ref_lengths_score(n: int, pos, dist_to_next, prm: Params, moved=-1) -> float:
    return ref().ref_lengths_score(int(n), _p(_f32(pos)), _p(_f64(dist_to_next)),
                                   C.byref(prm.c()), int(moved))


# ---------------------------------------------------------------------------
# Arc marking, HCM lines, Philox
# ---------------------------------------------------------------------------
def _mark(fn, anchors, raw):
    a = _i32(anchors).reshape(-1, 2)
    r = _i32(raw).reshape(-1, 4)
    a_s, a_e = _i32(a[:, 0]), _i32(a[:, 1])
    r_s, r_e, r_sc, r_f = (_i32(r[:, k]) for k in range(4))
    cap = 2 * len(r) + 8
    out = np.zeros((cap, 7), np.int32)
    nm = C.c_int()
    cnt = fn(len(a), _p(a_s), _p(a_e), len(r), _p(r_s), _p(r_e), _p(r_sc), _p(r_f),
             _p(out), cap, C.byref(nm))
    if cnt < 0:
        raise RuntimeError("mark_arcs output capacity exceeded")
    return out[:cnt].copy()


def mark_arcs(anchors, raw):
    """anchors: (A,2) [start,end]; raw: (R,4) [start,end,score,factor] ->
    (M,7) [start end genomic_start genomic_end score eff_score factor]."""
    return _mark(lib().orc_mark_arcs, anchors, raw)


def ref_mark_arcs(anchors, raw):
    return _mark(ref().ref_mark_arcs, anchors, raw)


def hcm_cluster_line(start, end, orient, xyz, children=(), use_ref=False) -> str:
    buf = C.create_string_buffer(4096)
    ch = _i32(list(children) if len(children) else [0])
    fn = ref().ref_hcm_cluster_line if use_ref else lib().orc_hcm_cluster_line
    fn(buf, 4096, int(start), int(end), C.c_char(orient.encode()),
       C.c_float(xyz[0]), C.c_float(xyz[1]), C.c_float(xyz[2]), len(children), _p(ch))
    return buf.value.decode()


def hcm_arc_line(a7, use_ref=False) -> str:
    buf = C.create_string_buffer(256)
    a = _i32(a7)
    fn = ref().ref_hcm_arc_line if use_ref else lib().orc_hcm_arc_line
    fn(buf, 256, _p(a))
    return buf.value.decode()


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().orc_philox4x32_10(c, k, o)
    return [o[i] for i in range(4)]


# ---------------------------------------------------------------------------
# Replay of a kernel trace
# ---------------------------------------------------------------------------
class ReplayOut(C.Structure):
    _fields_ = [("before", C.c_void_p), ("after", C.c_void_p), ("orc_acc", C.c_void_p),
                ("margin", C.c_void_p), ("proposal_mismatch", C.c_int),
                ("final_energy", C.c_double), ("stop_at", C.c_int64),
                ("stop_margin", C.c_double)]


def _replay_prep(trace):
    m = len(trace)
    bead = np.ascontiguousarray(trace["bead"], dtype=np.int32)
    disp = np.ascontiguousarray(np.stack([trace["dx"], trace["dy"], trace["dz"]], 1),
                                dtype=np.float32)
    acc = np.ascontiguousarray(trace["accepted"], dtype=np.int32)
    before = np.zeros(m, np.float64)
    after = np.zeros(m, np.float64)
    oacc = np.zeros(m, np.int32)
    margin = np.zeros(m, np.float64)
    out = ReplayOut(_p(before), _p(after), _p(oacc), _p(margin), 0, 0.0, -1, 0.0)
    keep = (bead, disp, acc, before, after, oacc, margin)
    return m, bead, disp, acc, out, keep


def _replay_result(out, keep):
    return {"before": keep[3], "after": keep[4], "orc_acc": keep[5], "margin": keep[6],
            "proposal_mismatch": out.proposal_mismatch, "final_energy": out.final_energy,
            "stop_at": out.stop_at, "stop_margin": out.stop_margin}


def arcs_replay(pr: ArcsProblem, prm: Params, step: float, seed: int, chain: int, trace,
                ext: Ext | None = None):
    m, bead, disp, acc, out, keep = _replay_prep(trace)
    la, lkeep = _loops(pr)
    fx = _u8(pr.fixed)
    lib().orc_arcs_replay_ext(pr.n, _p(_f32(pr.pos)), _p(fx), _p(_f32(pr.exp_dist)), *la,
                              C.byref(prm.c()), C.byref(ext) if ext is not None else None,
                              C.c_float(step), C.c_uint64(seed), C.c_uint32(chain), m,
                              _p(bead), _p(disp), _p(acc), C.byref(out))
    return _replay_result(out, keep)


def smooth_replay(pr: SmoothProblem, prm: Params, step: float, seed: int, chain: int, trace):
    m, bead, disp, acc, out, keep = _replay_prep(trace)
    fx = _u8(pr.fixed)
    lib().orc_smooth_replay(pr.n, _p(_f32(pr.pos)), _p(fx), _p(_f64(pr.dist_to_next)),
                            C.byref(prm.c()), C.c_float(step), C.c_uint64(seed),
                            C.c_uint32(chain), m, _p(bead), _p(disp), _p(acc), C.byref(out))
    return _replay_result(out, keep)


def heatmap_replay(pr: HeatmapProblem, prm: Params, step: float, seed: int, chain: int, trace):
    m, bead, disp, acc, out, keep = _replay_prep(trace)
    fx = _u8(pr.fixed)
    b = _i32(pr.bounds)
    lib().orc_heatmap_replay(pr.n, _p(_f32(pr.pos)), _p(fx), _p(_f32(pr.heat)), int(pr.diag),
                             len(b), _p(b), C.byref(prm.c()), C.c_float(step),
                             C.c_uint64(seed), C.c_uint32(chain), m, _p(bead), _p(disp),
                             _p(acc), C.byref(out))
    return _replay_result(out, keep)


def _ref_walk(level: int, n: int, pos, prm: Params, trace, matrix=None, diag: int = 0,
              bounds=None, dtn=None, pr_loops=None):
    m, bead, disp, acc, out, keep = _replay_prep(trace)
    before, after = keep[3], keep[4]
    mat = _f32(matrix) if matrix is not None else None
    b = _i32(bounds if bounds is not None else np.zeros(0, np.int32))
    d = _f64(dtn) if dtn is not None else None
    if pr_loops is not None:
        la, lkeep = _loops(pr_loops)
    else:
        la = (0, None, None, None, None)
    ref().ref_local_walk(level, n, _p(_f32(pos)), _p(mat) if mat is not None else None,
                         int(diag), len(b), _p(b), _p(d) if d is not None else None, *la,
                         C.byref(prm.c()), m, _p(bead), _p(disp), _p(acc), _p(before),
                         _p(after))
    return {"before": before, "after": after}


def ref_arcs_walk(pr: ArcsProblem, prm: Params, trace):
    """The reference's per-proposal local arc energy along a scripted walk
    (`trace`: bead, dx, dy, dz, accepted), before and after each move."""
    return _ref_walk(0, pr.n, pr.pos, prm, trace, matrix=pr.exp_dist, pr_loops=pr)


def ref_heatmap_walk(pr: HeatmapProblem, prm: Params, trace):
    return _ref_walk(1, pr.n, pr.pos, prm, trace, matrix=pr.heat, diag=pr.diag,
                     bounds=pr.bounds)


def ref_smooth_walk(pr: SmoothProblem, prm: Params, trace):
    return _ref_walk(2, pr.n, pr.pos, prm, trace, dtn=pr.dist_to_next)


def ref_rmsd(a, b) -> float:
    """The reference's Chromosome::calcRMSD (superposed RMSD, fast_rmsd)."""
    a, b = _f32(a).reshape(-1, 3), _f32(b).reshape(-1, 3)
    return ref().ref_rmsd(len(a), _p(a), _p(b))


def ref_distance_correlation(a, b) -> float:
    """The reference's MetricsFramework::distanceCorrelation (all pairs)."""
    a, b = _f32(a).reshape(-1, 3), _f32(b).reshape(-1, 3)
    return ref().ref_distance_correlation(len(a), _p(a), _p(b))


def ref_random_vectors(seed: int, count: int, max_size: float = 1.0, in2d: bool = False):
    out = np.zeros((count, 3), np.float32)
    ref().ref_random_vectors(C.c_uint(seed), count, C.c_float(max_size), int(in2d), _p(out))
    return out


def _anchor_args(t):
    a = {k: _i32(t[k]) for k in ("active", "arc_ptr", "arc_idx", "arc_start", "arc_end",
                                 "arc_score", "long_start", "long_end", "long_score",
                                 "anc_start", "anc_end")}
    heat = None if t.get("heat") is None else _f32(t["heat"])
    ca, cs, csh, cb = (C.c_float(float(x)) for x in t["count"])
    return a, _f32(t["memo"]), heat, (ca, cs, csh, cb)


def anchor_targets(t):
    """orc_anchor_targets on a problem dict (the keys of
    pmmc_gb300.capi.anchor_targets_arrays): (dense n x n, stats dict)."""
    a, memo, heat, cnt = _anchor_args(t)
    n = len(a["active"])
    dense = np.zeros((n, n), np.float32)
    st = np.zeros(4, np.int64)
    rc = lib().orc_anchor_targets(
        n, _p(a["active"]), _p(a["arc_ptr"]), _p(a["arc_idx"]), _p(a["arc_start"]),
        _p(a["arc_end"]), _p(a["arc_score"]), len(a["long_start"]), _p(a["long_start"]),
        _p(a["long_end"]), _p(a["long_score"]), len(a["anc_start"]), _p(a["anc_start"]),
        _p(a["anc_end"]), int(t["first_cluster"]), _p(memo), *cnt, _p(heat),
        C.c_float(float(t.get("influence", 0.0))), _p(dense), _p(st))
    if rc != 0:
        raise ValueError("an arc does not touch its cluster")
    return dense, dict(zip(("applied", "out_of_range", "inactive", "collision"),
                           (int(x) for x in st)))


def ref_anchor_targets(t):
    """The reference's calcAnchorExpectedDistancesHeatmap on the same dict."""
    a, memo, heat, cnt = _anchor_args(t)
    n = len(a["active"])
    dense = np.zeros((n, n), np.float32)
    st = np.zeros(4, np.int64)
    rc = ref().ref_anchor_targets(
        n, _p(a["active"]), _p(a["arc_ptr"]), _p(a["arc_idx"]), len(a["arc_start"]),
        _p(a["arc_start"]), _p(a["arc_end"]), _p(a["arc_score"]), len(a["long_start"]),
        _p(a["long_start"]), _p(a["long_end"]), _p(a["long_score"]), len(a["anc_start"]),
        _p(a["anc_start"]), _p(a["anc_end"]), int(t["first_cluster"]), _p(memo), *cnt,
        _p(heat), C.c_float(float(t.get("influence", 0.0))), _p(dense), _p(st))
    if rc != 0:
        raise RuntimeError("reference harness failed")
    return dense, dict(zip(("applied", "out_of_range", "inactive", "collision"),
                           (int(x) for x in st)))


class StressParams(C.Structure):
    _fields_ = [(k, C.c_float) for k in ("count_a", "count_scale", "count_shift", "count_base",
                                          "glen_base", "glen_scale", "glen_power", "k_stretch",
                                          "k_squeeze", "k_angular")]


class StressOut(C.Structure):
    _fields_ = [("iterations", C.c_int), ("stop", C.c_int), ("lr", C.c_float),
                ("total", C.c_double), ("backbone", C.c_double), ("hic", C.c_double),
                ("angular", C.c_double), ("n_pairs", C.c_longlong)]


def _stress_args(t):
    a = {k: _i32(t[k]) for k in ("active", "genomic_pos", "arc_start", "arc_end", "arc_score",
                                 "long_start", "long_end", "long_score", "anc_start",
                                 "anc_end")}
    prm = StressParams(*(float(x) for x in t["count"]), *(float(x) for x in t["glen"]),
                       *(float(x) for x in t["springs"]))
    return a, _f32(t["pos"]).reshape(-1, 3), prm


def stress_refine(t, max_iter: int, lr: float):
    """orc_stress_refine on a problem dict (keys of
    pmmc_gb300.capi.stress_arrays): (order, positions n x 3, out dict)."""
    a, pos, prm = _stress_args(t)
    n = len(a["active"])
    order = np.zeros(n, np.int32)
    out_pos = np.zeros((n, 3), np.float32)
    o = StressOut()
    lib().orc_stress_refine(n, _p(a["active"]), _p(a["genomic_pos"]), _p(pos),
                            len(a["arc_start"]), _p(a["arc_start"]), _p(a["arc_end"]),
                            _p(a["arc_score"]), len(a["long_start"]), _p(a["long_start"]),
                            _p(a["long_end"]), _p(a["long_score"]), len(a["anc_start"]),
                            _p(a["anc_start"]), _p(a["anc_end"]), int(t["first_cluster"]),
                            C.byref(prm), int(max_iter), C.c_float(lr), _p(order), _p(out_pos),
                            C.byref(o))
    return order, out_pos, {k: getattr(o, k) for k, _ in StressOut._fields_}


def ref_stress_refine(t, max_iter: int, lr: float):
    """The reference's stressRefineAnchors on the same dict: (order, positions)."""
    a, pos, prm = _stress_args(t)
    n = len(a["active"])
    order = np.zeros(n, np.int32)
    out_pos = np.zeros((n, 3), np.float32)
    ref().ref_stress_refine(n, _p(a["active"]), _p(a["genomic_pos"]), _p(pos),
                            len(a["arc_start"]), _p(a["arc_start"]), _p(a["arc_end"]),
                            _p(a["arc_score"]), len(a["long_start"]), _p(a["long_start"]),
                            _p(a["long_end"]), _p(a["long_score"]), len(a["anc_start"]),
                            _p(a["anc_start"]), _p(a["anc_end"]), int(t["first_cluster"]),
                            C.byref(prm), int(max_iter), C.c_float(lr), _p(order), _p(out_pos))
    return order, out_pos
