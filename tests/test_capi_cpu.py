"""Host-side checks of the C ABI that need no GPU: the library loads, exports
every symbol the header declares, converts the reference's dense layout, and
fails loudly (no CPU fallback) when no device is present."""
import os
import re

import numpy as np
import pytest

from pmmc_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_header_symbols_exported(built_lib):
    h = open(os.path.join(ROOT, "include", "pmmc_gb300.h")).read()
    declared = set(re.findall(r"\b(pmmc_[a-z0-9_]+)\s*\(", h))
    assert declared == set(capi.HEADER_SYMBOLS)
    for name in declared:
        assert hasattr(built_lib, name), name


def test_default_params_match_reference_settings(built_lib):
    p = capi.default_params(capi.LEVEL_ARCS)
    # Settings::init, src/include/Settings.hpp:479-505
    assert (p.max_temp, p.jump_scale, p.jump_coef, p.min_successes, p.milestone_steps) == \
        (20.0, 50.0, 20.0, 5, 10000)
    assert abs(p.dt_temp - 0.99995) < 1e-7 and abs(p.improvement - 0.995) < 1e-7
    assert (p.k_stretch, p.k_squeeze, p.milestone_fails) == (1.0, 1.0, 3)
    s = capi.default_params(capi.LEVEL_SMOOTH)
    assert abs(s.k_stretch - 0.1) < 1e-7 and abs(s.k_angle - 0.1) < 1e-7


def test_dense_to_csr_reads_columns(built_lib):
    d = np.full((4, 4), -1.0, np.float32)
    np.fill_diagonal(d, 0.0)
    d[0, 2], d[2, 0] = 1.5, 2.5     # asymmetric on purpose: row i gets column i
    d[1, 3] = d[3, 1] = 0.0         # listed but inert
    rp, col, tgt = capi.dense_to_csr(d)
    assert list(rp) == [0, 1, 2, 3, 4]
    assert list(col) == [2, 3, 0, 1]
    np.testing.assert_array_equal(tgt, np.array([2.5, 0.0, 1.5, 0.0], np.float32))


def test_rows_to_csr_equals_dense_to_csr(built_lib):
    """The reference's row pointers (Heatmap::v) give the CSR of its dense
    matrix, with no n x n copy; a short capacity reports the count."""
    import ctypes as C
    rng = np.random.default_rng(4)
    n = 300
    d = np.full((n, n), -1.0, np.float32)
    m = rng.random((n, n)) < 0.02
    d[m] = rng.uniform(0.0, 3.0, m.sum()).astype(np.float32)
    d[rng.random((n, n)) < 0.003] = 0.0
    np.fill_diagonal(d, 0.0)
    rp, col, tgt = capi.dense_to_csr(d)
    rows = (C.POINTER(C.c_float) * n)(*[d[j].ctypes.data_as(C.POINTER(C.c_float))
                                        for j in range(n)])
    rp2 = np.zeros(n + 1, np.int32)
    nnz = C.c_int64()
    short = np.zeros(4, np.int32), np.zeros(4, np.float32)
    st = capi.lib().pmmc_arcs_rows_to_csr(n, rows, rp2.ctypes.data_as(C.c_void_p),
                                          short[0].ctypes.data_as(C.c_void_p),
                                          short[1].ctypes.data_as(C.c_void_p), C.c_int64(4),
                                          C.byref(nnz))
    assert st == capi.PMMC_ERR_INVALID and nnz.value == len(col)
    col2 = np.zeros(nnz.value, np.int32)
    tgt2 = np.zeros(nnz.value, np.float32)
    st = capi.lib().pmmc_arcs_rows_to_csr(n, rows, rp2.ctypes.data_as(C.c_void_p),
                                          col2.ctypes.data_as(C.c_void_p),
                                          tgt2.ctypes.data_as(C.c_void_p), C.c_int64(nnz.value),
                                          C.byref(nnz))
    assert st == capi.PMMC_OK
    np.testing.assert_array_equal(rp2, rp)
    np.testing.assert_array_equal(col2, col)
    np.testing.assert_array_equal(tgt2, tgt)
    # row i lists column i of the matrix, ascending
    for i in (0, 7, 299):
        js = [j for j in range(n) if j != i and d[j, i] >= 0]
        assert list(col[rp[i]:rp[i + 1]]) == js


def test_no_device_is_an_error(built_lib):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a device is present")
    except ImportError:
        pass
    with pytest.raises(capi.PmmcError) as e:
        capi.Context(0)
    assert e.value.status == capi.PMMC_ERR_NO_DEVICE


def test_serve_trace_shape():
    """The serving trace: sizes log-uniform in [64, 8192], Poisson arrivals
    at about 200 requests/s, reproducible from its seed."""
    from pmmc_gb300 import workloads as W
    s1, a1 = W.serve_trace(5000)
    s2, a2 = W.serve_trace(5000)
    np.testing.assert_array_equal(s1, s2)
    np.testing.assert_array_equal(a1, a2)
    assert s1.min() >= 64 and s1.max() <= 8192
    assert abs(np.log(s1).mean() - 0.5 * (np.log(64) + np.log(8192))) < 0.1
    rate = len(a1) / a1[-1]
    assert 180 < rate < 220
    assert np.all(np.diff(a1) >= 0) and a1[0] == 0.0


def test_hcm_writer_matches_reference_lines(tmp_path):
    """pmmc_hcm_write: cluster and arc lines equal the reference's own
    Cluster::toFile / InteractionArc::toFile output (golden lines)."""
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "hcm.npz"))["lines"]
    path = str(tmp_path / "model.hcm")
    capi.hcm_write(path, [10, 0], [20, 0], ["N", "L"],
                   np.array([[1.5, -2.25, 3.125], [1e-7, 123456.789, -0.5]], np.float32),
                   [[4, 5], []], ["CTCF"],
                   [("chr1", 0, [[1, 2, 300, 400, 5, 6, -1], [7, 9, -1, -1, 0, 12, 2]])])
    lines = open(path).read().splitlines(keepends=True)
    assert lines[0] == "2 1 -1 1\n"
    assert lines[1] == "CTCF \n"
    assert lines[2] == str(g[0]) and lines[3] == str(g[1])
    assert lines[4] == "chr1 0 2\n"
    assert lines[5] == str(g[2]) and lines[6] == str(g[3])


def test_ctypes_structs_match_header_layouts(tmp_path):
    """Every struct the binding mirrors has the header's size and field
    offsets (a C program built against include/pmmc_gb300.h prints them)."""
    import ctypes
    import shutil
    import subprocess
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    pairs = {"AnnealParams": "pmmc_anneal_params", "Result": "pmmc_result",
             "ArcsProblem": "pmmc_arcs_problem", "HeatmapProblem": "pmmc_heatmap_problem",
             "SmoothProblem": "pmmc_smooth_problem", "BatchOpts": "pmmc_batch_opts",
             "AnchorTargetsProblem": "pmmc_anchor_targets_problem",
             "AnchorTargetsStats": "pmmc_anchor_targets_stats",
             "StressProblem": "pmmc_stress_problem", "StressResult": "pmmc_stress_result",
             "ServerOpts": "pmmc_server_opts", "ServerStats": "pmmc_server_stats"}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "pmmc_gb300.h"',
             "int main(void) {"]
    want = []
    for py, c in pairs.items():
        cls = getattr(capi, py)
        lines.append(f'  printf("%zu\\n", sizeof({c}));')
        want.append(ctypes.sizeof(cls))
        for name, _ in cls._fields_:
            lines.append(f'  printf("%zu\\n", offsetof({c}, {name}));')
            want.append(getattr(cls, name).offset)
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run(["gcc", "-std=c11", f"-I{root}/include", str(src), "-o",
                        str(tmp_path / "layout")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    got = [int(x) for x in subprocess.run([str(tmp_path / "layout")], capture_output=True,
                                          text=True).stdout.split()]
    assert got == want


def test_kernel_choice_setters_need_a_context(built_lib):
    """pmmc_smooth_set_window and pmmc_heatmap_set_cluster validate their
    arguments on the host; a null context is refused without device work."""
    assert built_lib.pmmc_smooth_set_window(None, 8, 32, 20) == capi.PMMC_ERR_INVALID
    assert built_lib.pmmc_heatmap_set_cluster(None, 8) == capi.PMMC_ERR_INVALID


def test_smooth_packed_regions_concatenate_the_segments():
    """The packed genome-smoothing arrays (one set of arrays, regions back to
    back) hold exactly the list form's regions, in order."""
    from pmmc_gb300 import workloads as W
    segs = W.smooth_segments()
    off, pos, dtn, fixed = W.smooth_packed()
    assert len(off) == len(segs) + 1 and off[0] == 0 and off[-1] == len(pos) == len(dtn)
    for u in range(0, len(segs), 997):
        p, d, f = segs[u]
        np.testing.assert_array_equal(pos[off[u]:off[u + 1]], np.asarray(p, np.float32))
        np.testing.assert_array_equal(dtn[off[u]:off[u + 1]], np.asarray(d, np.float32))
        np.testing.assert_array_equal(fixed[off[u]:off[u + 1]], np.asarray(f, np.uint8))
