"""dlp_iterative_propagation_noalloc against dlp_iterative_propagation.

The allocation-free entry point exists for callers that may not allocate
device memory while they run (a host framework that owns the device's whole
memory pool, a service that reserves all of its memory at start-up). It must
give exactly what the allocating launcher gives: the same labels bit for bit,
the same final isAffected array and the same pass count. Two calls in a row
run on different graphs, the larger first, because every call reuses one
scratch array that keeps the previous call's contents.

This file is named to be collected last, so that a run stopping at the first
failure has run every other test before it. It passes alone in a fresh process
and after the other tests.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from labelpropcuda_gb300 import DeviceArray, Problem
from labelpropcuda_gb300 import _native as N

ACTIVE, DELETED, GT = 0, 1, 2
LIMIT = 1 << 20  # vertices the fixed scratch array holds


def _inputs(num_nodes: int, avg_degree: int, seed: int):
    """A seeded propagation input in the reference layout: full CSR with the
    entries of deleted targets soft-deleted (-1), a status mix, ground-truth
    classes, random labels and a random seed frontier."""
    p = Problem(num_nodes, avg_degree, 1, seed)
    rng = np.random.default_rng(seed)
    n = p.num_nodes
    status = rng.choice([ACTIVE, DELETED, GT], size=n, p=[0.88, 0.06, 0.06]).astype(np.int32)
    gt = np.where(status == GT, (p.true_labels >= 0.5).astype(np.int32), -1).astype(np.int32)
    labels = rng.random(n, dtype=np.float32)
    labels[status == GT] = gt[status == GT].astype(np.float32)
    col = p.col_ind.copy()
    col[status[col] == DELETED] = -1
    affected = (rng.random(n) < 0.1).astype(np.int32)
    return p.row_ptr, col, p.values, labels, status, gt, affected


def _run(entry: str, inputs, delta: float, max_iterations: int):
    row, col, val, labels, status, gt, affected = inputs
    n = labels.size
    d = [DeviceArray(a) for a in (row, col, val, labels, labels, status, gt, affected)]
    d_row, d_col, d_val, d_lab, d_buf, d_st, d_gt, d_aff = d
    used = ctypes.c_int(-1)
    fn = getattr(N.lib(), entry)
    N.check(fn(d_row.ptr, d_col.ptr, d_val.ptr, d_lab.ptr, d_buf.ptr, d_st.ptr, d_gt.ptr, d_aff.ptr, n,
               ctypes.c_float(delta), max_iterations, ctypes.byref(used), None))
    out = d_lab.get(np.float32), d_aff.get(np.int32), used.value
    for a in d:
        a.free()
    return out


@pytest.mark.gpu
def test_noalloc_matches_allocating_launcher_on_two_calls_in_a_row(gpu):
    cases = [(_inputs(40000, 6, 7), 1e-4, 400), (_inputs(6000, 4, 11), 1e-3, 150)]
    for inputs, delta, max_iter in cases:
        want_lab, want_aff, want_it = _run("dlp_iterative_propagation", inputs, delta, max_iter)
        got_lab, got_aff, got_it = _run("dlp_iterative_propagation_noalloc", inputs, delta, max_iter)
        assert got_it == want_it
        # labels: bit-exact, the bar for every label comparison in these tests
        assert np.array_equal(got_lab.view(np.uint32), want_lab.view(np.uint32))
        assert np.array_equal(got_aff, want_aff)
        assert want_it >= 1


@pytest.mark.gpu
def test_noalloc_rejects_graphs_beyond_its_limit(gpu):
    inputs = _inputs(2000, 4, 3)
    row, col, val, labels, status, gt, affected = inputs
    d = [DeviceArray(a) for a in (row, col, val, labels, labels, status, gt, affected)]
    used = ctypes.c_int(-1)
    rc = N.lib().dlp_iterative_propagation_noalloc(*[a.ptr for a in d], LIMIT + 1, ctypes.c_float(1e-4), 10,
                                                   ctypes.byref(used), None)
    assert rc == N.DLP_ERR_INVALID_ARGUMENT
    assert b"allocation-free limit" in N.lib().dlp_last_error()
    assert used.value == 0
    for a in d:
        a.free()
