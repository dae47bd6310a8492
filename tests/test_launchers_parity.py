"""GPU parity of the five reference-layout step launchers.

The test replays the reference's per-batch orchestration (src/dynLP.cu:284-558)
in Python: host CSR rebuild (taken from the oracle, whose rebuild is pinned to
the reference's updateHostCSR by test_golden_inputs), full upload, then
dlp_mark_deletions, dlp_build_sparsified_subgraph, dlp_connected_components,
dlp_label_initialization and dlp_iterative_propagation on device arrays in the
reference's layout, and compares every batch with the oracle bit for bit.
The one deliberate difference from the reference: the components step is given
min(numSubEdges, numNewEdges) raw edges, the pinned convention for the
reference's read past the end of the edge list.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import labelpropcuda_gb300 as dlp
from labelpropcuda_gb300 import DeviceArray
from labelpropcuda_gb300 import _native as N

ACTIVE, DELETED, GT = 0, 1, 2


def _i(x):
    return ctypes.c_void_p(x.addr)


def replay(oracle, p, nb=None):
    L = N.lib()
    n = p.num_nodes
    orc = oracle.OracleRun.from_problem(p, record=True, threads=4)
    tau = np.float32(orc.tau)
    status = np.full(n, DELETED, np.int32)
    gt = np.full(n, -1, np.int32)
    labels = np.full(n, 0.5, np.float32)
    m_full = p.num_edges
    i32 = lambda c: DeviceArray(dtype=np.int32, count=max(c, 1))
    f32 = lambda c: DeviceArray(dtype=np.float32, count=max(c, 1))
    d_row, d_col, d_val = i32(n + 1), i32(m_full), f32(m_full)
    d_lab, d_buf = f32(n), f32(n)
    d_st, d_gt, d_aff, d_comp, d_new = i32(n), i32(n), i32(n), i32(n), i32(n)
    L.dlp_memset(d_comp.ptr, 0xFF, 4 * n)
    batches = p.batches if nb is None else p.batches[:nb]
    for b, bt in enumerate(batches):
        want = orc.apply(b, bt)
        gt[bt.gt_ids] = np.where(bt.gt_labels < 0.5, 0, 1)
        labels[bt.gt_ids] = bt.gt_labels
        status[bt.deleted] = DELETED
        status[bt.inserted] = ACTIVE
        status[bt.gt_ids] = GT
        rp = orc.artefact(oracle.ART_ROW_PTR)
        ci = orc.artefact(oracle.ART_COL_IND)
        va = orc.artefact(oracle.ART_VALUES)
        d_row.set(rp)
        if ci.size:
            d_col.set(ci)
            d_val.set(va)
        d_st.set(status)
        d_gt.set(gt)
        d_lab.set(labels)
        L.dlp_memset(d_new.ptr, 0, 4 * n)
        L.dlp_memset(d_aff.ptr, 0, 4 * n)
        if bt.inserted.size:
            flags = np.zeros(n, np.int32)
            flags[bt.inserted] = 1
            d_new.set(flags)
        if bt.deleted.size:
            dd = DeviceArray(bt.deleted)
            N.check(L.dlp_mark_deletions(d_row.ptr, d_col.ptr, d_st.ptr, d_aff.ptr, dd.ptr, bt.deleted.size, n, None))
        I, E = bt.inserted.size, bt.edge_src.size
        num_comp = 0
        if I and E:
            es, ed, ew, ins = DeviceArray(bt.edge_src), DeviceArray(bt.edge_dst), DeviceArray(bt.edge_weight), \
                DeviceArray(bt.inserted)
            sub_col, sub_val, sub_row = i32(2 * E), f32(2 * E), i32(I + 1)
            nsn, nse = ctypes.c_int(0), ctypes.c_int(0)
            N.check(L.dlp_build_sparsified_subgraph(d_row.ptr, d_col.ptr, d_val.ptr, d_aff.ptr, d_st.ptr, es.ptr,
                                                    ed.ptr, ew.ptr, E, ins.ptr, I, d_new.ptr, float(tau), sub_row.ptr,
                                                    sub_col.ptr, sub_val.ptr, ctypes.byref(nsn), ctypes.byref(nse),
                                                    None))
            assert nse.value == want["num_sub_edges"], (b, nse.value, want["num_sub_edges"])
            # kept edges, both directions, raw order
            kept = orc.artefact(oracle.ART_SUB_EDGES).reshape(-1, 2)
            got_dst = sub_col.get()[: nse.value]
            np.testing.assert_array_equal(got_dst, kept[:, 1])
            if nse.value > 0:
                nc = ctypes.c_int(0)
                N.check(L.dlp_connected_components(es.ptr, ed.ptr, min(nse.value, E), ins.ptr, I, d_comp.ptr,
                                                   ctypes.byref(nc), n, None))
                num_comp = nc.value
                comp = d_comp.get()
                np.testing.assert_array_equal(comp[bt.inserted], orc.artefact(oracle.ART_COMP_ID), err_msg=str(b))
            else:
                num_comp = I
                comp = np.full(n, -1, np.int32)
                comp[bt.inserted] = np.arange(I, dtype=np.int32)
                d_comp.set(comp)
            assert num_comp == want["num_components"], (b, num_comp, want["num_components"])
            N.check(L.dlp_label_initialization(d_row.ptr, d_col.ptr, d_val.ptr, d_lab.ptr, d_st.ptr, d_comp.ptr,
                                               num_comp, ins.ptr, I, d_gt.ptr, n, None))
            init = d_lab.get()[bt.inserted]
            assert init.tobytes() == orc.artefact(oracle.ART_INIT_LABELS).tobytes(), b
        elif I:
            cur = d_lab.get()
            for v in bt.inserted:
                cur[v] = 0.5 if gt[v] < 0 else cur[v]
            batch_gt = dict(zip(bt.gt_ids.tolist(), bt.gt_labels.tolist()))
            for v in bt.inserted:
                if gt[v] >= 0:
                    cur[v] = batch_gt.get(int(v), 0.5)
            d_lab.set(cur)
        it = ctypes.c_int(0)
        N.check(L.dlp_iterative_propagation(d_row.ptr, d_col.ptr, d_val.ptr, d_lab.ptr, d_buf.ptr, d_st.ptr,
                                            d_gt.ptr, d_aff.ptr, n, ctypes.c_float(1e-4), 100000, ctypes.byref(it),
                                            None))
        assert it.value == want["iterations"], (b, it.value, want["iterations"])
        labels = d_lab.get()
        assert labels.tobytes() == orc.labels().tobytes(), b


@pytest.mark.gpu
@pytest.mark.parametrize("cfg", [(1000, 3, 5, 7), (5000, 5, 10, 42), (2000, 7, 6, 3)],
                         ids=lambda c: "n%d_d%d_b%d_s%d" % c)
def test_launchers_replay_matches_oracle(gpu, oracle, cfg):
    replay(oracle, dlp.Problem(*cfg))


@pytest.mark.gpu
def test_irlp_matches_oracle(gpu, oracle):
    L = N.lib()
    p = dlp.Problem(5000, 5, 10, 42)
    orc = oracle.OracleRun.from_problem(p, record=True, threads=4)
    for b, bt in enumerate(p.batches):
        orc.apply(b, bt)
    rp, ci, va = orc.artefact(oracle.ART_ROW_PTR), orc.artefact(oracle.ART_COL_IND), orc.artefact(oracle.ART_VALUES)
    status = orc.artefact(oracle.ART_STATUS).astype(np.int32)
    gt = np.full(p.num_nodes, -1, np.int32)
    lab0 = np.full(p.num_nodes, 0.5, np.float32)
    for bt in p.batches:
        gt[bt.gt_ids] = np.where(bt.gt_labels < 0.5, 0, 1)
        lab0[bt.gt_ids] = bt.gt_labels
    want, it_want, _ = oracle.irlp(p.num_nodes, rp, ci, va, status, gt, lab0, threads=4)
    d = [DeviceArray(x) for x in (rp, ci, va, lab0, status, gt)]
    it = ctypes.c_int(0)
    N.check(L.dlp_irlp(d[0].ptr, d[1].ptr, d[2].ptr, d[3].ptr, d[4].ptr, d[5].ptr, p.num_nodes,
                       ctypes.c_float(1e-4), 100000, ctypes.byref(it), None))
    assert it.value == it_want
    assert d[3].get().tobytes() == want.tobytes()
