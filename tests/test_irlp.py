"""IrLP full recompute: the snapshot the reference's driver builds for it
(src/main.cu:127-176) and the GPU recompute (dlp_irlp, src/validation.cu:145-208)
against the oracle's restatement (oracle/irlp_oracle.cpp), after several
batches of a replay, not only the last."""
from __future__ import annotations

import numpy as np
import pytest

import labelpropcuda_gb300 as dlp

CFG = (5000, 5, 10, 42)


def driver_snapshot_loop(p, last):
    """src/main.cu:127-176 transcribed line by line (plain loops, small n)."""
    n = p.num_nodes
    status, gt, lab, bm = [1] * n, [-1] * n, [0.5] * n, [-1] * n
    for b in range(last + 1):
        bt = p.batches[b]
        for v in bt.inserted:
            status[v] = 0
        for v in bt.deleted:
            status[v] = 1
        for v, x in zip(bt.gt_ids, bt.gt_labels):
            status[v] = 2
            gt[v] = 0 if x < 0.5 else 1
            lab[v] = float(x)
        for v in bt.inserted:
            bm[v] = b
    rp, col, val = [0], [], []
    for u in range(n):
        if status[u] != 1 and bm[u] >= 0:
            for e in range(p.row_ptr[u], p.row_ptr[u + 1]):
                v = int(p.col_ind[e])
                if v >= 0 and status[v] != 1 and bm[v] >= 0:
                    col.append(v)
                    val.append(p.values[e])
        rp.append(len(col))
    return rp, col, np.array(val, np.float32), status, gt, np.array(lab, np.float32)


def test_snapshot_is_the_drivers(native):
    """The vectorised snapshot equals a line-by-line transcription of the
    driver's loops after every batch."""
    p = dlp.Problem(2000, 5, 6, 3, cache_dir="")
    for b in range(len(p.batches)):
        rp, col, val, status, gt, lab = driver_snapshot_loop(p, b)
        snap = dlp.irlp_snapshot(p, b)
        assert snap.row_ptr.tolist() == rp and snap.col_ind.tolist() == col, b
        assert snap.values.tobytes() == val.tobytes()
        assert snap.status.tolist() == status and snap.gt_class.tolist() == gt
        assert snap.labels.tobytes() == lab.tobytes()


def test_snapshot_against_oracle_rebuild(native, oracle):
    """The oracle's active graph (src/dynLP.cu:111-166, updateHostCSR) after the
    same batch differs from main.cu's IrLP snapshot only through vertices
    inserted and deleted in one batch: updateHostCSR marks deletions before
    insertions (such a vertex stays active), main.cu's snapshot loop marks
    them after (it is deleted). With those vertices' rows and entries taken
    out of both, the graphs are equal."""
    p = dlp.Problem(*CFG, cache_dir="")
    orc = oracle.OracleRun.from_problem(p, record=True, threads=2)
    both = np.zeros(p.num_nodes, bool)
    seen = np.zeros(p.num_nodes, bool)
    for b, bt in enumerate(p.batches):
        orc.apply(b, bt)
        both[np.intersect1d(bt.inserted, bt.deleted)] = True
        seen[bt.inserted] = True
        snap = dlp.irlp_snapshot(p, b)
        orp, ocol = orc.artefact(oracle.ART_ROW_PTR), orc.artefact(oracle.ART_COL_IND)
        oval = orc.artefact(oracle.ART_VALUES)

        def strip(rp, col, val):
            rows = np.repeat(np.arange(p.num_nodes), np.diff(rp))
            keep = ~both[rows] & ~both[col]
            return rows[keep], col[keep], val[keep]
        mine, theirs = strip(snap.row_ptr, snap.col_ind, snap.values), strip(orp, ocol, oval)
        for x, y in zip(mine, theirs):
            np.testing.assert_array_equal(x, y, err_msg=f"batch {b}")
        ok = seen & ~both
        assert np.array_equal(snap.status[ok], orc.artefact(oracle.ART_STATUS)[ok])
    assert both.any()  # the generator does delete vertices in the batch that inserts them


def test_snapshot_of_an_empty_prefix(native):
    p = dlp.Problem(1000, 3, 4, 5, cache_dir="")
    snap = dlp.irlp_snapshot(p, -1)  # before the first batch: nothing inserted
    assert snap.row_ptr.shape == (1001,) and snap.row_ptr[-1] == 0 and snap.col_ind.size == 0
    assert np.all(snap.status == 1)


@pytest.mark.gpu
@pytest.mark.parametrize("batch", [1, 4, 9])
def test_gpu_irlp_matches_oracle_on_driver_snapshots(gpu, oracle, batch):
    p = dlp.Problem(*CFG, cache_dir="")
    snap = dlp.irlp_snapshot(p, batch)
    want, it_want, _ = oracle.irlp(p.num_nodes, snap.row_ptr, snap.col_ind, snap.values, snap.status, snap.gt_class,
                                   snap.labels, threads=4)
    got, it = dlp.irlp(snap)
    assert it == it_want
    assert got.tobytes() == want.tobytes()
