"""Size-independent properties at the largest configuration: 20,000,000
vertices, average degree 7, the first batches of the 100-batch sequence
(seed 42).

The oracle replays only the first batches of this size within a test
(test_largest_configuration_first_batches_match_oracle, below); beyond them
correctness rests on properties that hold at any size and fail on any race or
indexing slip:
1. The arithmetic must not depend on the launch shape. A one-graph engine
   with 8-lane row groups and an engine with 4-lane groups must give
   bit-identical statistics and labels. The second engine also shares every
   launch with another graph, so flattened work lists and per-graph offsets
   are exercised too.
2. Ground-truth vertices hold exactly their given labels.
3. Every label is in [0, 1].
4. The accuracy counters agree with themselves.
At the sizes the oracle can run, the same engine is checked against it bit
for bit (test_session_parity, test_engine_parity).
"""
from __future__ import annotations

import numpy as np
import pytest

import labelpropcuda_gb300 as dlp

EXACT = ["iterations", "num_components", "num_sub_edges", "hook_edges", "seed_frontier",
         "seed_marks", "affected_edges", "frontier_visits", "correct", "total", "init_branch", "hook_truncated",
         "dirty_rows", "dirty_entries"]
BATCHES = 3


@pytest.mark.gpu
def test_largest_configuration_properties(gpu):
    p = dlp.Problem(20_000_000, 7, 100, 42)
    small = dlp.Problem(3000, 5, BATCHES, 11)
    a = dlp.Engine(1, narrow_lanes=8)
    ga = a.add_problem(p)
    b = dlp.Engine(2, narrow_lanes=4)
    gs = b.add_problem(small)
    gb = b.add_problem(p)
    for k in range(BATCHES):
        bt = p.batches[k]
        sa = a.step([(ga, k, bt)])[0]
        sb = b.step([(gs, k, small.batches[k]), (gb, k, bt)])[1]
        for key in EXACT:
            assert sa[key] == sb[key], (k, key, sa[key], sb[key])
        assert 0 <= sa["correct"] <= sa["total"]
        if sa["total"]:
            assert abs(sa["accuracy"] - sa["correct"] / sa["total"]) < 1e-6
    la, lb = a.labels(ga), b.labels(gb)
    assert la.tobytes() == lb.tobytes()
    assert np.all((la >= 0.0) & (la <= 1.0))
    for k in range(BATCHES):
        bt = p.batches[k]
        assert np.array_equal(la[bt.gt_ids], bt.gt_labels)


ORACLE_BATCHES = 6


@pytest.mark.gpu
def test_largest_configuration_first_batches_match_oracle(gpu, oracle):
    """The first batches of the 20,000,000-vertex problem against the oracle
    (all host threads), element by element, in three launch shapes: the
    default (small frontiers on one block or a 16-block sub-grid) and every
    pass on the full grid with 4-lane row groups or a lane per short row."""
    from parity_checks import check_batch
    p = dlp.Problem(20_000_000, 7, 100, 42)
    orc = oracle.OracleRun.from_problem(p, record=True, threads=0)
    runs = [dlp.Session.from_problem(p, record=True),
            dlp.Session.from_problem(p, record=True, small_frontier_solo=0, narrow_lanes=4),
            dlp.Session.from_problem(p, record=True, small_frontier_solo=0, narrow_lanes=1)]
    for b in range(ORACLE_BATCHES):
        want = orc.apply(b, p.batches[b])
        for sess in runs:
            got = sess.apply(b, p.batches[b])
            check_batch(b, got, want, sess, orc, oracle)
        assert want["affected_edges"] > 0 or b == 0
