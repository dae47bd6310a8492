"""Element-wise comparison of one batch of the CUDA path with the oracle
(shared by the parity tests; not a test module itself)."""
from __future__ import annotations

import numpy as np

from labelpropcuda_gb300 import _native as N

EXACT_STATS = ["iterations", "num_components", "num_sub_edges", "hook_edges", "seed_frontier", "seed_marks",
               "affected_edges", "frontier_visits", "correct", "total", "init_branch", "hook_truncated"]


def pairs(a: np.ndarray) -> np.ndarray:
    p = a.reshape(-1, 2)
    return p[np.lexsort((p[:, 1], p[:, 0]))]


def check_batch(b, got: dict, want: dict, sess, orc, oracle, labels=None) -> None:
    """Bit-exact: every statistic, the affected seed set, the first frontier,
    the kept edges, the component partition (roots = minimum vertex ids), the
    initial labels, the frontier size of every pass, the live row lengths and
    the labels after the batch. `sess` has to record artefacts (record=True)."""
    assert got["status"] == N.DLP_OK
    for k in EXACT_STATS:
        assert got[k] == want[k], (b, k, got[k], want[k])
    assert np.float32(got["accuracy"]) == np.float32(want["accuracy"])
    np.testing.assert_array_equal(np.sort(sess.artefact(N.ART_SEED_MARKS)), orc.artefact(oracle.ART_SEED_MARKS))
    np.testing.assert_array_equal(np.sort(sess.artefact(N.ART_FRONTIER0)), orc.artefact(oracle.ART_FRONTIER0))
    np.testing.assert_array_equal(pairs(sess.artefact(N.ART_SUB_EDGES)), pairs(orc.artefact(oracle.ART_SUB_EDGES)))
    if want["init_branch"] == 1:
        np.testing.assert_array_equal(sess.artefact(N.ART_COMP_ROOT), orc.artefact(oracle.ART_COMP_ROOT))
    assert sess.artefact(N.ART_INIT_LABELS).tobytes() == orc.artefact(oracle.ART_INIT_LABELS).tobytes()
    np.testing.assert_array_equal(sess.artefact(N.ART_FRONTIER_SIZES), orc.artefact(oracle.ART_FRONTIER_SIZES))
    np.testing.assert_array_equal(sess.artefact(N.ART_ROW_LENGTHS), np.diff(orc.artefact(oracle.ART_ROW_PTR)))
    gl = sess.labels() if labels is None else labels
    wl = orc.labels()
    assert gl.tobytes() == wl.tobytes(), (b, int(np.sum(gl != wl)), float(np.max(np.abs(gl - wl))))
