"""GPU parity of the resident session against the CPU oracle, batch by batch.

Bit-exact: every per-batch count (frontier sizes, passes, affected edges,
components, kept edges, accuracy counters), the affected seed set, the first
frontier, the kept (sparsified) edge set, the component partition
(canonicalised to the minimum vertex id) and the fp32 labels.
"""
from __future__ import annotations

import numpy as np
import pytest

import labelpropcuda_gb300 as dlp
from labelpropcuda_gb300 import _native as N

EXACT_STATS = ["iterations", "num_components", "num_sub_edges", "hook_edges", "seed_frontier", "seed_marks",
               "affected_edges", "frontier_visits", "correct", "total", "init_branch", "hook_truncated"]

CONFIGS = [
    # (n, degree, batches, seed, semantics, lanes)
    (1000, 3, 5, 7, dlp.SEMANTICS_REF, 8),
    (5000, 5, 10, 42, dlp.SEMANTICS_REF, 8),
    (2000, 7, 6, 3, dlp.SEMANTICS_REF, 4),
    (3000, 4, 3, 11, dlp.SEMANTICS_REF, 16),
    (5000, 5, 10, 42, dlp.SEMANTICS_REF, 32),
    (5000, 5, 10, 42, dlp.SEMANTICS_REF, 1),
    (2000, 7, 6, 3, dlp.SEMANTICS_SPEC, 1),
    (5000, 5, 10, 42, dlp.SEMANTICS_SPEC, 8),
    (2000, 7, 6, 3, dlp.SEMANTICS_SPEC, 4),
    (50000, 5, 10, 42, dlp.SEMANTICS_REF, 8),
]


def pairs(a: np.ndarray) -> np.ndarray:
    p = a.reshape(-1, 2)
    return p[np.lexsort((p[:, 1], p[:, 0]))]


@pytest.mark.gpu
@pytest.mark.parametrize("cfg", CONFIGS, ids=lambda c: "n%d_d%d_b%d_s%d_sem%d_g%d" % c)
def test_session_matches_oracle(gpu, oracle, cfg):
    n, deg, nb, seed, sem, lanes = cfg
    p = dlp.Problem(n, deg, nb, seed)
    sess = dlp.Session.from_problem(p, semantics=sem, record=True, narrow_lanes=lanes)
    orc = oracle.OracleRun.from_problem(p, semantics=sem, record=True, threads=4)
    assert np.float32(sess.tau) == np.float32(orc.tau)
    for b, batch in enumerate(p.batches):
        got = sess.apply(b, batch)
        want = orc.apply(b, batch)
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
        rp = orc.artefact(oracle.ART_ROW_PTR)
        np.testing.assert_array_equal(sess.artefact(N.ART_ROW_LENGTHS), np.diff(rp))
        gl, wl = sess.labels(), orc.labels()
        assert gl.tobytes() == wl.tobytes(), (b, int(np.sum(gl != wl)), float(np.max(np.abs(gl - wl))))


MODES = [
    dict(),                                            # default: team, one-block, sub-grid, full grid
    dict(small_frontier_solo=3),                       # one-block passes without the 8-warp team
    dict(small_frontier_solo=1),                       # one-block only
    dict(small_frontier_solo=0),                       # every pass on the full grid
    dict(small_frontier_solo=0, narrow_lanes=1),       # full grid, a lane per short row
    dict(solo_entry=1024, subgrid_entry=4096),         # the largest thresholds
    dict(solo_entry=256, subgrid_entry=1024, narrow_lanes=16),
]


@pytest.mark.gpu
@pytest.mark.parametrize("sem", [dlp.SEMANTICS_REF, dlp.SEMANTICS_SPEC])
@pytest.mark.parametrize("n", [5000, 50000])
def test_pass_modes_give_identical_results(gpu, sem, n):
    """The passes give the same results whichever mode runs them: the 8-warp
    team, the one-block mode, the sub-grid, the full grid (lane groups or a
    lane per short row), at any thresholds."""
    p = dlp.Problem(n, 5, 10, 42)
    runs = [dlp.Session.from_problem(p, semantics=sem, **m) for m in MODES]
    for i, bt in enumerate(p.batches):
        st = [r.apply(i, bt) for r in runs]
        labs = [r.labels().tobytes() for r in runs]
        for j in range(1, len(runs)):
            for k in EXACT_STATS:
                assert st[j][k] == st[0][k], (MODES[j], i, k)
            assert labs[j] == labs[0], (MODES[j], i)


@pytest.mark.gpu
def test_reset_replays_identically(gpu):
    p = dlp.Problem(5000, 5, 10, 42)
    sess = dlp.Session.from_problem(p)
    first = [sess.apply(b, bt) for b, bt in enumerate(p.batches)]
    l1 = sess.labels()
    sess.reset()
    second = [sess.apply(b, bt) for b, bt in enumerate(p.batches)]
    for a, c in zip(first, second):
        for k in EXACT_STATS:
            assert a[k] == c[k]
    assert l1.tobytes() == sess.labels().tobytes()


@pytest.mark.gpu
def test_device_resident_batches_match_host_batches(gpu):
    p = dlp.Problem(5000, 5, 10, 42)
    a = dlp.Session.from_problem(p)
    b = dlp.Session.from_problem(p)
    dev = [dlp.DeviceBatch(bt) for bt in p.batches]
    for i, bt in enumerate(p.batches):
        a.apply(i, bt)
        b.apply_device(i, dev[i])
    b.synchronize()
    for i in range(len(p.batches)):
        sa, sb = a.stats(i), b.stats(i)
        for k in EXACT_STATS:
            assert sa[k] == sb[k]
    assert a.labels().tobytes() == b.labels().tobytes()


@pytest.mark.gpu
def test_invalid_vertex_id_rejected(gpu):
    p = dlp.Problem(1000, 3, 5, 7)
    sess = dlp.Session.from_problem(p)
    bad = dlp.Batch.make(inserted=[5, 1000])
    with pytest.raises(dlp.DlpError) as e:
        sess.apply(0, bad)
    assert e.value.status == N.DLP_ERR_INVALID_ARGUMENT
    # the session is still usable
    st = sess.apply(0, p.batches[0])
    assert st["status"] == N.DLP_OK
