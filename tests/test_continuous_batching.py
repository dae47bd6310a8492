"""GPU parity of continuous batching: sliced engine steps and the server.

A batch whose propagation is cut into slices, continued next to other graphs'
batches that start and end at other times, must give exactly what the same
batch gives when it runs alone in one unsliced step: the same statistics and
the same labels, bit for bit. The unsliced engine is itself checked against
the oracle by test_engine_parity.
"""
from __future__ import annotations

import numpy as np
import pytest

import labelpropcuda_gb300 as dlp
from labelpropcuda_gb300 import _native as N

EXACT = ["iterations", "num_components", "num_sub_edges", "hook_edges", "seed_frontier",
         "seed_marks", "affected_edges", "frontier_visits", "correct", "total", "init_branch", "hook_truncated",
         "dirty_rows", "dirty_entries"]

GRAPHS = [(1000, 3, 5, 7), (2000, 7, 6, 3), (3000, 4, 3, 11), (5000, 5, 10, 42), (1500, 5, 8, 1)]
MAX_ITER = 300  # keeps the oscillating batches short when sliced one pass at a time


def alone(p, **kw):
    eng = dlp.Engine(1, max_iterations=MAX_ITER, **kw)
    gid = eng.add_problem(p)
    out = []
    for b, bt in enumerate(p.batches):
        st = eng.step([(gid, b, bt)])[0]
        out.append((st, eng.labels(gid)))
    eng.close()
    return out


def same(st, want, where):
    for k in EXACT:
        assert st[k] == want[k], (where, k, st[k], want[k])


@pytest.mark.gpu
@pytest.mark.parametrize("solo", [0, 1, 3, 7])
@pytest.mark.parametrize("budget", [1, 7, 64])
def test_sliced_batches_match_unsliced(gpu, budget, solo):
    p = dlp.Problem(5000, 5, 10, 42)
    want = alone(p, small_frontier_solo=solo)
    eng = dlp.Engine(1, max_iterations=MAX_ITER, small_frontier_solo=solo)
    gid = eng.add_problem(p)
    for b, bt in enumerate(p.batches):
        db = dlp.DeviceBatch(bt)
        fin, cont = eng.step_sliced([(gid, b, db)], pass_budget=budget)
        steps = 1
        while not fin:
            assert cont == 1 and eng.in_progress(gid)
            fin, cont = eng.step_sliced([], pass_budget=budget)
            steps += 1
        assert fin == [gid] and cont == 0
        st = eng.stats(gid, b)
        same(st, want[b][0], (budget, solo, b))
        assert steps >= min(1, st["iterations"]) and steps <= st["iterations"] // budget + 1
        assert eng.labels(gid).tobytes() == want[b][1].tobytes(), (budget, solo, b)


@pytest.mark.gpu
def test_staggered_batches_match_alone(gpu):
    """Batches of several graphs start while others are mid-propagation and
    end at different steps; each must equal its graph run alone."""
    probs = [dlp.Problem(*g) for g in GRAPHS]
    want = [alone(p) for p in probs]
    eng = dlp.Engine(len(probs), max_iterations=MAX_ITER)
    gids = [eng.add_problem(p) for p in probs]
    nxt = [0] * len(probs)
    live: dict[int, tuple[int, dlp.DeviceBatch]] = {}
    rng = np.random.default_rng(9)
    while any(nxt[i] < len(p.batches) for i, p in enumerate(probs)) or live:
        start = []
        for i, p in enumerate(probs):
            if i not in live and nxt[i] < len(p.batches) and rng.random() < 0.6:
                db = dlp.DeviceBatch(p.batches[nxt[i]])
                live[i] = (nxt[i], db)
                start.append((gids[i], nxt[i], db))
                nxt[i] += 1
        if not start and not live:
            continue
        fin, cont = eng.step_sliced(start, pass_budget=int(rng.integers(1, 20)))
        for gid in fin:
            i = gids.index(gid)
            b, _ = live.pop(i)
            same(eng.stats(gid, b), want[i][b][0], (i, b))
            assert eng.labels(gid).tobytes() == want[i][b][1].tobytes(), (i, b)
        assert cont == len(live)


@pytest.mark.gpu
def test_time_sliced_steps_match_alone(gpu):
    probs = [dlp.Problem(*g) for g in GRAPHS[:3]]
    want = [alone(p) for p in probs]
    eng = dlp.Engine(len(probs), max_iterations=MAX_ITER)
    gids = [eng.add_problem(p) for p in probs]
    for b in range(max(len(p.batches) for p in probs)):
        dbs = [(gids[i], b, dlp.DeviceBatch(p.batches[b])) for i, p in enumerate(probs) if b < len(p.batches)]
        done, _ = eng.step_sliced(dbs, slice_us=20.0)
        while len(done) < len(dbs):
            more, _ = eng.step_sliced([], slice_us=20.0)
            done += more
        for gid, _, _ in dbs:
            i = gids.index(gid)
            same(eng.stats(gid, b), want[i][b][0], (i, b))
            assert eng.labels(gid).tobytes() == want[i][b][1].tobytes()


@pytest.mark.gpu
def test_in_progress_graph_is_guarded(gpu):
    p = dlp.Problem(5000, 5, 10, 42)
    eng = dlp.Engine(1, max_iterations=MAX_ITER)
    gid = eng.add_problem(p)
    # find a batch that needs more than one pass
    for b, bt in enumerate(p.batches):
        db = dlp.DeviceBatch(bt)
        fin, _ = eng.step_sliced([(gid, b, db)], pass_budget=1)
        if not fin:
            break
    else:
        pytest.fail("no batch ran more than one pass")
    with pytest.raises(dlp.DlpError) as e:
        eng.step([(gid, b + 1, p.batches[b + 1])])
    assert e.value.status == N.DLP_ERR_INVALID_ARGUMENT
    with pytest.raises(dlp.DlpError):
        eng.labels(gid)
    with pytest.raises(dlp.DlpError):
        eng.stats(gid, b)
    while eng.in_progress(gid):
        eng.step_sliced([], pass_budget=50)
    assert eng.stats(gid, b)["iterations"] >= 2


def _trace(probs, gids, seed, span_s):
    rng = np.random.default_rng(seed)
    items = []
    for i, p in enumerate(probs):
        t = np.sort(rng.uniform(0.0, span_s, len(p.batches)))
        items += [(float(t[b]), gids[i], b, p.batches[b]) for b in range(len(p.batches))]
    items.sort(key=lambda x: x[0])
    return items


@pytest.mark.gpu
@pytest.mark.parametrize("serial", [False, True])
def test_server_results_same_alone_and_in_the_mix(gpu, serial):
    probs = [dlp.Problem(*g) for g in GRAPHS]
    want = [alone(p) for p in probs]
    eng = dlp.Engine(len(probs), max_iterations=MAX_ITER)
    gids = [eng.add_problem(p) for p in probs]
    srv = dlp.Server(eng, slice_us=50.0, serial=serial)
    trace = _trace(probs, gids, 3, 0.05)
    res, span = srv.replay(trace)
    assert span > 0
    for (t, gid, b, _), r in zip(trace, res):
        i = gids.index(gid)
        assert r["status"] == 0 and r["graph_id"] == gid and r["batch_index"] == b
        assert r["finish_s"] >= r["admit_s"] >= r["arrival_s"] - 1e-9
        same(r["stats"], want[i][b][0], (serial, i, b))
    for i, gid in enumerate(gids):
        assert eng.labels(gid).tobytes() == want[i][-1][1].tobytes()
    srv.close()


@pytest.mark.gpu
def test_server_submit_poll_and_memory_budget(gpu):
    probs = [dlp.Problem(*g) for g in GRAPHS[:3]]
    want = [alone(p) for p in probs]
    eng = dlp.Engine(len(probs), max_iterations=MAX_ITER)
    gids = [eng.add_problem(p) for p in probs]
    # room for the resident graphs plus about one running request
    biggest = max(24 * bt.edge_src.size + bt.nbytes() + 8 * bt.deleted.size + 4096 for p in probs for bt in p.batches)
    srv = dlp.Server(eng, slice_us=30.0, memory_budget_bytes=eng.bytes_in_use + int(1.2 * biggest))
    rids = {}
    for b in range(max(len(p.batches) for p in probs)):
        for i, p in enumerate(probs):
            if b < len(p.batches):
                rids[srv.submit(gids[i], b, p.batches[b])] = (i, b)
    done = srv.drain()
    assert sorted(done) == sorted(rids)
    for rid, (i, b) in rids.items():
        r = srv.result(rid)
        assert r["status"] == 0
        same(r["stats"], want[i][b][0], (i, b))
    # a request that can never fit is failed, not queued forever
    tiny = dlp.Server(eng, memory_budget_bytes=eng.bytes_in_use + 16)
    rid = tiny.submit(gids[0], 0, probs[0].batches[1])
    assert tiny.poll() == [rid]
    assert tiny.result(rid)["status"] == N.DLP_ERR_OUT_OF_MEMORY


@pytest.mark.gpu
def test_snapshot_evict_restore_continues_identically(gpu):
    """A graph snapshotted after some batches, evicted, and restored (into
    another engine, under another id) continues exactly as if it had stayed."""
    p = dlp.Problem(5000, 5, 10, 42)
    want = alone(p)
    a = dlp.Engine(4, max_iterations=MAX_ITER)
    filler = a.add_problem(dlp.Problem(1000, 3, 5, 7))
    gid = a.add_problem(p)
    for b in range(4):
        a.step([(gid, b, p.batches[b])])
    snap = a.snapshot(gid)
    used = a.bytes_in_use
    a.remove_graph(gid)
    assert a.bytes_in_use < used
    other = dlp.Engine(2, max_iterations=MAX_ITER)
    other.add_problem(dlp.Problem(2000, 7, 6, 3))
    g2 = other.restore(snap)
    assert other.stats(g2, 3)["iterations"] == want[3][0]["iterations"]  # kept statistics travel along
    assert other.labels(g2).tobytes() == want[3][1].tobytes()
    for b in range(4, len(p.batches)):
        st = other.step([(g2, b, p.batches[b])])[0]
        same(st, want[b][0], ("restored", b))
        assert other.labels(g2).tobytes() == want[b][1].tobytes()
    # the engine it left keeps working, and a restore into it works too
    g3 = a.restore(snap)
    same(a.step([(g3, 4, p.batches[4])])[0], want[4][0], ("back", 4))
    a.step([(filler, 0, dlp.Problem(1000, 3, 5, 7).batches[0])])
    with pytest.raises(dlp.DlpError):
        dlp.Engine(1, max_iterations=MAX_ITER, semantics=dlp.SEMANTICS_SPEC).restore(snap)


@pytest.mark.gpu
def test_server_evicts_idle_graphs_to_fit_the_budget(gpu):
    """Five resident graphs under a budget that holds about two of them: the
    server evicts idle graphs to host memory and restores them (same ids)
    when their requests come; every result equals the graph run alone."""
    probs = [dlp.Problem(*g) for g in GRAPHS]
    want = [alone(p) for p in probs]
    eng = dlp.Engine(len(probs), max_iterations=MAX_ITER)
    gids = [eng.add_problem(p) for p in probs]
    L = N.lib()
    sizes = sorted(int(L.dlp_engine_graph_resident_bytes(eng._h, g)) for g in gids)
    biggest_req = max(24 * bt.edge_src.size + bt.nbytes() + 8 * bt.deleted.size + 4096
                      for p in probs for bt in p.batches)
    budget = sizes[-1] + sizes[-2] + 4 * biggest_req
    assert sum(sizes) > budget  # not everything fits at once
    srv = dlp.Server(eng, slice_us=50.0, memory_budget_bytes=budget, evict_idle=True)
    trace = _trace(probs, gids, 5, 0.05)
    res, _ = srv.replay(trace)
    for (t, gid, b, _), r in zip(trace, res):
        i = gids.index(gid)
        assert r["status"] == 0, r
        same(r["stats"], want[i][b][0], ("evict", i, b))
    ev, rs = srv.evictions()
    assert ev > 0 and rs > 0
    assert eng.bytes_in_use <= budget
    for i, gid in enumerate(gids):
        srv.make_resident(gid)
        assert eng.labels(gid).tobytes() == want[i][-1][1].tobytes()
    srv.close()


@pytest.mark.gpu
def test_evicted_graph_keeps_its_id(gpu):
    """A graph evicted by the server keeps its id: a graph added to the engine
    meanwhile takes another id, and the evicted one comes back intact."""
    p0, p1 = dlp.Problem(3000, 4, 3, 11), dlp.Problem(2000, 7, 6, 3)
    want0 = alone(p0)
    eng = dlp.Engine(4, max_iterations=MAX_ITER)
    g0, g1 = eng.add_problem(p0), eng.add_problem(p1)
    for b in range(len(p0.batches)):
        eng.step([(g0, b, p0.batches[b])])
    L = N.lib()
    size1 = int(L.dlp_engine_graph_resident_bytes(eng._h, g1))
    req = max(24 * bt.edge_src.size + 2 * bt.nbytes() + 8 * bt.deleted.size + 4096 for bt in p1.batches)
    srv = dlp.Server(eng, memory_budget_bytes=size1 + 4 * req, evict_idle=True)
    rid = srv.submit(g1, 0, p1.batches[0])
    srv.drain()
    assert srv.result(rid)["status"] == 0
    assert srv.evictions()[0] == 1 and eng.bytes_in_use <= size1 + 4 * req
    g2 = eng.add_problem(dlp.Problem(1000, 3, 5, 7))
    assert g2 not in (g0, g1)
    srv.make_resident(g0)
    assert eng.labels(g0).tobytes() == want0[-1][1].tobytes()
    srv.close()
