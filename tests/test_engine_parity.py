"""GPU parity of the multi-graph batch engine.

Each graph stepped in a mixed launch must give exactly what the oracle gives
for that graph alone: per-batch statistics and labels, bit for bit. The mixes
cover uneven sizes and degrees, both semantics, and graphs that join steps in
irregular subsets (the serving pattern).
"""
from __future__ import annotations

import numpy as np
import pytest

import labelpropcuda_gb300 as dlp

EXACT = ["iterations", "num_components", "num_sub_edges", "hook_edges", "seed_frontier", "seed_marks",
         "affected_edges", "frontier_visits", "correct", "total", "init_branch", "hook_truncated"]

GRAPHS = [(1000, 3, 5, 7), (2000, 7, 6, 3), (3000, 4, 3, 11), (5000, 5, 10, 42), (1500, 5, 8, 1)]


def oracle_run(oracle, p, sem):
    orc = oracle.OracleRun.from_problem(p, semantics=sem, threads=4)
    out = []
    for b, bt in enumerate(p.batches):
        st = orc.apply(b, bt)
        out.append((st, orc.labels()))
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("sem", [dlp.SEMANTICS_REF, dlp.SEMANTICS_SPEC])
def test_lockstep_mix_matches_oracle(gpu, oracle, sem):
    probs = [dlp.Problem(*g) for g in GRAPHS]
    want = [oracle_run(oracle, p, sem) for p in probs]
    eng = dlp.Engine(len(probs), semantics=sem)
    gids = [eng.add_problem(p) for p in probs]
    for b in range(max(len(p.batches) for p in probs)):
        items = [(gid, b, p.batches[b]) for gid, p in zip(gids, probs) if b < len(p.batches)]
        stats = eng.step(items)
        for (gid, _, _), st in zip(items, stats):
            w_st, w_lab = want[gids.index(gid)][b]
            for k in EXACT:
                assert st[k] == w_st[k], (gid, b, k, st[k], w_st[k])
            assert eng.labels(gid).tobytes() == w_lab.tobytes(), (gid, b)


@pytest.mark.gpu
def test_irregular_subsets_match_oracle(gpu, oracle):
    """Graphs take part in arbitrary subsets of steps; each graph's sequence of
    batches is still applied in order and must match the oracle."""
    probs = [dlp.Problem(*g) for g in GRAPHS]
    want = [oracle_run(oracle, p, dlp.SEMANTICS_REF) for p in probs]
    eng = dlp.Engine(len(probs))
    gids = [eng.add_problem(p) for p in probs]
    nxt = [0] * len(probs)
    rng = np.random.default_rng(5)
    while any(nxt[i] < len(p.batches) for i, p in enumerate(probs)):
        pick = [i for i, p in enumerate(probs) if nxt[i] < len(p.batches) and rng.random() < 0.5]
        if not pick:
            continue
        items = [(gids[i], nxt[i], probs[i].batches[nxt[i]]) for i in pick]
        stats = eng.step(items)
        for i, st in zip(pick, stats):
            w_st, w_lab = want[i][nxt[i]]
            for k in EXACT:
                assert st[k] == w_st[k], (i, nxt[i], k)
            assert eng.labels(gids[i]).tobytes() == w_lab.tobytes()
            nxt[i] += 1


@pytest.mark.gpu
def test_budget_admission_and_removal(gpu):
    p = dlp.Problem(5000, 5, 10, 42)
    need = dlp.Engine.graph_bytes(p.num_nodes, p.num_edges)
    eng = dlp.Engine(4, memory_budget_bytes=int(need * 1.5))
    g0 = eng.add_problem(p)
    with pytest.raises(dlp.DlpError) as e:
        eng.add_problem(p)
    assert e.value.status == dlp._n.DLP_ERR_OUT_OF_MEMORY
    eng.remove_graph(g0)
    g1 = eng.add_problem(p)
    st = eng.step([(g1, 0, p.batches[0])])
    assert st[0]["status"] == 0


@pytest.mark.gpu
def test_autotune_picks_a_measured_candidate(gpu):
    """The tuner times every launch shape (lane width x one-block and sub-grid
    thresholds) on a generated sample; all of them must agree on the
    statistics (checked inside) and the choice is the fastest measured one."""
    r = dlp.autotune([3000, 1000, 2000], [5, 3, 7], batches=5, max_iterations=300)
    key = lambda c: (c["narrow_lanes"], c["blocks_per_sm"], c["solo_entry"], c["subgrid_entry"])
    shapes = {key(c) for c in r["candidates"]}
    assert len(shapes) == len(r["candidates"]) >= 27  # every candidate a distinct launch shape
    assert all(c["ms"] > 0 for c in r["candidates"])
    best = min(r["candidates"], key=lambda c: c["ms"])
    chosen = (r["narrow_lanes"], r["blocks_per_sm"], r["engine_kw"]["solo_entry"], r["engine_kw"]["subgrid_entry"])
    assert chosen == key(best)
    # the chosen shape is usable as engine settings
    eng = dlp.Engine(2, narrow_lanes=r["narrow_lanes"], **r["engine_kw"])
    eng.close()


@pytest.mark.gpu
def test_multi_instance_sample_matches_oracle(gpu, oracle):
    """16 graphs of the 512-graph multi-instance set (n log-uniform on
    [1e3, 5e5], degree {3,5,7}, seeds i): the smallest, the largest and 14
    evenly spaced by size between them, all stepped together in one launch per
    step for all 10 batches, each checked against its own oracle run. Two
    more engines run every pass on the full grid, with 4-lane groups and with
    a lane per short row.
    Propagation is capped at 1,000 passes per batch on both sides (the
    workload's 100,000 would keep the oracle busy for many minutes on the
    batches that never converge); everything else is the workload's."""
    import bench
    specs = bench.mix_sizes(512, 1e3, 5e5, 1000003)
    order = sorted(range(len(specs)), key=lambda i: specs[i][0])
    pick = [order[round(k * (len(order) - 1) / 15)] for k in range(16)]
    probs = [dlp.Problem(*specs[i]) for i in pick]
    cap = 1000
    orcs = [oracle.OracleRun.from_problem(p, threads=0, max_iterations=cap) for p in probs]
    engines = [dlp.Engine(len(probs), max_iterations=cap),
               dlp.Engine(len(probs), max_iterations=cap, small_frontier_solo=0, narrow_lanes=4),
               dlp.Engine(len(probs), max_iterations=cap, small_frontier_solo=0, narrow_lanes=1)]
    gids = [[e.add_problem(p) for p in probs] for e in engines]
    for b in range(10):
        want = [(o.apply(b, p.batches[b]), o.labels()) for o, p in zip(orcs, probs)]
        for e, ids in zip(engines, gids):
            stats = e.step([(g, b, p.batches[b]) for g, p in zip(ids, probs)])
            for i, (st, g) in enumerate(zip(stats, ids)):
                for k in EXACT:
                    assert st[k] == want[i][0][k], (specs[pick[i]], b, k, st[k], want[i][0][k])
                assert e.labels(g).tobytes() == want[i][1].tobytes(), (specs[pick[i]], b)
