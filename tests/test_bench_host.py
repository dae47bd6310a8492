"""Host-side arithmetic of bench.py that its reported numbers rest on: the
stratified plain-path estimator, the shard split of the mixed stream, the
mixed-stream sizes, the algorithmic-byte count and the pass-mode deltas.
CPU only."""
from __future__ import annotations

import numpy as np

import bench


def test_stratified_estimate_is_exact_when_every_graph_is_sampled():
    sizes = [1000, 1500, 3000, 9000, 20000, 50000, 50001, 400000]
    times = {i: 0.001 * s for i, s in enumerate(sizes)}
    total, se, sampled = bench.stratified_plain(sizes, lambda i: times[i], per_stratum=10, bins=4, seed=3)
    assert sorted(sampled) == list(range(len(sizes)))
    assert abs(total - sum(times.values())) < 1e-9
    assert se == 0.0


def test_stratified_estimate_is_unbiased_and_samples_within_strata():
    specs = bench.mix_sizes(512, 1e3, 5e5, 1000003)
    sizes = [s[0] for s in specs]
    # a graph's time grows with its size, with scatter inside a stratum
    rng = np.random.default_rng(5)
    times = np.asarray(sizes, dtype=np.float64) ** 1.1 * rng.uniform(0.5, 1.5, len(sizes)) * 1e-6
    truth = times.sum()
    ests, ses = [], []
    for seed in range(200):
        calls = []
        total, se, sampled = bench.stratified_plain(sizes, lambda i: (calls.append(i), times[i])[1], 3, 8, seed)
        assert sampled == calls and len(set(sampled)) == len(sampled)
        ests.append(total)
        ses.append(se)
    ests = np.asarray(ests)
    # the mean of many estimates is within a few standard errors of the mean
    assert abs(ests.mean() - truth) < 4 * np.mean(ses) / np.sqrt(len(ests))
    # the reported standard error matches the spread of the estimates
    assert 0.6 < ests.std() / np.mean(ses) < 1.6


def test_mix_sizes_are_fixed_and_in_range():
    a = bench.mix_sizes(512, 1e3, 5e5, 1000003)
    assert a == bench.mix_sizes(512, 1e3, 5e5, 1000003)
    assert len(a) == 512
    assert all(1000 <= n <= 500000 for n, _, _, _ in a)
    assert [d for _, d, _, _ in a[:6]] == [3, 5, 7, 3, 5, 7]
    assert [s for _, _, _, s in a] == list(range(512))


def test_shard_split_covers_every_graph_once_and_balances_edges():
    specs = bench.mix_sizes(512, 1e3, 5e5, 1000003)
    for world in (1, 2, 3, 4, 8):
        parts = [bench.shard_graphs(specs, r, world) for r in range(world)]
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(specs)))
        loads = [sum(specs[i][0] * specs[i][1] for i in p) for p in parts]
        biggest = max(n * d for n, d, _, _ in specs)
        # greedy to the least-loaded rank: loads differ by at most one graph
        assert max(loads) - min(loads) <= biggest


def test_algorithmic_bytes_formula():
    st = {"affected_edges": 1000, "frontier_visits": 100, "dirty_entries": 50}
    assert bench.algorithmic_bytes(st, num_edges=10, num_inserted=7) == 12 * 1000 + 20 * 100 + 16 * 50 + 28 * 10 + 16 * 7


def test_mode_delta_per_step():
    before = {"one_block": {"passes": 10, "seconds": 1.0}, "team": {"passes": 4, "seconds": 0.0},
              "sub_grid": {"passes": 0, "seconds": 0.0}, "full_grid": {"passes": 5, "seconds": 0.5}}
    after = {"one_block": {"passes": 30, "seconds": 1.04}, "team": {"passes": 14, "seconds": 0.0},
             "sub_grid": {"passes": 0, "seconds": 0.0}, "full_grid": {"passes": 9, "seconds": 0.54}}
    d = bench.mode_delta(before, after, steps=2)
    assert d["one_block"]["passes"] == 10 and abs(d["one_block"]["ms"] - 20.0) < 1e-9
    assert abs(d["one_block"]["us_per_pass"] - 2000.0) < 1e-6
    assert d["team"] == {"passes": 5.0, "ms": "in one_block"}
    assert d["sub_grid"]["us_per_pass"] is None
    assert abs(d["full_grid"]["us_per_pass"] - 10000.0) < 1e-6


def test_percentile_matches_numpy_linear():
    rng = np.random.default_rng(2)
    for n in (1, 2, 7, 100, 1001):
        xs = rng.exponential(size=n).tolist()
        for q in (0.0, 0.5, 0.9, 0.99, 1.0):
            assert abs(bench.percentile(xs, q) - float(np.percentile(xs, 100 * q))) < 1e-12
    assert bench.percentile([], 0.5) is None
