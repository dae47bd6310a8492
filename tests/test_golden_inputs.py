"""The product's input generator and the oracle's host CSR rebuild against the
reference's own host code (golden fixtures made by tests/golden/make_golden.py
from the reference's generateSparseGraph, generateBatches, computeAvgEdgeWeight
and updateHostCSR)."""
from __future__ import annotations

import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"
DIGESTS = json.loads((GOLDEN / "ref_digests.json").read_text())
FIELDS = ["inserted", "gt_ids", "gt_labels", "deleted", "edge_src", "edge_dst", "edge_weight"]


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("key", sorted(DIGESTS["configs"]))
def test_generator_matches_reference(native, key):
    import labelpropcuda_gb300 as dlp
    g = DIGESTS["configs"][key]
    n, deg, nb, seed = g["args"]
    p = dlp.Problem(n, deg, nb, seed)
    assert p.num_nodes == g["n"] and p.num_edges == g["num_edges"]
    assert sha(p.row_ptr) == g["row_ptr"]
    assert sha(p.col_ind) == g["col_ind"]
    assert sha(p.values) == g["values"]
    assert sha(p.true_labels) == g["true_labels"]
    assert len(p.batches) == len(g["batches"])
    for b, gb in zip(p.batches, g["batches"]):
        for f in FIELDS:
            assert sha(getattr(b, f)) == gb[f], f


def test_generator_small_arrays(native):
    import labelpropcuda_gb300 as dlp
    z = np.load(GOLDEN / "ref_small.npz")
    p = dlp.Problem(*DIGESTS["small"])
    np.testing.assert_array_equal(p.row_ptr, z["row_ptr"])
    np.testing.assert_array_equal(p.col_ind, z["col_ind"])
    assert p.values.tobytes() == z["values"].tobytes()
    for i, b in enumerate(p.batches):
        for f in FIELDS:
            assert getattr(b, f).tobytes() == z[f"b{i}_{f}"].tobytes()


def test_auto_tau_matches_reference(native):
    import labelpropcuda_gb300 as dlp
    L = native
    for key, g in DIGESTS["configs"].items():
        p = dlp.Problem(*g["args"])
        tau = L.dlp_mean_edge_weight(p.num_edges, p.col_ind.ctypes.data, p.values.ctypes.data)
        assert np.float32(tau) == np.float32(g["tau"]), key


@pytest.mark.parametrize("key", sorted(DIGESTS["configs"]))
def test_oracle_host_rebuild_matches_reference(native, oracle, key):
    """The oracle's per-batch active CSR and host status equal the
    reference's updateHostCSR output (src/dynLP.cu:111-167) batch by batch."""
    import labelpropcuda_gb300 as dlp
    g = DIGESTS["configs"][key]
    p = dlp.Problem(*g["args"])
    run = oracle.OracleRun.from_problem(p, record=True, threads=4)
    assert np.float32(run.tau) == np.float32(g["tau"])
    for b, (batch, ga) in enumerate(zip(p.batches, g["active"])):
        run.apply(b, batch)
        assert sha(run.artefact(oracle.ART_ROW_PTR)) == ga["row_ptr"], b
        assert sha(run.artefact(oracle.ART_COL_IND)) == ga["col_ind"], b
        assert sha(run.artefact(oracle.ART_VALUES)) == ga["values"], b
        assert sha(run.artefact(oracle.ART_STATUS)) == ga["status"], b


@pytest.mark.parametrize("key", sorted(DIGESTS["configs"]))
def test_oracle_generator_matches_reference(oracle, key):
    """The oracle's own restatement of the generator (used where the product
    library must not be loaded) makes the reference's inputs too."""
    g = DIGESTS["configs"][key]
    p = oracle.OracleProblem(*g["args"])
    assert p.num_nodes == g["n"] and p.num_edges == g["num_edges"]
    for name in ("row_ptr", "col_ind", "values", "true_labels"):
        assert sha(getattr(p, name)) == g[name], name
    assert len(p.batches) == len(g["batches"])
    for b, gb in zip(p.batches, g["batches"]):
        for f in FIELDS:
            assert sha(getattr(b, f)) == gb[f], (b, f)
