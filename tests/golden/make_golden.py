"""Regenerates the golden fixtures from the reference's own host code.

Runs oracle/_ref/ref_harness (built by `make -C oracle ref` from the reference
checkout; see oracle/ref_harness.cu), which calls the reference's
generateSparseGraph, generateBatches, computeAvgEdgeWeight and updateHostCSR,
and stores what they produced:

  ref_small.npz       every array for n=1000, degree 3, 5 batches, seed 7
  ref_digests.json    SHA-256 of every array for the larger configurations

Usage: python tests/golden/make_golden.py   (needs the reference checkout)
"""
from __future__ import annotations

import hashlib
import json
import struct
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
HARNESS = ROOT / "oracle" / "_ref" / "ref_harness"

SMALL = (1000, 3, 5, 7)
DIGEST_CONFIGS = [(1000, 3, 5, 7), (2000, 7, 6, 3), (3000, 4, 3, 11), (5000, 5, 10, 42), (50000, 5, 10, 42)]
BATCH_FIELDS = ["inserted", "gt_ids", "gt_labels", "deleted", "edge_src", "edge_dst", "edge_weight"]
BATCH_TYPES = [np.int32, np.int32, np.float32, np.int32, np.int32, np.int32, np.float32]


def read_dump(path: Path) -> dict:
    buf = path.read_bytes()
    off = 0

    def i64():
        nonlocal off
        (v,) = struct.unpack_from("<q", buf, off)
        off += 8
        return v

    def vec(dt):
        nonlocal off
        n = i64()
        a = np.frombuffer(buf, dtype=dt, count=n, offset=off).copy()
        off += n * np.dtype(dt).itemsize
        return a

    out = {"n": i64(), "row_ptr": vec(np.int32), "col_ind": vec(np.int32), "values": vec(np.float32),
           "true_labels": vec(np.float32)}
    nb = i64()
    out["batches"] = [{f: vec(t) for f, t in zip(BATCH_FIELDS, BATCH_TYPES)} for _ in range(nb)]
    (out["tau"],) = struct.unpack_from("<f", buf, off)
    off += 4
    out["active"] = [{"row_ptr": vec(np.int32), "col_ind": vec(np.int32), "values": vec(np.float32),
                      "status": vec(np.int32)} for _ in range(nb)]
    assert off == len(buf)
    return out


def run_harness(n, deg, nb, seed) -> dict:
    with tempfile.TemporaryDirectory() as td:
        p = Path(td) / "dump.bin"
        subprocess.run([str(HARNESS), str(n), str(deg), str(nb), str(seed), str(p)], check=True,
                       stdout=subprocess.DEVNULL)
        return read_dump(p)


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def digests_of(d: dict) -> dict:
    out = {"n": d["n"], "num_edges": int(d["col_ind"].size), "tau": float(d["tau"]),
           "row_ptr": digest(d["row_ptr"]), "col_ind": digest(d["col_ind"]), "values": digest(d["values"]),
           "true_labels": digest(d["true_labels"]), "batches": [], "active": []}
    for b in d["batches"]:
        out["batches"].append({f: digest(b[f]) for f in BATCH_FIELDS} | {"sizes": [int(b[f].size) for f in BATCH_FIELDS]})
    for a in d["active"]:
        out["active"].append({k: digest(v) for k, v in a.items()} | {"num_edges": int(a["col_ind"].size)})
    return out


def main() -> int:
    if not HARNESS.exists():
        subprocess.run(["make", "-C", str(ROOT / "oracle"), "ref"], check=True)
    d = run_harness(*SMALL)
    arrays = {"row_ptr": d["row_ptr"], "col_ind": d["col_ind"], "values": d["values"],
              "true_labels": d["true_labels"], "tau": np.float32(d["tau"])}
    for i, b in enumerate(d["batches"]):
        for f in BATCH_FIELDS:
            arrays[f"b{i}_{f}"] = b[f]
    for i, a in enumerate(d["active"]):
        for k, v in a.items():
            arrays[f"a{i}_{k}"] = v
    np.savez_compressed(HERE / "ref_small.npz", **arrays)
    meta = {"generated_by": "tests/golden/make_golden.py via oracle/_ref/ref_harness", "small": list(SMALL),
            "configs": {}}
    for cfg in DIGEST_CONFIGS:
        meta["configs"]["n%d_d%d_b%d_s%d" % cfg] = {"args": list(cfg)} | digests_of(run_harness(*cfg))
    (HERE / "ref_digests.json").write_text(json.dumps(meta, indent=1) + "\n")
    print("wrote", HERE / "ref_small.npz", HERE / "ref_digests.json")
    return 0


if __name__ == "__main__":
    sys.exit(main())
