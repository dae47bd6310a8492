"""The oracle and the CUDA path against the reference's own kernels, on the GPU.

oracle/_ref/ref_kernels is the reference's runDynLP with its own step
launchers and kernels, built with its own flags (-O3 --use_fast_math) from a
copy of its sources in which three index -1 accesses of the components step
are guarded (oracle/guard_reference.py), and its components step bounded to
the edges it was given (oracle/ref_kernels.cu). It records, batch by batch,
what each step produced and the exact state its propagation started from.

Checked on every batch:
  bit-exact   kept-edge count (numSubEdges), edges hooked, component count,
              component id of every inserted vertex (the reference numbers
              components by ascending root; roots are minimum vertex ids),
              the affected set when propagation starts
  1e-5        initial labels of the inserted vertices (the reference sums
              supernode weights with float atomics in a varying order and
              divides with --use_fast_math)
Propagation, from the reference's own recorded input state of each batch:
  this library's propagation launcher with the reference's fast-math
  division (DLP_ARITH_REFERENCE_FAST_MATH) must take the same number of
  passes and give labels within 1e-5 of the reference's, with identical
  0.5-threshold predictions except where |label - 0.5| < 1e-4, on every
  batch whose propagation converges (runs below maxIter). With IEEE division
  (the default, bit-exact with the oracle) the differences are reported.
  Batches that run to maxIter never reach a fixed point (the labels keep
  swinging); there a last-bit difference changes the state the run stops in,
  so those are reported, not asserted, as are the labels after a whole replay
  (every later batch starts from the state the earlier ones left).

Needs the guarded copy of the reference's sources in oracle/_ref/src (made
with `make -C oracle refsrc REF=<reference checkout>`; git-ignored, it travels
with the working tree). Without it the test is skipped.
"""
from __future__ import annotations

import ctypes
import json
import os
from pathlib import Path

import numpy as np
import pytest

import labelpropcuda_gb300 as dlp
from labelpropcuda_gb300 import DeviceArray
from labelpropcuda_gb300 import _native as N

CASES = [(5000, 5, 10, 42), (50000, 5, 10, 42)]
MAX_ITER = 100000


def _report(name: str, rows) -> None:
    d = os.environ.get("DLP_REPORT_DIR")
    if d:
        Path(d).mkdir(parents=True, exist_ok=True)
        (Path(d) / f"{name}.json").write_text(json.dumps(rows, indent=1))


def _label_diff(mine: np.ndarray, theirs: np.ndarray) -> dict:
    diff = np.abs(mine.astype(np.float64) - theirs.astype(np.float64))
    flips = (mine >= 0.5) != (theirs >= 0.5)
    near = np.abs(theirs.astype(np.float64) - 0.5) < 1e-4
    return {"max_abs": float(diff.max()) if diff.size else 0.0, "differing": int(np.sum(mine != theirs)),
            "flips": int(flips.sum()), "flips_outside_band": int(np.sum(flips & ~near))}


def _propagate_from(rb: dict, arithmetic: int) -> tuple[int, np.ndarray]:
    """This library's propagation launcher on the reference's recorded input
    state of one batch."""
    L = N.lib()
    N.check(L.dlp_set_launcher_arithmetic(arithmetic))
    try:
        n = rb["in_labels"].size
        d = [DeviceArray(rb[k]) for k in ("in_row_ptr", "in_col_ind", "in_values", "in_labels")]
        buf = DeviceArray(rb["in_labels"])
        st, gt, aff = (DeviceArray(rb[k]) for k in ("in_status", "in_gt", "in_affected"))
        it = ctypes.c_int(0)
        N.check(L.dlp_iterative_propagation(d[0].ptr, d[1].ptr, d[2].ptr, d[3].ptr, buf.ptr, st.ptr, gt.ptr, aff.ptr,
                                            n, ctypes.c_float(1e-4), MAX_ITER, ctypes.byref(it), None))
        N.check(L.dlp_device_synchronize())
        return it.value, d[3].get()
    finally:
        N.check(L.dlp_set_launcher_arithmetic(N.ARITH_IEEE))


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=lambda c: "n%d_d%d_b%d_s%d" % c)
def test_against_reference_kernels(gpu, oracle, case, tmp_path):
    if oracle.build_ref_kernels() is None:
        pytest.skip("the guarded copy of the reference's sources (oracle/_ref/src) is absent")
    n, deg, nb, seed = case
    ref = oracle.run_ref_kernels(n, deg, nb, seed, MAX_ITER, tmp_path / "ref.bin", record=True)
    p = oracle.OracleProblem(n, deg, nb, seed)
    orc = oracle.OracleRun.from_problem(p, record=True, threads=0, max_iterations=MAX_ITER)
    assert np.float32(ref["tau"]) == np.float32(orc.tau)
    assert len(ref["batches"]) == nb
    rows, problems = [], []
    for b, (bt, rb) in enumerate(zip(p.batches, ref["batches"])):
        st = orc.apply(b, bt)
        row = {"batch": b, "ref_passes": rb["iterations"], "oracle_passes": st["iterations"]}
        # structural outputs: bit-exact
        if rb["num_new_edges"] >= 0:
            assert rb["num_sub_edges"] == st["num_sub_edges"], (b, "numSubEdges")
        else:
            assert st["num_sub_edges"] == 0, b
        if rb["hook_edges"] >= 0:
            assert rb["hook_edges"] == st["hook_edges"], (b, "hooked edges")
            assert rb["num_components"] == st["num_components"], (b, "components")
            np.testing.assert_array_equal(rb["comp_id"], orc.artefact(oracle.ART_COMP_ID), err_msg=f"batch {b}")
        np.testing.assert_array_equal(rb["seed_marks"], orc.artefact(oracle.ART_SEED_MARKS), err_msg=f"batch {b}")
        if rb["init_labels"].size:
            d0 = np.abs(rb["init_labels"].astype(np.float64) - orc.artefact(oracle.ART_INIT_LABELS))
            row["init_max_abs"] = float(d0.max())
            assert d0.max() <= 1e-5, (b, float(d0.max()))
        # propagation from the reference's own input state of this batch
        for name, mode in (("fast_math", N.ARITH_REFERENCE_FAST_MATH), ("ieee", N.ARITH_IEEE)):
            it, lab = _propagate_from(rb, mode)
            row[name] = dict(passes=it, **_label_diff(lab, rb["labels"]))
        converges = rb["iterations"] < MAX_ITER
        row["reference_converges"] = converges
        if converges:
            fm = row["fast_math"]
            if fm["passes"] != rb["iterations"] or fm["max_abs"] > 1e-5 or fm["flips_outside_band"]:
                problems.append(b)
        # whole replay, state carried from batch to batch (reported)
        row["replay"] = _label_diff(orc.labels(), rb["labels"])
        rows.append(row)
    _report(f"reference_kernels_n{n}", rows)
    assert not problems, [rows[b] for b in problems]
