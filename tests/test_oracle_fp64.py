"""The FP64 oracle: each batch's propagation repeated in double precision from
the same state (oracle mode fp64=2), against the fp32 schedule the CUDA path
reproduces bit for bit.

The fp32 labels differ from the FP64 ones by far more than rounding: the
propagation stops once no label moves by more than delta = 1e-4, and which
vertices stop when depends on the arithmetic, so the two runs stop at
different points near the fixed point (and some fp32 batches run to maxIter
where the FP64 run converges). These bounds pin the figures stated for the
two small configurations: every batch within 2e-2 of the FP64 labels, and
fewer than 0.2% of the vertices on the other side of 0.5.
"""
from __future__ import annotations

import numpy as np
import pytest

CASES = [(5000, 5, 10, 42), (50000, 5, 10, 42)]


@pytest.mark.parametrize("args", CASES, ids=lambda a: "n%d" % a[0])
def test_fp32_schedule_against_fp64_shadow(oracle, args):
    p = oracle.OracleProblem(*args)
    run = oracle.OracleRun.from_problem(p, threads=0, fp64=2)
    worst = 0.0
    for b, bt in enumerate(p.batches):
        st = run.apply(b, bt)
        lab32, lab64 = run.labels().astype(np.float64), run.labels64()
        err = np.abs(lab32 - lab64)
        worst = max(worst, float(err.max()))
        flips = int(np.sum((lab32 >= 0.5) != (lab64 >= 0.5)))
        assert err.max() < 2e-2, (b, float(err.max()))
        assert flips < 0.002 * p.num_nodes, (b, flips)
        if st["iterations"] < 100000:  # converged in fp32: the shadow converges too
            assert run.shadow_iterations() < 100000, b
    assert worst > 0.0  # the shadow really is a different computation


def test_fp64_full_run_keeps_ground_truth(oracle):
    p = oracle.OracleProblem(2000, 7, 6, 3)
    run = oracle.OracleRun.from_problem(p, threads=0, fp64=1)
    for b, bt in enumerate(p.batches):
        run.apply(b, bt)
        lab = run.labels64()
        assert np.array_equal(lab[bt.gt_ids], bt.gt_labels.astype(np.float64))
        assert np.all((lab >= 0.0) & (lab <= 1.0))
