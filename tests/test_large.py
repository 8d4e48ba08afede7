"""Full-size runs of the larger workloads, checked through properties that hold at any
size (the FP64 oracle cannot replay them in test time).

The 1,000,990 x 624,961 workload: 252,800,275 training ratings, Zipf(0.9) degrees on both
sides, integer ratings 0-100 from a planted rank-30 model, k = 100."""
import numpy as np
import pytest

KW = dict(dim=100, lrate=0.0005, drate=0.05, reg=0.05, mode="async", init_parts=16)


@pytest.mark.gpu
def test_precision_workload_properties(ng, gpu_ok):
    """Every training rating is updated once per epoch in both forms; the test RMSE falls
    every epoch; after the first epoch the bf16 form's test RMSE stays within 1% of the
    fp32 form's at equal epochs.  (The two forms differ in storage rounding and in their
    asynchronous update order, which dominates the first epoch: 2-3% apart there.)"""
    train, test = ng.synth(3)
    assert (train.m, train.n, train.nnz) == (1000990, 624961, 252800275)
    curves = {}
    for prec in ("fp32", "bf16"):
        with ng.Nomad(train, test, precision=prec, **KW) as nm:
            r = []
            for _ in range(4):
                st = nm.epoch(1)
                assert st["updates"] == train.nnz
                r.append(nm.rmse(train=False)[1])
        assert all(np.isfinite(r)) and all(b < a for a, b in zip(r, r[1:])), (prec, r)
        curves[prec] = r
    gap = max(abs(b - f) / f for f, b in zip(curves["fp32"][1:], curves["bf16"][1:]))
    assert gap <= 0.01, (gap, curves)
