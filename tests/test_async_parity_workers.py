"""Per-epoch parity of the asynchronous kernel against the many-worker FP64 oracle, on a
case with the 480,189 x 17,770 workload's shape at a smaller size (Zipf(0.8) users,
Zipf(1.1) items, integer ratings 1-5): enough ratings for priority columns (block
visits) and the kernel's full worker count.

The oracle is the reference's algorithm with the same number of workers in FP64, run as
the oracle's deterministic event simulation (oracle/nomad_oracle.cpp, async_sim).  Its
trajectory is robust to schedule details (other worker counts, route seeds and timing
constants move it by at most ~0.1%), so it is the comparator for an asynchronous run.
Tolerances, measured and stated.  The first epoch starts from errors near 3 and its test
RMSE depends on how the schedule interleaves columns: on this case the kernel lands 2.1%
below the oracle with its priority columns (heavy columns visiting whole thread blocks)
and 1.4% above it with them switched off; bound 5%.  The second epoch is within 0.6%;
bound 1.5%.  From the third epoch on the kernel is within 0.11% of the oracle either way;
bound 0.5%, the bar of the asynchronous form.  (On the full 480,189 x 17,770 workload the
gap after the first epoch stays between 0.3% and 0.7% until about epoch 18; the bench
line reports it per epoch.)"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HP = dict(dim=100, lrate=0.002, drate=0.05, reg=0.05)
EPOCHS = 4


def _case(ng):
    return ng.synth(ng.synth_spec(2, m=60000, n=3000, nnz_train=4000000, nnz_test=100000, seed=4242))


def _gpu_curve(ng, train, test, **kw):
    with ng.Nomad(train, test, mode="async", init_parts=16, **HP, **kw) as nm:
        workers = nm.info()["workers"]
        prio = nm.info()["priority_tokens"]
        rm = []
        for _ in range(EPOCHS):
            assert nm.epoch(1)["updates"] == train.nnz
            rm.append(nm.rmse(train=False)[1])
    return rm, workers, prio


def _oracle_curve(O, train, test, workers):
    csc = O.row_major_to_csc(train.m, train.n, train.row_counts, train.cols, train.vals)
    tcsc = O.row_major_to_csc(test.m, test.n, test.row_counts, test.cols, test.vals)
    W, H = O.init_factors(train.m, train.n, HP["dim"], 12345, 16)
    rm = []
    for e in range(EPOCHS):
        O.async_sim(csc, W, H, workers, e, 1, HP["lrate"], HP["drate"], HP["reg"], seed=12345, partition=1)
        rm.append(O.rmse(tcsc, W, H))
    return rm


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_per_epoch_gap_to_many_worker_oracle(ng, O, gpu_ok, precision):
    train, test = _case(ng)
    gpu, workers, prio = _gpu_curve(ng, train, test, precision=precision)
    assert prio > 0 and workers >= 1500
    ref = _oracle_curve(O, train, test, workers)
    gaps = [(g - r) / r for g, r in zip(gpu, ref)]
    print(precision, "workers", workers, "priority columns", prio, "gaps", [round(100 * g, 3) for g in gaps])
    gpu_np, workers_np, prio_np = _gpu_curve(ng, train, test, precision=precision, priority_permille=-1)
    assert prio_np == 0 and workers_np == workers
    gaps_np = [(g - r) / r for g, r in zip(gpu_np, ref)]
    print(precision, "no priority columns: gaps", [round(100 * g, 3) for g in gaps_np])
    for gs in (gaps, gaps_np):
        assert abs(gs[0]) <= 0.05, gs
        assert abs(gs[1]) <= 0.015, gs
        assert max(abs(g) for g in gs[2:]) <= 0.005, gs
