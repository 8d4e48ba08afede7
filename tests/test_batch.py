"""The batched form: many independent problems, one graph-captured launch per epoch.

Each problem runs the reference's one-worker schedule (columns in index order), so the
oracle's replay of that problem is its exact counterpart:
  * exact arithmetic, fp32: every problem's factors equal the oracle's nomad_float replay
    bit for bit;
  * FMA arithmetic (fp32 and bf16 with stochastic rounding): every problem's test RMSE is
    within 0.5% of the FP64 oracle (nomad_double replay) at equal epochs.
"""
import ctypes

import numpy as np
import pytest

LR, DR, REG = 0.002, 0.1, 0.05


def batch_shapes(ng, count, seed=12345):
    out = []
    for i in range(count):
        spec, dim = ng._abi.SynthSpec(), ctypes.c_int32()
        ng.check(ng.lib().nomad_synth_batch_problem(seed, i, ctypes.byref(spec), ctypes.byref(dim)),
                 "nomad_synth_batch_problem")
        out.append((spec.m, spec.n, spec.nnz_train, spec.nnz_test, dim.value))
    return out


def test_batch_generator_ranges(ng):
    """Shapes follow the batched workload's laws: m in [200, 20,000], n in [100, 5,000],
    density in [0.5%, 5%], k in {16, 32, 64}; the same seed gives the same problems."""
    a = batch_shapes(ng, 300)
    assert a == batch_shapes(ng, 300)
    assert a != batch_shapes(ng, 300, seed=7)
    for m, n, ntr, nte, k in a:
        assert 200 <= m <= 20000 and 100 <= n <= 5000
        dens = (ntr + nte) / (m * n)
        assert 0.0049 <= dens <= 0.0501
        assert k in (16, 32, 64)
        assert nte == max(1, (ntr + nte) // 10)
    ks = [x[4] for x in a]
    assert all(ks.count(k) > 50 for k in (16, 32, 64))


def small_batch(ng, count=10, max_nnz=150_000, seed=12345):
    """The first `count` problems of the batched workload with at most `max_nnz` cells
    (the oracle replays them in seconds)."""
    probs, i = [], 0
    while len(probs) < count:
        spec, dim = ng._abi.SynthSpec(), ctypes.c_int32()
        ng.check(ng.lib().nomad_synth_batch_problem(seed, i, ctypes.byref(spec), ctypes.byref(dim)),
                 "nomad_synth_batch_problem")
        i += 1
        if spec.nnz_train + spec.nnz_test > max_nnz:
            continue
        train, test = ng.synth(spec)
        W0, H0 = ng.reference_init(train.m, train.n, dim.value, 12345, 1)
        probs.append((train, test, dim.value, W0, H0))
    return probs


@pytest.mark.gpu
def test_batch_exact_equals_replay(ng, O, gpu_ok):
    probs = small_batch(ng)
    with ng.Batch(probs, lrate=LR, drate=DR, reg=REG, exact=1) as b:
        st = b.epoch(2)
        st2 = b.epoch(1)  # the pass count continues across graph replays
        got = [b.factors(i) for i in range(len(probs))]
    total = sum(p[0].nnz for p in probs)
    assert st["updates"] == 2 * total and st2["updates"] == total
    assert st2["epochs_done"] == 3
    for (train, test, dim, W0, H0), (Wg, Hg) in zip(probs, got):
        Wo, Ho = W0.copy(), H0.copy()
        O.replay(train.to_csc(), Wo, Ho, 0, 3, LR, DR, REG)
        assert np.array_equal(Wg, Wo) and np.array_equal(Hg, Ho), (train.m, train.n, dim)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "bf16"])
@pytest.mark.parametrize("blocks_per_sm", [1, 4])  # the FMA kernel's two builds
def test_batch_rmse_vs_fp64_oracle(ng, O, gpu_ok, precision, blocks_per_sm):
    probs = small_batch(ng, count=12)
    epochs = 10
    with ng.Batch(probs, lrate=LR, drate=DR, reg=REG, precision=precision, blocks_per_sm=blocks_per_sm) as b:
        b.epoch(epochs)
        _, te = b.rmse()
    for (train, test, dim, W0, H0), r in zip(probs, te):
        Wd, Hd = W0.astype(np.float64), H0.astype(np.float64)
        O.replay(train.to_csc(), Wd, Hd, 0, epochs, LR, DR, REG)
        ref = O.rmse(test.to_csc(), Wd, Hd)
        assert abs(r - ref) <= 0.005 * ref, (train.m, train.n, dim, r, ref)


@pytest.mark.gpu
def test_batch_rmse_matches_single_problem_evaluation(ng, gpu_ok):
    """The per-problem RMSE kernel agrees with the single-problem context's evaluation of
    the same factors (FP64 sums of the same squared errors)."""
    probs = small_batch(ng, count=4)
    with ng.Batch(probs, lrate=LR, drate=DR, reg=REG) as b:
        b.epoch(2)
        tr, te = b.rmse()
        facs = [b.factors(i) for i in range(len(probs))]
    for (train, test, dim, _, _), (W, H), a, c in zip(probs, facs, tr, te):
        with ng.Nomad(train, test, W0=W, H0=H, dim=dim, mode="replay") as nm:
            r_tr, r_te = nm.rmse()
        assert abs(a - r_tr) <= 1e-5 * r_tr and abs(c - r_te) <= 1e-5 * r_te


def bf16_rn(x):
    """float32 values rounded to the nearest bfloat16 (ties to even), as float32."""
    b = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    return (((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16).astype(np.uint32).view(np.float32)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "bf16"])
@pytest.mark.parametrize("parts", [1, 3])
def test_batch_reference_init_on_device(ng, gpu_ok, precision, parts):
    """Rows not given take the reference init, drawn once per stream on the host and
    expanded on the device: every problem's rows equal nomad_reference_init's (rounded to
    bf16 for bf16 storage); given rows are kept as given."""
    probs = small_batch(ng, count=6)
    batch = []
    for i, (train, test, dim, W0, H0) in enumerate(probs):
        W1, H1 = W0 + 0.25, H0 + 0.5  # given rows that differ from the init
        batch.append((train, test, dim, W1 if i == 1 else None, H1 if i in (2, 4) else None))
    seed = 777
    with ng.Batch(batch, lrate=LR, drate=DR, reg=REG, precision=precision, seed=seed, init_parts=parts) as b:
        got = [b.factors(i) for i in range(len(batch))]
    conv = bf16_rn if precision == "bf16" else (lambda x: x)
    for (train, test, dim, Wg, Hg), (W, H) in zip(batch, got):
        Wr, Hr = ng.reference_init(train.m, train.n, dim, seed, parts)
        assert np.array_equal(W, conv(Wg if Wg is not None else Wr)), (train.m, dim)
        assert np.array_equal(H, conv(Hg if Hg is not None else Hr)), (train.n, dim)
