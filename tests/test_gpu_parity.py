"""GPU parity against the CPU oracle, through the C-ABI.

Bars (stated in each test):
  * replay mode: GPU factors equal the oracle's nomad_float replay bit for bit (the
    stated tolerance is 1e-5 relative per element; the kernel meets it with 0);
  * async mode, exact arithmetic, one worker: bit-identical to replay (same schedule);
  * async mode, many workers: per-epoch test RMSE within 0.5% of the FP64 oracle
    (nomad_double replay) at equal epochs;
  * DSGD, exact arithmetic: bit-identical to the oracle's DSGD restatement;
  * evaluation: FP64-accumulated SSE within 1e-6 relative of the oracle's.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LR, DR, REG = 0.001, 0.1, 0.05


def small_problem(ng, m=600, n=150, nnz_train=9000, nnz_test=1000, seed=12345):
    return ng.synth(ng.synth_spec(1, m=m, n=n, nnz_train=nnz_train, nnz_test=nnz_test,
                                  seed=seed))


def relerr(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-30)))


@pytest.mark.parametrize("dim", [32, 100])
def test_replay_bit_exact(ng, O, gpu_ok, dim):
    train, test = small_problem(ng)
    W0, H0 = ng.reference_init(train.m, train.n, dim, 12345, 1)
    with ng.Nomad(train, test, W0=W0, H0=H0, dim=dim, lrate=LR, drate=DR, reg=REG,
                  mode="replay") as nm:
        nm.epoch(2)
        nm.epoch(1)  # continues the pass count across calls
        Wg, Hg = nm.factors()
    Wo, Ho = W0.copy(), H0.copy()
    O.replay(train.to_csc(), Wo, Ho, 0, 3, LR, DR, REG)
    assert np.array_equal(Wg, Wo) and np.array_equal(Hg, Ho), (relerr(Wg, Wo), relerr(Hg, Ho))


@pytest.mark.parametrize("dim", [1, 7, 33, 129, 200])
def test_replay_odd_dims(ng, O, gpu_ok, dim):
    """Row padding (dim not a multiple of 4) and 2 / 4 vectors per lane."""
    train, test = small_problem(ng, m=300, n=80, nnz_train=3000, nnz_test=300)
    W0, H0 = ng.reference_init(train.m, train.n, dim, 7, 3)
    with ng.Nomad(train, test, W0=W0, H0=H0, dim=dim, lrate=LR, drate=DR, reg=REG,
                  mode="replay") as nm:
        nm.epoch(2)
        Wg, Hg = nm.factors()
    Wo, Ho = W0.copy(), H0.copy()
    O.replay(train.to_csc(), Wo, Ho, 0, 2, LR, DR, REG)
    assert np.array_equal(Wg, Wo) and np.array_equal(Hg, Ho), (relerr(Wg, Wo), relerr(Hg, Ho))


def test_replay_workload1_per_element(ng, O, gpu_ok):
    """The 10,000 x 2,000 workload, k = 100: per-element relative error <= 1e-5."""
    train, test = ng.synth(1)
    dim = 100
    W0, H0 = ng.reference_init(train.m, train.n, dim, 12345, 1)
    with ng.Nomad(train, test, W0=W0, H0=H0, dim=dim, lrate=LR, drate=DR, reg=REG,
                  mode="replay") as nm:
        nm.epoch(2)
        Wg, Hg = nm.factors()
    Wo, Ho = W0.copy(), H0.copy()
    O.replay(train.to_csc(), Wo, Ho, 0, 2, LR, DR, REG)
    assert relerr(Wg, Wo) <= 1e-5 and relerr(Hg, Ho) <= 1e-5


def test_async_one_worker_exact_equals_replay(ng, O, gpu_ok):
    """One worker: the queue is FIFO in column order, so async == replay exactly."""
    train, test = small_problem(ng)
    dim = 32
    W0, H0 = ng.reference_init(train.m, train.n, dim, 12345, 1)
    with ng.Nomad(train, test, W0=W0, H0=H0, dim=dim, lrate=LR, drate=DR, reg=REG,
                  mode="async", workers=1, exact=1) as nm:
        st = nm.epoch(3)
        Wg, Hg = nm.factors()
    assert st["updates"] == 3 * train.nnz
    Wo, Ho = W0.copy(), H0.copy()
    O.replay(train.to_csc(), Wo, Ho, 0, 3, LR, DR, REG)
    assert np.array_equal(Wg, Wo) and np.array_equal(Hg, Ho), (relerr(Wg, Wo), relerr(Hg, Ho))


@pytest.mark.parametrize("long_visit", [7, 1000])
def test_async_one_worker_close_to_replay(ng, O, gpu_ok, long_visit):
    """The pipelined kernel (FMA arithmetic, blocked 7-rating path for long visits,
    algebraically equal to the reference update) against the nomad_float replay, with
    one worker and no priority queue so the visit order is the replay's.  Tolerance:
    1e-4 absolute per factor element (entries are ~0.1), 1e-5 relative on test RMSE."""
    train, test = small_problem(ng, m=400, n=60, nnz_train=9000, nnz_test=900)
    dim = 32
    W0, H0 = ng.reference_init(train.m, train.n, dim, 12345, 1)
    with ng.Nomad(train, test, W0=W0, H0=H0, dim=dim, lrate=0.01, drate=DR, reg=REG,
                  mode="async", workers=1, long_visit=long_visit,
                  priority_permille=-1) as nm:
        st = nm.epoch(3)
        Wg, Hg = nm.factors()
        rm = nm.rmse()[1]
    assert st["updates"] == 3 * train.nnz
    Wo, Ho = W0.copy(), H0.copy()
    O.replay(train.to_csc(), Wo, Ho, 0, 3, 0.01, DR, REG)
    assert np.max(np.abs(Wg - Wo)) <= 1e-4 and np.max(np.abs(Hg - Ho)) <= 1e-4
    ref = O.rmse(test.to_csc(), Wo, Ho)
    assert abs(rm - ref) <= 1e-5 * ref


@pytest.mark.parametrize("wpb,dim,precision", [(1, 32, "fp32"), (3, 100, "fp32"), (8, 100, "fp32"),
                                               (8, 7, "fp32"), (8, 200, "fp32"), (10, 100, "fp32"),
                                               (8, 100, "bf16"), (3, 7, "bf16"), (8, 200, "bf16"),
                                               (12, 100, "bf16")])
def test_block_visits_close_to_replay(ng, O, gpu_ok, wpb, dim, precision):
    """Every column on the priority route and one thread block of `wpb` warps: each visit
    is a whole column, processed by the block's warps together in blocks of 32 ratings
    (tensor-core Gram -- 3xTF32 for fp32 rows, bf16 products for bf16 rows -- and the
    exact chain algebra), in the replay's FIFO column order.  Tolerance, fp32: 1e-4
    absolute per factor element (entries are ~0.1) and 1e-5 relative on test RMSE; bf16
    (stochastic rounding of every stored value): test RMSE within 0.5% of the replay's."""
    train, test = small_problem(ng, m=400, n=60, nnz_train=9000, nnz_test=900)
    W0, H0 = ng.reference_init(train.m, train.n, dim, 12345, 1)
    with ng.Nomad(train, test, W0=W0, H0=H0, dim=dim, lrate=0.01, drate=DR, reg=REG,
                  mode="async", precision=precision, workers=wpb, warps_per_block=wpb,
                  priority_permille=1) as nm:
        info = nm.info()
        st = nm.epoch(3)
        Wg, Hg = nm.factors()
        rm = nm.rmse()[1]
    assert info["grid_blocks"] == 1
    assert info["priority_tokens"] == info["active_tokens"] == train.n
    assert st["updates"] == 3 * train.nnz and st["hops"] == 3 * train.n
    Wo, Ho = W0.copy(), H0.copy()
    O.replay(train.to_csc(), Wo, Ho, 0, 3, 0.01, DR, REG)
    ref = O.rmse(test.to_csc(), Wo, Ho)
    if precision == "fp32":
        assert np.max(np.abs(Wg - Wo)) <= 1e-4 and np.max(np.abs(Hg - Ho)) <= 1e-4, \
            (np.max(np.abs(Wg - Wo)), np.max(np.abs(Hg - Ho)))
        assert abs(rm - ref) <= 1e-5 * ref
    else:
        assert abs(rm - ref) <= 5e-3 * ref, (rm, ref)


@pytest.mark.parametrize("workers,wpb", [(64, 8), (40, 3)])
def test_block_visits_mixed_counts(ng, gpu_ok, workers, wpb):
    """Priority columns on block routes next to worker routes, several blocks (the last
    one partly filled when workers % wpb != 0): every rating once per epoch."""
    train, test = ng.synth(ng.synth_spec(2, m=3000, n=300, nnz_train=60000, nnz_test=2000,
                                         seed=12345))
    with ng.Nomad(train, test, dim=32, lrate=LR, drate=DR, reg=REG, mode="async",
                  workers=workers, warps_per_block=wpb, priority_permille=100) as nm:
        info = nm.info()
        st = nm.epoch(2)
    assert 0 < info["priority_tokens"] < info["active_tokens"]
    assert info["grid_blocks"] == (workers + wpb - 1) // wpb
    assert st["updates"] == 2 * train.nnz
    assert st["hops"] == 2 * info["segments"]


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_block_visits_mixed_rmse_vs_fp64_oracle(ng, O, gpu_ok, precision):
    """A skewed 20,000 x 1,000 problem (the Netflix shape, scaled down) with its long
    columns on block routes: test RMSE within 0.5% of the FP64 oracle at every epoch."""
    train, test = ng.synth(ng.synth_spec(2, m=20000, n=1000, nnz_train=400000,
                                         nnz_test=20000, seed=12345))
    dim, epochs = 32, 10
    W0, H0 = ng.reference_init(train.m, train.n, dim, 12345, 1)
    gpu = []
    with ng.Nomad(train, test, W0=W0, H0=H0, dim=dim, lrate=LR, drate=DR, reg=REG,
                  mode="async", precision=precision, workers=256, warps_per_block=8) as nm:
        assert 0 < nm.info()["priority_tokens"] < nm.info()["active_tokens"]
        for _ in range(epochs):
            nm.epoch(1)
            gpu.append(nm.rmse()[1])
    csc, tcsc = train.to_csc(), test.to_csc()
    Wd, Hd = W0.astype(np.float64), H0.astype(np.float64)
    ref = []
    for e in range(epochs):
        O.replay(csc, Wd, Hd, e, 1, LR, DR, REG)
        ref.append(O.rmse(tcsc, Wd, Hd))
    gap = np.abs(np.array(gpu) - np.array(ref)) / np.array(ref)
    assert gap.max() <= 0.005, (gap.max(), gpu[-1], ref[-1])


@pytest.mark.parametrize("workers", [0, 7, 64])
def test_async_counts(ng, gpu_ok, workers):
    """Every rating is visited once per epoch (u=); one hop per (worker, column) visit."""
    train, test = small_problem(ng)
    with ng.Nomad(train, test, dim=32, lrate=LR, drate=DR, reg=REG, mode="async",
                  workers=workers) as nm:
        info = nm.info()
        st = nm.epoch(2)
        st2 = nm.epoch(1)
    assert st["updates"] == 2 * train.nnz
    assert st["hops"] == 2 * info["segments"]
    assert st2["updates"] == train.nnz and st2["epochs_done"] == 3
    if workers:
        assert info["workers"] == workers


@pytest.mark.parametrize("precision,workers", [("fp32", 0), ("bf16", 0), ("fp32", 8),
                                               ("bf16", 8)])
def test_async_rmse_vs_fp64_oracle(ng, O, gpu_ok, precision, workers):
    """10,000 x 2,000 workload, 20 epochs: test RMSE within 0.5% of the FP64 oracle
    (nomad_double replay) at every epoch.  With 8 workers the visits hold ~22 ratings,
    so most of them run the blocked path."""
    train, test = ng.synth(1)
    dim, epochs = 100, 20
    W0, H0 = ng.reference_init(train.m, train.n, dim, 12345, 1)
    gpu = []
    with ng.Nomad(train, test, W0=W0, H0=H0, dim=dim, lrate=LR, drate=DR, reg=REG,
                  mode="async", precision=precision, workers=workers) as nm:
        for _ in range(epochs):
            nm.epoch(1)
            gpu.append(nm.rmse()[1])
    csc, tcsc = train.to_csc(), test.to_csc()
    Wd, Hd = W0.astype(np.float64), H0.astype(np.float64)
    ref = []
    for e in range(epochs):
        O.replay(csc, Wd, Hd, e, 1, LR, DR, REG)
        ref.append(O.rmse(tcsc, Wd, Hd))
    gap = np.abs(np.array(gpu) - np.array(ref)) / np.array(ref)
    assert gap.max() <= 0.005, (gap.max(), gpu[-1], ref[-1])


def test_sse_kernel_vs_oracle(ng, O, gpu_ok):
    train, test = small_problem(ng, m=2000, n=500, nnz_train=60000, nnz_test=6000)
    dim = 100
    rng = np.random.default_rng(3)
    W = rng.standard_normal((train.m, dim)).astype(np.float32) * 0.1
    H = rng.standard_normal((train.n, dim)).astype(np.float32) * 0.1
    with ng.Nomad(train, test, W0=W, H0=H, dim=dim, mode="async") as nm:
        s_tr, c_tr, s_te, c_te = nm.sse()
    o_tr, oc_tr = O.sse(train.to_csc(), W.astype(np.float64), H.astype(np.float64))
    o_te, oc_te = O.sse(test.to_csc(), W.astype(np.float64), H.astype(np.float64))
    assert (c_tr, c_te) == (oc_tr, oc_te) == (train.nnz, test.nnz)
    assert abs(s_tr - o_tr) <= 1e-6 * o_tr and abs(s_te - o_te) <= 1e-6 * o_te


@pytest.mark.parametrize("strategy", [0, 2])
def test_dsgd_exact_vs_oracle(ng, O, gpu_ok, strategy):
    train, test = small_problem(ng, m=500, n=120, nnz_train=8000, nnz_test=500)
    dim, nthreads = 40, 3
    W0, H0 = ng.reference_init(train.m, train.n, dim, 5, 1)
    with ng.Nomad(train, test, W0=W0, H0=H0, dim=dim, lrate=0.01, drate=0.1, reg=REG,
                  mode="dsgd", exact=1, dsgd_inner_blocks=2 * nthreads,
                  dsgd_strategy=strategy) as nm:
        st = nm.epoch(3)
        Wg, Hg = nm.factors()
    assert st["updates"] == 3 * train.nnz
    Wo, Ho = W0.copy(), H0.copy()
    O.dsgd(train.m, train.n, train.row_counts, train.cols, train.vals, Wo, Ho, nthreads, 1, 3,
           0.01, 0.1, REG, strategy)
    assert np.array_equal(Wg, Wo) and np.array_equal(Hg, Ho), (relerr(Wg, Wo), relerr(Hg, Ho))


def test_dsgd_fast_rmse(ng, O, gpu_ok):
    train, test = ng.synth(1)
    dim = 100
    W0, H0 = ng.reference_init(train.m, train.n, dim, 12345, 1)
    with ng.Nomad(train, test, W0=W0, H0=H0, dim=dim, lrate=LR, drate=DR, reg=REG,
                  mode="dsgd", dsgd_inner_blocks=64) as nm:
        nm.epoch(5)
        rm = nm.rmse()[1]
    Wo, Ho = W0.astype(np.float64), H0.astype(np.float64)
    O.dsgd(train.m, train.n, train.row_counts, train.cols, train.vals, Wo, Ho, 32, 1, 5,
           LR, DR, REG, 0)
    ref = O.rmse(test.to_csc(), Wo, Ho)
    assert abs(rm - ref) <= 0.005 * ref, (rm, ref)


def test_timeout_is_a_status_and_context_survives(ng, gpu_ok):
    """A device wait that can never be satisfied (no token is ever enqueued) ends in
    NOMAD_ERR_TIMEOUT after the spin budget instead of hanging; the context stays
    usable, and a context without the hook trains normally."""
    train, test = small_problem(ng)
    p = ng.default_params(dim=32, lrate=LR, drate=DR, reg=REG, mode="async",
                          spin_budget_ms=200, debug_flags=1)
    with ng.Nomad(train, test, params=p) as nm:
        for _ in range(2):
            with pytest.raises(ng.NomadError) as ei:
                nm.epoch(1)
            assert ei.value.status == -4
        assert nm.epoch(0)["epochs_done"] == 0
        assert np.isfinite(nm.rmse()[0])
    p.debug_flags = 0
    with ng.Nomad(train, test, params=p) as nm2:
        st = nm2.epoch(1)
        assert st["updates"] == train.nnz


def test_block_visit_join_timeout_is_a_status(ng, gpu_ok):
    """A worker that never joins its thread block's visit of a priority column (test
    hook, debug bit 1) leaves the block's other workers waiting at the join; their
    bounded wait ends in NOMAD_ERR_TIMEOUT after the spin budget, every warp leaves (the
    phase barriers inside a block visit are bounded waits as well), and the context
    stays usable; a context without the hook trains every rating."""
    train, test = ng.synth(ng.synth_spec(2, m=3000, n=300, nnz_train=60000, nnz_test=2000,
                                         seed=12345))
    p = ng.default_params(dim=32, lrate=LR, drate=DR, reg=REG, mode="async", workers=64,
                          warps_per_block=8, priority_permille=100, spin_budget_ms=200,
                          debug_flags=2)
    with ng.Nomad(train, test, params=p) as nm:
        assert nm.info()["priority_tokens"] > 0
        for _ in range(2):
            with pytest.raises(ng.NomadError) as ei:
                nm.epoch(1)
            assert ei.value.status == -4
        assert nm.epoch(0)["epochs_done"] == 0
        assert np.isfinite(nm.rmse()[0])
    p.debug_flags = 0
    with ng.Nomad(train, test, params=p) as nm2:
        st = nm2.epoch(2)
        assert st["updates"] == 2 * train.nnz


def test_factor_roundtrip(ng, gpu_ok):
    train, test = small_problem(ng)
    rng = np.random.default_rng(0)
    W = rng.standard_normal((train.m, 30)).astype(np.float32)
    H = rng.standard_normal((train.n, 30)).astype(np.float32)
    with ng.Nomad(train, test, dim=30, mode="async") as nm:
        nm.set_factors(W, H)
        W2, H2 = nm.factors()
    assert np.array_equal(W, W2) and np.array_equal(H, H2)
    with ng.Nomad(train, test, dim=30, mode="async", precision="bf16") as nm:
        nm.set_factors(W, H)
        W3, _ = nm.factors()
    assert np.max(np.abs(W3 - W) / np.maximum(np.abs(W), 1e-6)) <= 2 ** -8


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_async_block_size_and_wide_rows(ng, gpu_ok, precision):
    """The pipelined kernel is compiled for 10 compute warps per block with fp32 rows and
    12 with bf16 rows (plus the pop and push warps); a request for more is capped, and
    rows of 512 values (where block visits may not fit shared memory beside the warps'
    staging rings and are then switched off) still train every rating once per epoch."""
    train, test = small_problem(ng, m=3000, n=300, nnz_train=60000, nnz_test=2000)
    cap = 10 if precision == "fp32" else 12
    with ng.Nomad(train, test, dim=32, lrate=LR, drate=DR, reg=REG, mode="async", precision=precision,
                  warps_per_block=14) as nm:
        info = nm.info()
        st = nm.epoch(2)
    assert info["block_threads"] == (cap + 2) * 32
    assert (info["grid_blocks"] - 1) * cap < info["workers"] <= info["grid_blocks"] * cap
    assert st["updates"] == 2 * train.nnz
    rm = []
    with ng.Nomad(train, test, dim=512, lrate=LR, drate=DR, reg=REG, mode="async", precision=precision) as nm:
        for _ in range(3):
            st = nm.epoch(1)
            assert st["updates"] == train.nnz
            rm.append(nm.rmse()[1])
    assert all(np.isfinite(rm)) and rm[-1] < rm[0], rm
