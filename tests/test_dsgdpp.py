"""DSGD++ and the bold-driver learning rate (Code/competitor/dsgdpp.cpp,
Code/competitor/sgd-mpi-omp.cpp), one process.

Pins of the oracle (CPU):
  * a pure-Python restatement of glibc's srand/rand (TYPE_3 additive feedback
    generator) reproduces the oracle's DSGD and DSGD++ stratum schedules;
  * a pure-Python float64 restatement of DSGD / DSGD++ (block grid, schedule, reverse
    walk, FIXED and bold-driver rates, calobj_mpi) equals the oracle bit for bit.
GPU parity: exact-order DSGD++ and bold-driver runs equal the oracle bit for bit; the
objective kernel matches the oracle's; resume from a checkpoint keeps the bold
driver's state.
"""
import numpy as np
import pytest

REG = 0.05


class GlibcRand:
    """glibc srand()/rand() (random_r.c, TYPE_3: degree 31, separation 3)."""

    def __init__(self, seed):
        seed &= 0xFFFFFFFF
        if seed == 0:
            seed = 1
        r = [seed]
        for _ in range(30):
            hi, lo = divmod(r[-1], 127773)
            word = 16807 * lo - 2836 * hi
            if word < 0:
                word += 2147483647
            r.append(word)
        self.r = [x & 0xFFFFFFFF for x in r]
        self.f, self.b = 3, 0
        for _ in range(310):
            self.next()

    def next(self):
        self.r[self.f] = (self.r[self.f] + self.r[self.b]) & 0xFFFFFFFF
        out = self.r[self.f] >> 1
        self.f = (self.f + 1) % 31
        self.b = (self.b + 1) % 31
        return out


def random_shuffle(a, g):
    """libstdc++ std::random_shuffle(first, last) with rand()."""
    for i in range(1, len(a)):
        j = g.next() % (i + 1)
        a[i], a[j] = a[j], a[i]


def py_schedule(innerB, it, strategy, variant):
    perm, offset = list(range(innerB)), list(range(innerB))
    if variant == 0:  # persists across iterations (sgd-mpi-omp.cpp)
        for t in range(1, it + 1):
            g = GlibcRand(34586 + t)
            if strategy == 2:
                random_shuffle(perm, g)
                random_shuffle(offset, g)
    elif strategy == 2:  # fresh every iteration (dsgdpp.cpp)
        g = GlibcRand(34586 + it)
        random_shuffle(perm, g)
        random_shuffle(offset, g)
    out = []
    for phase in range(2 if variant == 1 else 1):
        for i in range(innerB):
            cur = [0] * innerB
            for ii in range(innerB):
                cur[perm[ii]] = (ii + offset[i]) % innerB
            out.append([phase * innerB + cur[bi] for bi in range(innerB)])
    return np.array(out, np.int32)


def py_objective(m, n, row_counts, cols, vals, W, H, reg):
    loss, idx = 0.0, 0
    ccnt = [0] * n
    for r in range(m):
        for _ in range(row_counts[r]):
            c = cols[idx]
            dot = 0.0
            for k in reversed(range(len(W[r]))):
                dot += W[r][k] * H[c][k]
            diff = -vals[idx] + dot
            loss += diff * diff
            ccnt[c] += 1
            idx += 1
    norm = lambda x: sum(x[k] * x[k] for k in reversed(range(len(x))))  # noqa: E731
    regs = 0.0
    for r in range(m):
        regs += row_counts[r] * norm(W[r])
    for c in range(n):
        regs += ccnt[c] * norm(H[c])
    return loss + reg * regs


def py_dsgd(m, n, row_counts, cols, vals, W, H, nthreads, iters, lrate, decay, reg, strategy,
            variant, bold):
    """Float64 DSGD (variant 0) / DSGD++ (variant 1) from the reference's loops."""
    innerB = 2 * nthreads
    cb = 2 * innerB if variant == 1 else innerB
    ibm = m // innerB + (1 if m % innerB else 0)
    ibn = n // cb + (1 if n % cb else 0)
    blocks = [[] for _ in range(innerB * cb)]
    idx = 0
    for r in range(m):
        for _ in range(row_counts[r]):
            blocks[(r // ibm) * cb + cols[idx] // ibn].append((r, cols[idx], vals[idx]))
            idx += 1
    lr, old = lrate, None
    if bold:
        old = py_objective(m, n, row_counts, cols, vals, W, H, reg)
    for it in range(1, iters + 1):
        cur = lr if bold else 1.5 * lrate / (1.0 + decay * it ** 1.5)
        for stratum in py_schedule(innerB, it, strategy, variant):
            for bi in range(innerB):
                for (i, j, v) in reversed(blocks[bi * cb + int(stratum[bi])]):
                    Wi, Hj = W[i], H[j]
                    dot = 0.0
                    for k in reversed(range(len(Wi))):
                        dot += Wi[k] * Hj[k]
                    err = dot - v
                    for k in range(len(Wi)):
                        tmp = Wi[k]
                        Wi[k] -= cur * (err * Hj[k] + reg * Wi[k])
                        Hj[k] -= cur * (err * tmp + reg * Hj[k])
        if bold:
            obj = py_objective(m, n, row_counts, cols, vals, W, H, reg)
            lr *= decay if obj > old else 1.05
            old = obj
    return lr, old


def tiny(ng, m=13, n=11, nnz=60, seed=9):
    spec = ng.synth_spec(1, m=m, n=n, nnz_train=nnz, nnz_test=6)
    spec.seed = seed
    return ng.synth(spec)


@pytest.mark.parametrize("innerB,strategy", [(4, 0), (6, 2), (5, 2)])
def test_schedules_match_glibc_restatement(O, innerB, strategy):
    for it in (1, 2, 7):
        assert np.array_equal(O.dsgd_schedule(innerB, it, strategy),
                              py_schedule(innerB, it, strategy, 0))
        s = O.dsgdpp_schedule(innerB, it, strategy)
        assert np.array_equal(s, py_schedule(innerB, it, strategy, 1))
        for phase in range(2):
            half = s[phase * innerB:(phase + 1) * innerB]
            want = list(range(phase * innerB, (phase + 1) * innerB))
            for row in half:
                assert sorted(row) == want  # a stratum: disjoint column blocks
            for bi in range(innerB):
                assert sorted(half[:, bi]) == want  # every block once per pass


def test_glibc_restatement_known_answer():
    """glibc rand() after srand(1) begins 1804289383, 846930886, 1681692777."""
    g = GlibcRand(1)
    assert [g.next() for _ in range(3)] == [1804289383, 846930886, 1681692777]


@pytest.mark.parametrize("variant,strategy,bold", [(0, 0, 0), (0, 2, 1), (1, 0, 0), (1, 2, 0),
                                                   (1, 2, 1), (1, 0, 1)])
def test_oracle_matches_python_restatement(ng, O, variant, strategy, bold):
    train, _ = tiny(ng)
    dim, nthreads, iters = 3, 2, 3
    lrate = 0.05 if bold else 0.02
    W0, H0 = ng.reference_init(train.m, train.n, dim, 3, 1)
    Wo, Ho = W0.astype(np.float64), H0.astype(np.float64)
    state = np.array([lrate, -1.0])
    O.dsgd2(train.m, train.n, train.row_counts, train.cols, train.vals, Wo, Ho, nthreads, 1,
            iters, lrate, 0.5, REG, strategy, variant, bold, state if bold else None)
    Wp = [list(map(float, r)) for r in W0.astype(np.float64)]
    Hp = [list(map(float, r)) for r in H0.astype(np.float64)]
    lr, obj = py_dsgd(train.m, train.n, list(train.row_counts), list(train.cols),
                      list(map(float, train.vals)), Wp, Hp, nthreads, iters, lrate, 0.5, REG,
                      strategy, variant, bold)
    assert np.array_equal(Wo, np.array(Wp)) and np.array_equal(Ho, np.array(Hp))
    if bold:
        assert state[0] == lr and state[1] == obj


def test_objective_matches_python_restatement(ng, O):
    train, _ = tiny(ng, m=17, n=9, nnz=70)
    rng = np.random.default_rng(4)
    W = rng.standard_normal((train.m, 5))
    H = rng.standard_normal((train.n, 5))
    got = O.objective(train.m, train.n, train.row_counts, train.cols, train.vals, W, H, 0.3)
    want = py_objective(train.m, train.n, list(train.row_counts), list(train.cols),
                        list(map(float, train.vals)), W.tolist(), H.tolist(), 0.3)
    assert got == want


def test_bold_driver_rule_in_oracle(ng, O):
    """Pass by pass, the rate is multiplied by 1.05 when the objective fell and by the
    decay when it rose; a rate of 0.8 on this problem does both."""
    train, _ = _problem(ng, seed=7)
    W, H = ng.reference_init(train.m, train.n, 16, 5, 1)
    state = np.array([0.8, -1.0])
    prev = O.objective(train.m, train.n, train.row_counts, train.cols, train.vals, W, H, REG)
    factors = []
    for it in range(1, 7):
        lr = state[0]
        O.dsgd2(train.m, train.n, train.row_counts, train.cols, train.vals, W, H, 2, it, 1,
                0.8, 0.5, REG, 0, 1, 1, state)
        obj = O.objective(train.m, train.n, train.row_counts, train.cols, train.vals, W, H, REG)
        assert state[1] == obj
        factors.append(0.5 if obj > prev else 1.05)
        assert state[0] == lr * factors[-1]
        prev = obj
    assert 0.5 in factors and 1.05 in factors


def test_bold_driver_needs_dsgd(ng):
    train, test = tiny(ng)
    with pytest.raises(ng.NomadError) as e:
        ng.Nomad(train, test, dim=4, mode="async", lr_strategy="bold")
    assert e.value.status in (-9, -8, -2)  # unsupported (or no device on a CPU host)
    p = ng.default_params(lr_strategy=7)
    with pytest.raises(ng.NomadError) as e:
        ng.Nomad(train, test, params=p)
    assert e.value.status == -1


def _problem(ng, m=500, n=120, nnz=8000, seed=12345):
    spec = ng.synth_spec(1, m=m, n=n, nnz_train=nnz, nnz_test=500)
    spec.seed = seed
    return ng.synth(spec)


def relerr(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-30))


@pytest.mark.gpu
@pytest.mark.parametrize("strategy", [0, 2])
def test_dsgdpp_exact_vs_oracle(ng, O, gpu_ok, strategy):
    train, test = _problem(ng)
    dim, nthreads = 40, 3
    W0, H0 = ng.reference_init(train.m, train.n, dim, 5, 1)
    with ng.Nomad(train, test, W0=W0, H0=H0, dim=dim, lrate=0.01, drate=0.1, reg=REG,
                  mode="dsgdpp", exact=1, dsgd_inner_blocks=2 * nthreads,
                  dsgd_strategy=strategy) as nm:
        st = nm.epoch(3)
        Wg, Hg = nm.factors()
    assert st["updates"] == 3 * train.nnz
    Wo, Ho = W0.copy(), H0.copy()
    O.dsgd2(train.m, train.n, train.row_counts, train.cols, train.vals, Wo, Ho, nthreads, 1, 3,
            0.01, 0.1, REG, strategy, 1)
    assert np.array_equal(Wg, Wo) and np.array_equal(Hg, Ho), (relerr(Wg, Wo), relerr(Hg, Ho))


@pytest.mark.gpu
@pytest.mark.parametrize("mode,variant", [("dsgd", 0), ("dsgdpp", 1)])
def test_bold_driver_exact_vs_oracle(ng, O, gpu_ok, mode, variant):
    """Bit-exact factors and the same learning-rate trajectory, pass by pass; the rate
    both rises (small start) and falls (large start)."""
    train, test = _problem(ng, seed=7)
    dim, nthreads = 16, 2
    W0, H0 = ng.reference_init(train.m, train.n, dim, 5, 1)
    for lrate in (0.005, 0.8):
        Wo, Ho = W0.copy(), H0.copy()
        state = np.array([lrate, -1.0])
        with ng.Nomad(train, test, W0=W0, H0=H0, dim=dim, lrate=lrate, drate=0.5, reg=REG,
                      mode=mode, exact=1, dsgd_inner_blocks=2 * nthreads,
                      lr_strategy="bold") as nm:
            for it in range(1, 7):
                st = nm.epoch(1)
                O.dsgd2(train.m, train.n, train.row_counts, train.cols, train.vals, Wo, Ho,
                        nthreads, it, 1, lrate, 0.5, REG, 0, variant, 1, state)
                Wg, Hg = nm.factors()
                assert np.array_equal(Wg, Wo) and np.array_equal(Hg, Ho), (lrate, it)
                assert st["lrate"] == state[0], (lrate, it, st["lrate"], state[0])
                assert abs(st["objective"] - state[1]) <= 1e-5 * state[1]


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_objective_kernel_vs_oracle(ng, O, gpu_ok, precision):
    train, test = _problem(ng, m=3000, n=700, nnz=90000)
    dim = 48
    rng = np.random.default_rng(3)
    W = (rng.standard_normal((train.m, dim)) * 0.2).astype(np.float32)
    H = (rng.standard_normal((train.n, dim)) * 0.2).astype(np.float32)
    with ng.Nomad(train, test, W0=W, H0=H, dim=dim, mode="dsgd", precision=precision,
                  reg=0.7) as nm:
        got = nm.objective()
        Ws, Hs = nm.factors()  # as stored (bf16: rounded)
    want = O.objective(train.m, train.n, train.row_counts, train.cols, train.vals,
                       Ws.astype(np.float64), Hs.astype(np.float64), 0.7)
    assert abs(got - want) <= 1e-5 * want, (got, want)


@pytest.mark.gpu
def test_dsgdpp_fast_rmse(ng, O, gpu_ok):
    train, test = ng.synth(1)
    dim, LR, DR = 100, 0.001, 0.1
    W0, H0 = ng.reference_init(train.m, train.n, dim, 12345, 1)
    with ng.Nomad(train, test, W0=W0, H0=H0, dim=dim, lrate=LR, drate=DR, reg=REG,
                  mode="dsgdpp", dsgd_inner_blocks=64) as nm:
        nm.epoch(5)
        rm = nm.rmse()[1]
    Wo, Ho = W0.astype(np.float64), H0.astype(np.float64)
    O.dsgd2(train.m, train.n, train.row_counts, train.cols, train.vals, Wo, Ho, 32, 1, 5,
            LR, DR, REG, 0, 1)
    ref = O.rmse(test.to_csc(), Wo, Ho)
    assert abs(rm - ref) <= 0.005 * ref, (rm, ref)


@pytest.mark.gpu
@pytest.mark.parametrize("mode,precision", [("dsgdpp", "fp32"), ("dsgdpp", "bf16"), ("dsgd", "bf16")])
def test_bold_driver_resume_is_bit_exact(ng, gpu_ok, tmp_path, mode, precision):
    train, test = _problem(ng, seed=11)
    kw = dict(dim=16, lrate=0.02, drate=0.5, reg=REG, mode=mode, lr_strategy="bold",
              dsgd_inner_blocks=8, precision=precision)
    with ng.Nomad(train, test, **kw) as a:
        a.epoch(4)
        Wa, Ha = a.factors()
        ra = a.epoch(0)
    p = str(tmp_path / "cp.ckpt")
    with ng.Nomad(train, test, **kw) as b:
        st2 = b.epoch(2)
        b.save_checkpoint(p)
    info = ng.read_checkpoint(p, with_info=True)[2]
    assert info["lrate"] == st2["lrate"] and info["objective"] == st2["objective"]
    with ng.Nomad(train, test, **kw) as c:
        c.load_checkpoint(p)
        st = c.epoch(2)
        Wc, Hc = c.factors()
    assert np.array_equal(Wa, Wc) and np.array_equal(Ha, Hc)
    assert st["epochs_done"] == 4 and ra["epochs_done"] == 4
