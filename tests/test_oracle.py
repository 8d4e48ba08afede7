"""Pins of the CPU oracle (no GPU).

The reference ships no tests or golden vectors, so the oracle is pinned by:
  * the C++ standard's known answer for std::mt19937_64 (the init RNG);
  * hand-computed updates: an independent numpy restatement of the per-rating update
    of Code/nomad/nb_main.cpp:520-542, evaluated operation by operation in float32
    and float64, must equal the oracle bit for bit;
  * committed golden vectors (tests/golden/, made by tests/golden/make_golden.py);
  * internal consistency: async with one thread == replay, DSGD schedule structure.
"""
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_mt19937_64_known_answer(O):
    # ISO C++ [rand.predef]: the 10000th consecutive invocation of a default-constructed
    # mt19937_64 produces 9981545732273789042.
    assert O.mt19937_64_10000th() == 9981545732273789042


def test_step_size_formula(O):
    for lr, dr in [(0.001, 0.1), (0.002, 0.05), (0.008, 0.01), (0.0005, 0.0)]:
        for cnt in [0, 1, 5, 37]:
            # nb_main.cpp:514-515 in double
            ref = lr * 1.5 / (1.0 + dr * (cnt + 1) ** 1.5)
            assert O.step(lr, dr, cnt, np.float64) == pytest.approx(ref, rel=1e-15)
            # float form: lrate/drate held in float, expression in double, result float
            lf, df = float(np.float32(lr)), float(np.float32(dr))
            assert O.step(lr, dr, cnt, np.float32) == np.float32(lf * 1.5 / (1.0 + df * (cnt + 1) ** 1.5))


def _numpy_visit(col, W, rows, vals, step, lam, dt):
    """Independent restatement of one column visit, one rounded operation at a time."""
    col = col.astype(dt)
    for r, v in zip(rows, vals):
        row = W[r]
        cur = dt(-dt(v))
        for i in range(col.size):
            cur = dt(cur + dt(col[i] * row[i]))
        for i in range(col.size):
            tmp = row[i]
            row[i] = dt(row[i] - dt(step * dt(dt(cur * col[i]) + dt(lam * tmp))))
            col[i] = dt(col[i] - dt(step * dt(dt(cur * tmp) + dt(lam * col[i]))))
    return col


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_hand_computed_updates(O, dt):
    """Three ratings in two columns, two epochs, against the numpy restatement."""
    m, n, dim = 3, 2, 5
    rng = np.random.default_rng(11)
    W0 = rng.uniform(0, 0.4, (m, dim)).astype(dt)
    H0 = rng.uniform(0, 0.4, (n, dim)).astype(dt)
    # column 0: rows 0, 2 ; column 1: row 1
    col_ptr = np.array([0, 2, 3], np.int64)
    row_idx = np.array([0, 2, 1], np.int32)
    vals = np.array([1.5, -0.25, 3.0])
    lr, dr, reg = 0.01, 0.1, 0.05
    W, H = W0.copy(), H0.copy()
    for ep in range(2):
        step = O.step(lr, dr, ep, dt)
        lam = dt(reg)
        for j in range(n):
            b, e = col_ptr[j], col_ptr[j + 1]
            vv = vals[b:e].astype(dt)
            H[j] = _numpy_visit(H[j], W, row_idx[b:e], vv, step, lam, dt)
    Wo, Ho = W0.copy(), H0.copy()
    O.replay((col_ptr, row_idx, vals), Wo, Ho, 0, 2, lr, dr, reg)
    assert np.array_equal(W, Wo) and np.array_equal(H, Ho)


def test_sse_matches_numpy(O):
    rng = np.random.default_rng(2)
    m, n, dim = 40, 30, 8
    W = rng.standard_normal((m, dim))
    H = rng.standard_normal((n, dim))
    rows = rng.integers(0, m, 200)
    cols = rng.integers(0, n, 200)
    keep = np.unique(rows * n + cols, return_index=True)[1]
    rows, cols = rows[keep], cols[keep]
    vals = rng.standard_normal(rows.size)
    order = np.lexsort((rows, cols))
    col_ptr = np.zeros(n + 1, np.int64)
    np.cumsum(np.bincount(cols, minlength=n), out=col_ptr[1:])
    s, c = O.sse((col_ptr, rows[order].astype(np.int32), vals[order]), W, H)
    ref = np.sum((np.einsum("ij,ij->i", W[rows], H[cols]) - vals) ** 2)
    assert c == rows.size and s == pytest.approx(ref, rel=1e-12)


def test_init_matches_golden(O):
    with open(os.path.join(GOLDEN, "init_seed12345.json")) as f:
        g = json.load(f)
    W, H = O.init_factors(g["m"], g["n"], g["dim"], g["seed"], g["nthreads"])
    assert np.array_equal(W.ravel()[: len(g["W_head"])], np.array(g["W_head"]))
    assert np.array_equal(H.ravel()[: len(g["H_head"])], np.array(g["H_head"]))


def _golden_problem():
    d = np.load(os.path.join(GOLDEN, "replay_small.npz"))
    return d


@pytest.mark.parametrize("kind", ["f32", "f64"])
def test_replay_matches_golden(O, kind):
    d = _golden_problem()
    dt = np.float32 if kind == "f32" else np.float64
    W = d["W0"].astype(dt)
    H = d["H0"].astype(dt)
    O.replay((d["col_ptr"], d["row_idx"], d["vals"]), W, H, 0, int(d["epochs"]),
             float(d["lrate"]), float(d["drate"]), float(d["reg"]))
    assert np.array_equal(W, d["W_" + kind]) and np.array_equal(H, d["H_" + kind])


def test_async_one_thread_equals_replay(O):
    d = _golden_problem()
    for dt in (np.float32, np.float64):
        W1, H1 = d["W0"].astype(dt), d["H0"].astype(dt)
        W2, H2 = W1.copy(), H1.copy()
        csc = (d["col_ptr"], d["row_idx"], d["vals"])
        args = (float(d["lrate"]), float(d["drate"]), float(d["reg"]))
        O.replay(csc, W1, H1, 0, 3, *args)
        st = O.async_train(csc, W2, H2, nthreads=1, n_epochs=3, lrate=args[0], drate=args[1],
                           reg=args[2])
        assert st["updates"] == 3 * d["row_idx"].size
        assert np.array_equal(W1, W2) and np.array_equal(H1, H2)


def test_async_threads_visit_every_rating(O):
    d = _golden_problem()
    W, H = d["W0"].astype(np.float64), d["H0"].astype(np.float64)
    csc = (d["col_ptr"], d["row_idx"], d["vals"])
    st = O.async_train(csc, W, H, nthreads=4, n_epochs=2, lrate=0.001, drate=0.1, reg=0.05)
    assert st["updates"] == 2 * d["row_idx"].size


@pytest.mark.parametrize("innerB,strategy", [(4, 0), (6, 2), (8, 2)])
def test_dsgd_schedule_is_latin(O, innerB, strategy):
    for it in (1, 2, 5):
        s = O.dsgd_schedule(innerB, it, strategy)
        for i in range(innerB):
            assert sorted(s[i]) == list(range(innerB))  # a stratum: disjoint blocks
        for bi in range(innerB):
            assert sorted(s[:, bi]) == list(range(innerB))  # every block once per epoch


def test_dsgd_semi_wor_is_diagonal(O):
    s = O.dsgd_schedule(5, 3, 0)
    for i in range(5):
        assert list(s[i]) == [(bi + i) % 5 for bi in range(5)]


def test_row_major_to_csc(O):
    rc = np.array([2, 0, 3], np.int32)
    cols = np.array([1, 3, 0, 1, 3], np.int32)
    vals = np.arange(5, dtype=np.float64)
    cp, ri, cv = O.row_major_to_csc(3, 4, rc, cols, vals)
    assert list(cp) == [0, 1, 3, 3, 5]
    assert list(ri) == [2, 0, 2, 0, 2]
    assert list(cv) == [2.0, 0.0, 3.0, 1.0, 4.0]
