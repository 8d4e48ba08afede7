"""The oracle checked against the reference's own updater.

The reference's Code/nomad/nb_main.cpp, nb_data.cpp and pool.cpp compile unmodified
against single-process stand-ins for TBB, glog, boost::format and MPI
(oracle/Makefile.ref, oracle/refshim/), and oracle/refshim/ref_driver.cpp runs its
updater thread on one rank with one thread: columns round-robin in index order, the
reference's own loader, row init, per-rating update, step schedule and evaluation pass.

* Golden outputs of that build (tests/golden/reference_replay.npz, made by
  tests/golden/make_reference_golden.py) pin the oracle on every machine: the oracle's
  double-precision replay from the reference init reproduces the reference's columns
  and its evaluation sums bit for bit.
* Where the reference tree is present, the same comparison runs live on further cases,
  including the reference's train.dat reader on both header forms and k = 100.
"""
import os
import tempfile

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_replay.npz")


def _golden_cases():
    z = np.load(GOLDEN)
    names = sorted({k.split(".")[0] for k in z.files})
    return z, names


def _oracle_run(O, m, n, dim, tr, te, lrate, drate, reg, seed, epochs):
    W, H = O.init_factors(m, n, dim, seed, 1)
    csc = O.row_major_to_csc(m, n, *tr)
    tcsc = O.row_major_to_csc(m, n, *te)
    err = O.replay(csc, W, H, 0, epochs, lrate, drate, reg)
    return W, H, O.sse(csc, W, H), O.sse(tcsc, W, H), err


@pytest.mark.parametrize("name", ["uniform", "ragged"])
def test_oracle_matches_reference_golden(O, name):
    """Oracle double replay == the reference's updater, bit for bit (columns and the
    evaluation sums), plus its update count and per-column online errors."""
    z, names = _golden_cases()
    assert name in names
    g = lambda k: z[f"{name}.{k}"]  # noqa: E731
    m, n, dim, epochs = int(g("m")), int(g("n")), int(g("dim")), int(g("epochs"))
    tr = (g("train.row_counts"), g("train.cols"), g("train.vals"))
    te = (g("test.row_counts"), g("test.cols"), g("test.vals"))
    W, H, (tsse, tcnt), (esse, ecnt), err = _oracle_run(
        O, m, n, dim, tr, te, float(g("lrate")), float(g("drate")), float(g("reg")), int(g("seed")), epochs)
    assert np.array_equal(H, g("out.H"))
    assert tsse == float(g("out.train_sse")) and tcnt == int(g("out.train_count"))
    assert esse == float(g("out.test_sse")) and ecnt == int(g("out.test_count"))
    assert int(g("out.updates")) == epochs * tr[1].size
    # the reference sums each column's errors over all passes, the oracle each epoch's
    # over all columns: the same terms in another order
    assert np.isclose(err.sum(), g("out.col_err").sum(), rtol=1e-12)


def _live_cases(O):
    """Cases run against the reference build itself (only where the tree is present)."""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    import make_reference_golden as M
    rng = np.random.default_rng(2024)
    m, n = 2000, 400
    cells = np.sort(rng.choice(m * n, 40000, replace=False))
    r, c = np.divmod(cells, n)
    big = dict(m=m, n=n, dim=100, lrate=0.002, drate=0.05, reg=0.05, seed=12345, epochs=2, file_id=1211216,
               r=r, c=c, v=rng.integers(1, 6, r.size).astype(np.float64), test=rng.random(r.size) < 0.1)
    return M, [M.case_uniform(), M.case_ragged(), big]


def test_oracle_matches_reference_live(O):
    """Runs the reference build on the golden cases and a k = 100 case, and compares the
    oracle with it; also checks the reference's row dump (6 significant digits)."""
    if O.reference_tree() is None:
        pytest.skip("the reference tree is not on this machine (the golden test pins the oracle)")
    O.build_ref()
    M, cases = _live_cases(O)
    for cs in cases:
        d, res = M.run_reference(cs, rows_prefix="rows")
        tr, te = M.split(cs)
        W, H, (tsse, tcnt), (esse, ecnt), _ = _oracle_run(
            O, cs["m"], cs["n"], cs["dim"], tr, te, cs["lrate"], cs["drate"], cs["reg"], cs["seed"], cs["epochs"])
        assert np.array_equal(H, res["H"]), cs["dim"]
        assert (tsse, tcnt, esse, ecnt) == (res["train_sse"], res["train_count"], res["test_sse"], res["test_count"])
        rows = np.loadtxt(os.path.join(d, "rows0"), delimiter=",", usecols=range(1, cs["dim"] + 2), ndmin=2)
        idx = rows[:, 0].astype(np.int64)
        assert np.array_equal(idx, np.arange(cs["m"]))
        np.testing.assert_allclose(rows[:, 1:], W, rtol=5e-6, atol=1e-12)


def test_reference_rejects_what_it_cannot_read(O):
    """A missing test.dat is a status from the driver, not a crash."""
    if O.reference_tree() is None:
        pytest.skip("the reference tree is not on this machine")
    d = tempfile.mkdtemp()
    O.write_matrix(os.path.join(d, "train.dat"), 3, 2, np.array([1, 0, 1], np.int32),
                   np.array([0, 1], np.int32), np.array([1.0, 2.0]))
    with pytest.raises(RuntimeError):
        O.ref_replay(d, 2, 4, 0.01, 0.1, 0.05, 1, 1)
