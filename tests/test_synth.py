"""Seeded synthetic workloads (no GPU): exact sizes, no repeated cells, disjoint
train/test, deterministic whatever the thread count."""
import numpy as np
import pytest


def cells(A):
    return A.rows().astype(np.int64) * A.n + A.cols


def check_matrix(A):
    assert A.row_counts.sum() == A.nnz
    assert A.cols.min() >= 0 and A.cols.max() < A.n
    # columns ascending inside each row, so no repeated (row, column) cell
    starts = np.concatenate([[0], np.cumsum(A.row_counts)[:-1]])
    d = np.diff(A.cols.astype(np.int64))
    same_row = np.ones(A.nnz - 1, bool)
    same_row[starts[1:][A.row_counts[1:] > 0] - 1] = False
    assert np.all(d[same_row] > 0)


def test_uniform_workload(ng):
    tr, te = ng.synth(ng.synth_spec(1, m=500, n=300, nnz_train=9000, nnz_test=1000))
    assert (tr.nnz, te.nnz) == (9000, 1000)
    check_matrix(tr)
    check_matrix(te)
    assert np.intersect1d(cells(tr), cells(te)).size == 0


def test_degree_workload(ng):
    spec = ng.synth_spec(2, m=3000, n=800, nnz_train=60000, nnz_test=3000)
    tr, te = ng.synth(spec)
    assert (tr.nnz, te.nnz) == (60000, 3000)
    check_matrix(tr)
    check_matrix(te)
    assert np.intersect1d(cells(tr), cells(te)).size == 0
    assert set(np.unique(tr.vals)) <= {1.0, 2.0, 3.0, 4.0, 5.0}
    deg = np.bincount(tr.cols, minlength=tr.n)
    assert deg.max() > 20 * np.median(deg)  # heavy-tailed item degrees


def test_geometric_rows(ng):
    spec = ng.synth_spec(4, m=20000, n=500, nnz_train=1000000, nnz_test=50000)
    tr, te = ng.synth(spec)
    assert tr.nnz == 1000000 and te.nnz == 50000
    check_matrix(tr)
    assert tr.vals.dtype == np.float64 and not np.all(tr.vals == np.round(tr.vals))


@pytest.mark.parametrize("workload", [1, 2])
def test_thread_count_independent(ng, workload):
    kw = dict(m=2000, n=700, nnz_train=40000, nnz_test=2000)
    a = ng.synth(ng.synth_spec(workload, threads=1, **kw))
    b = ng.synth(ng.synth_spec(workload, threads=5, **kw))
    for x, y in zip(a, b):
        assert np.array_equal(x.row_counts, y.row_counts)
        assert np.array_equal(x.cols, y.cols) and np.array_equal(x.vals, y.vals)


def test_seed_changes_data(ng):
    a, _ = ng.synth(ng.synth_spec(1, m=300, n=200, nnz_train=2000, nnz_test=100, seed=1))
    b, _ = ng.synth(ng.synth_spec(1, m=300, n=200, nnz_train=2000, nnz_test=100, seed=2))
    assert not np.array_equal(a.cols, b.cols)


def test_presets(ng):
    s = ng.synth_spec(2)
    assert (s.m, s.n, s.nnz_train, s.nnz_test) == (480189, 17770, 100480507, 1408395)
    s = ng.synth_spec(3)
    assert (s.m, s.n, s.nnz_train, s.nnz_test) == (1000990, 624961, 252800275, 4003960)
    s = ng.synth_spec(4)
    assert (s.m, s.n, s.nnz_train, s.nnz_test) == (50082603, 39780, 2740000000, 30000000)
    with pytest.raises(ng.NomadError):
        ng.synth_spec(9)


def test_impossible_sizes_rejected(ng):
    with pytest.raises(ng.NomadError):
        ng.synth(ng.synth_spec(1, m=10, n=10, nnz_train=90, nnz_test=20))
