"""The context's CSC built on the device (nomad_gb300/csrc/csc_device.cu) against the host
build (host_layout.cpp: build_csc), through the C-ABI.

Row-major rating sets -- the train.dat layout -- are sorted into column order on the
device; COO sets (row indices given) are sorted on the host.  The same ratings given both
ways must leave the same CSC: the replay kernel walks it in order, so its factors after
an epoch are equal bit for bit exactly when the two CSCs are.  A repeated (row, column)
cell is refused on either path, and so is a column index out of range (checked on the
device before the sort, on the host path during it).
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


class CooRatings:
    """The same rating set handed over as COO (rows given, no row counts)."""

    def __init__(self, ng, r):
        self.m, self.n, self.nnz = r.m, r.n, r.nnz
        self.rows = r.rows()
        self.cols, self.vals = r.cols, r.vals
        self._ng = ng

    def _c(self):
        ng = self._ng
        return ng._abi.Matrix(self.nnz, None, ng._ptr(self.rows), ng._ptr(self.cols), ng._ptr(self.vals), None)


def shuffled_within_rows(r, seed):
    """A row-major set whose columns are not ascending inside a row (the sort must not
    rely on it) and with empty rows and columns."""
    rng = np.random.default_rng(seed)
    cols, vals = r.cols.copy(), r.vals.copy()
    start = 0
    for c in r.row_counts:
        p = rng.permutation(c)
        cols[start:start + c] = cols[start:start + c][p]
        vals[start:start + c] = vals[start:start + c][p]
        start += c
    return cols, vals


@pytest.mark.parametrize("mode", ["replay", "async"])
def test_device_csc_equals_host_csc(ng, gpu_ok, mode):
    train, test = ng.synth(ng.synth_spec(1, m=700, n=190, nnz_train=12000, nnz_test=900, seed=77))
    cols, vals = shuffled_within_rows(train, 5)
    train = ng.RatingMatrix(train.m + 40, train.n + 25, np.concatenate([train.row_counts, np.zeros(40, np.int32)]),
                            cols, vals)
    test = ng.RatingMatrix(test.m + 40, test.n + 25, np.concatenate([test.row_counts, np.zeros(40, np.int32)]),
                           test.cols, test.vals)
    dim = 24
    W0, H0 = ng.reference_init(train.m, train.n, dim, 12345, 1)
    kw = dict(W0=W0, H0=H0, dim=dim, lrate=0.001, drate=0.1, reg=0.05, mode=mode)
    if mode == "async":
        kw.update(exact=True, workers=1)  # one worker: the deterministic schedule of the CSC order
    out = []
    for tr, te in ((train, test), (CooRatings(ng, train), CooRatings(ng, test))):
        with ng.Nomad(tr, te, **kw) as nm:
            nm.epoch(2)
            out.append((*nm.factors(), nm.rmse()))
    (Wa, Ha, ra), (Wb, Hb, rb) = out
    assert np.array_equal(Wa, Wb) and np.array_equal(Ha, Hb)
    assert ra == rb


@pytest.mark.parametrize("coo", [False, True])
def test_repeated_cell_refused(ng, gpu_ok, coo):
    m, n = 50, 20
    rc = np.full(m, 3, np.int32)
    cols = np.tile(np.array([1, 5, 9], np.int32), m)
    cols[3 * 17 + 2] = 5  # row 17 rates column 5 twice
    train = ng.RatingMatrix(m, n, rc, cols, np.ones(cols.size))
    test = ng.RatingMatrix(m, n, np.zeros(m, np.int32), np.zeros(0, np.int32), np.zeros(0))
    tr = CooRatings(ng, train) if coo else train
    with pytest.raises(Exception, match=r"repeated \(row, column\) cell in column 5"):
        ng.Nomad(tr, test, dim=8, mode="replay").close()


@pytest.mark.parametrize("col", [20, -3])
def test_column_out_of_range_refused(ng, gpu_ok, col):
    m, n = 50, 20
    rc = np.full(m, 3, np.int32)
    cols = np.tile(np.array([1, 5, 9], np.int32), m)
    cols[3 * 31 + 1] = col
    train = ng.RatingMatrix(m, n, rc, cols, np.ones(cols.size))
    test = ng.RatingMatrix(m, n, np.zeros(m, np.int32), np.zeros(0, np.int32), np.zeros(0))
    with pytest.raises(Exception, match=rf"column index {col} out of range \[0, 20\)"):
        ng.Nomad(train, test, dim=8, mode="replay").close()
