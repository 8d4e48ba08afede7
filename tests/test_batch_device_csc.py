"""The batched form's CSCs built on the device in one sort of every problem's entries
(nomad_gb300/csrc/csc_device.cu: device_batch_csc, device_batch_segs) against the host
builds (host_layout.cpp: build_csc, and the concatenation and visit bounds of batch.cpp),
through the C-ABI.

Row-major sets (the train.dat layout) take the device build; a batch with any COO set
takes the host build.  params.debug_flags bit 2 makes the library build both and refuse
with NOMAD_ERR_BOUNDS unless the ratings, column pointers, active-column counts and the
large problems' visit bounds are equal entry for entry.  The same problems given both
ways must also train to the same factors bit for bit (exact = 1 runs each problem's
one-worker schedule in CSC order).  A fault the device build finds (a column out of range,
a repeated cell) is named by the host build, problem index and all.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LR, DR, REG = 0.002, 0.1, 0.05


class CooRatings:
    """A rating set handed over as COO (rows given, no row counts)."""

    def __init__(self, ng, r):
        self.m, self.n, self.nnz = r.m, r.n, r.nnz
        self.rows = r.rows()
        self.cols, self.vals = r.cols, r.vals
        self._ng = ng

    def _c(self):
        ng = self._ng
        return ng._abi.Matrix(self.nnz, None, ng._ptr(self.rows), ng._ptr(self.cols), ng._ptr(self.vals), None)


class F32Ratings:
    """A row-major rating set with fp32 values."""

    def __init__(self, ng, r):
        self.m, self.n, self.nnz = r.m, r.n, r.nnz
        self.row_counts, self.cols = r.row_counts, r.cols
        self.vals = r.vals.astype(np.float32)
        self._ng = ng

    def _c(self):
        ng = self._ng
        return ng._abi.Matrix(self.nnz, ng._ptr(self.row_counts), None, ng._ptr(self.cols), None,
                              ng._ptr(self.vals))


class NoRatings:
    """An empty rating set given without arrays."""

    def __init__(self, ng, m, n):
        self.m, self.n, self.nnz = m, n, 0
        self._ng = ng

    def _c(self):
        return self._ng._abi.Matrix(0, None, None, None, None, None)


def uneven_batch(ng, seed=3):
    """Problems of uneven shape, with empty rows and columns, columns not ascending inside
    a row, a problem without test ratings (given without arrays), and two problems large
    enough for the whole-block path when batch_share is 1."""
    rng = np.random.default_rng(seed)
    shapes = [(700, 190, 12000, 900), (300, 120, 4000, 0), (2000, 400, 60000, 3000), (250, 100, 1500, 150),
              (900, 333, 20000, 2000), (200, 100, 800, 80)]
    probs = []
    for i, (m, n, ntr, nte) in enumerate(shapes):
        train, test = ng.synth(ng.synth_spec(1, m=m, n=n, nnz_train=ntr, nnz_test=max(nte, 1), seed=77 + i))
        cols, vals = train.cols.copy(), train.vals.copy()
        start = 0
        for c in train.row_counts:  # columns out of order inside each row
            p = rng.permutation(c)
            cols[start:start + c] = cols[start:start + c][p]
            vals[start:start + c] = vals[start:start + c][p]
            start += c
        pad_m, pad_n = 17 + i, 9 + i  # empty rows and columns at the end
        train = ng.RatingMatrix(m + pad_m, n + pad_n, np.concatenate([train.row_counts, np.zeros(pad_m, np.int32)]),
                                cols, vals)
        if nte:
            test = ng.RatingMatrix(m + pad_m, n + pad_n,
                                   np.concatenate([test.row_counts, np.zeros(pad_m, np.int32)]), test.cols, test.vals)
        else:
            test = NoRatings(ng, m + pad_m, n + pad_n)
        dim = (16, 32, 64)[i % 3]
        W0, H0 = ng.reference_init(train.m, train.n, dim, 12345, 1)
        probs.append((train, test, dim, W0, H0))
    return probs


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_batch_device_csc_equals_host_build(ng, gpu_ok, precision):
    """debug_flags bit 2: the library compares the device build with the host's, the
    large problems' visit bounds included (batch_share 1 puts two problems on blocks)."""
    probs = uneven_batch(ng)
    best, trials = ng.batch_autotune(probs, lrate=LR, drate=DR, reg=REG, precision=precision, batch_share=1,
                                     debug_flags=4)
    assert trials and trials[0]["large_problems"] >= 2
    with ng.Batch(probs, lrate=LR, drate=DR, reg=REG, precision=precision, batch_share=1, debug_flags=4) as b:
        st = b.epoch(2)
        tr, te = b.rmse()
    assert st["updates"] == 2 * sum(p[0].nnz for p in probs)
    assert np.all(np.isfinite(tr)) and te[1] == 0.0 and np.all(te[[0, 2, 3, 4, 5]] > 0)


@pytest.mark.parametrize("values", ["f64", "f32"])
def test_batch_device_csc_trains_like_host_build(ng, gpu_ok, values):
    """The same problems row-major (device build) and with one COO set (host build for the
    whole batch) train to equal factors and equal RMSE."""
    probs = uneven_batch(ng)
    if values == "f32":
        probs = [(F32Ratings(ng, tr), te if isinstance(te, NoRatings) else F32Ratings(ng, te), d, W, H)
                 for tr, te, d, W, H in probs]
    host = list(probs)
    tr0 = probs[3][0]
    host[3] = (CooRatings(ng, tr0 if values == "f64" else ng.RatingMatrix(tr0.m, tr0.n, tr0.row_counts, tr0.cols,
                                                                          tr0.vals.astype(np.float64))),
               *probs[3][1:])
    out = []
    for batch in (probs, host):
        with ng.Batch(batch, lrate=LR, drate=DR, reg=REG, exact=1) as b:
            b.epoch(3)
            out.append(([b.factors(i) for i in range(len(batch))], b.rmse()))
    (fa, (tra, tea)), (fb, (trb, teb)) = out
    for (Wa, Ha), (Wb, Hb) in zip(fa, fb):
        assert np.array_equal(Wa, Wb) and np.array_equal(Ha, Hb)
    assert np.array_equal(tra, trb) and np.array_equal(tea, teb)


def test_batch_column_out_of_range_named(ng, gpu_ok):
    probs = uneven_batch(ng)
    train, test, dim, W0, H0 = probs[4]
    cols = test.cols.copy()
    cols[7] = test.n + 2
    probs[4] = (train, ng.RatingMatrix(test.m, test.n, test.row_counts, cols, test.vals), dim, W0, H0)
    with pytest.raises(Exception, match=rf"problem 4: column index {test.n + 2} out of range \[0, {test.n}\)"):
        ng.Batch(probs, lrate=LR, drate=DR, reg=REG).close()


def test_batch_repeated_cell_named(ng, gpu_ok):
    probs = uneven_batch(ng)
    m, n = 60, 30
    rc = np.full(m, 3, np.int32)
    cols = np.tile(np.array([2, 6, 11], np.int32), m)
    cols[3 * 40 + 2] = 6  # row 40 rates column 6 twice
    train = ng.RatingMatrix(m, n, rc, cols, np.ones(cols.size))
    probs[2] = (train, NoRatings(ng, m, n), 16, None, None)
    with pytest.raises(Exception, match=r"problem 2: repeated \(row, column\) cell in column 6"):
        ng.Batch(probs, lrate=LR, drate=DR, reg=REG).close()
