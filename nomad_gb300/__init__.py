"""nomad_gb300 -- NOMAD asynchronous SGD matrix completion on one GB300 (sm_103a).

Python face of libnomad_gpu.so.  The library's C-ABI (include/nomad_gpu.h,
include/nomad_io.h) is the product; this module wraps it with numpy arrays:

    train, test = nomad_gb300.synth(1)                 # or RatingMatrix.read(path)
    with nomad_gb300.Nomad(train, test, dim=100, lrate=0.001, drate=0.1, reg=0.05) as nm:
        stats = nm.epoch(1)
        train_rmse, test_rmse = nm.rmse()

Every call goes to the CUDA library; there is no CPU fallback.
"""
import ctypes
import os

import numpy as np

from . import _abi
from ._abi import NomadError, check, lib  # noqa: F401

MODES = {"async": _abi.MODE_ASYNC, "dsgd": _abi.MODE_DSGD, "replay": _abi.MODE_REPLAY,
         "dsgdpp": _abi.MODE_DSGDPP}
LR_STRATEGIES = {"fixed": _abi.LR_FIXED, "bold": _abi.LR_BOLD_DRIVER}
PRECISIONS = {"fp32": _abi.PREC_FP32, "bf16": _abi.PREC_BF16_SR}
INITS = {"reference": _abi.INIT_REFERENCE, "hash": _abi.INIT_HASH}


def _ptr(a):
    return None if a is None else a.ctypes.data


class _Owned:
    """Keeps library-owned arrays of an nomad_io_matrix alive; frees them on collection."""

    def __init__(self, io):
        self.io = io

    def __del__(self):
        try:
            lib().nomad_io_free(ctypes.byref(self.io))
        except Exception:  # interpreter shutdown
            pass


def _wrap(ptr, count, ctype, dtype, owner):
    if count == 0:
        return np.zeros(0, dtype)
    arr_t = ctype * count
    buf = arr_t.from_address(ctypes.addressof(ptr.contents))
    buf._owner = owner
    return np.frombuffer(buf, dtype=dtype)


class RatingMatrix:
    """A rating set in the train.dat row-major layout: row_counts[m], cols[nnz], vals[nnz]."""

    def __init__(self, m, n, row_counts, cols, vals, file_id=0):
        self.m, self.n = int(m), int(n)
        self.row_counts = np.ascontiguousarray(row_counts, np.int32)
        self.cols = np.ascontiguousarray(cols, np.int32)
        self.vals = np.ascontiguousarray(vals, np.float64)
        self.file_id = int(file_id)
        assert self.row_counts.shape == (self.m,)
        assert self.cols.shape == self.vals.shape

    @property
    def nnz(self):
        return int(self.cols.size)

    @classmethod
    def _from_io(cls, io):
        owner = _Owned(io)
        return cls(io.m, io.n,
                   _wrap(io.row_counts, io.m, ctypes.c_int32, np.int32, owner),
                   _wrap(io.cols, io.nnz, ctypes.c_int32, np.int32, owner),
                   _wrap(io.vals, io.nnz, ctypes.c_double, np.float64, owner), io.file_id)

    @classmethod
    def read(cls, path):
        io = _abi.IoMatrix()
        check(lib().nomad_io_read(os.fsencode(path), ctypes.byref(io)), "nomad_io_read")
        return cls._from_io(io)

    def write(self, path, file_id=0):
        check(lib().nomad_io_write(os.fsencode(path), self.m, self.n, self.nnz,
                                   _ptr(self.row_counts), _ptr(self.cols), _ptr(self.vals),
                                   file_id), "nomad_io_write")

    def rows(self):
        """Row index of every entry (COO rows)."""
        return np.repeat(np.arange(self.m, dtype=np.int32), self.row_counts)

    def to_csc(self):
        """(col_ptr int64[n+1], row_idx int32[nnz], vals float64[nnz]), rows ascending."""
        rows = self.rows()
        order = np.lexsort((rows, self.cols))
        col_ptr = np.zeros(self.n + 1, np.int64)
        np.cumsum(np.bincount(self.cols, minlength=self.n), out=col_ptr[1:])
        return col_ptr, rows[order].astype(np.int32), self.vals[order]

    def _c(self):
        return _abi.Matrix(self.nnz, _ptr(self.row_counts), None, _ptr(self.cols),
                           _ptr(self.vals), None)


def read_header(path):
    fid, m, n, nnz = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int64()
    check(lib().nomad_io_read_header(os.fsencode(path), ctypes.byref(fid), ctypes.byref(m),
                                     ctypes.byref(n), ctypes.byref(nnz)), "nomad_io_read_header")
    return {"file_id": fid.value, "m": m.value, "n": n.value, "nnz": nnz.value}


def synth_spec(workload, **overrides):
    spec = _abi.SynthSpec()
    check(lib().nomad_synth_preset(int(workload), ctypes.byref(spec)), "nomad_synth_preset")
    for k, v in overrides.items():
        setattr(spec, k, v)
    return spec


def synth(workload_or_spec, **overrides):
    """Generate (train, test) RatingMatrix for a named workload (1-4) or a SynthSpec."""
    spec = workload_or_spec if isinstance(workload_or_spec, _abi.SynthSpec) else \
        synth_spec(workload_or_spec, **overrides)
    tr, te = _abi.IoMatrix(), _abi.IoMatrix()
    check(lib().nomad_synth_generate(ctypes.byref(spec), ctypes.byref(tr), ctypes.byref(te)),
          "nomad_synth_generate")
    return RatingMatrix._from_io(tr), RatingMatrix._from_io(te)


def synth_batch_problem(index, seed=12345, threads=0):
    """Problem `index` of the batched workload (4,096 problems of uneven shape and rank):
    (train, test, dim).  `threads` generator threads (0: every core); the data does not
    depend on it."""
    spec, dim = _abi.SynthSpec(), ctypes.c_int32()
    check(lib().nomad_synth_batch_problem(int(seed), int(index), ctypes.byref(spec),
                                          ctypes.byref(dim)), "nomad_synth_batch_problem")
    spec.threads = int(threads)
    train, test = synth(spec)
    return train, test, dim.value


def reference_init(m, n, dim, seed=12345, parts=1):
    """The reference's initial factors (float32 W[m,dim], H[n,dim])."""
    W = np.empty((m, dim), np.float32)
    H = np.empty((n, dim), np.float32)
    check(lib().nomad_reference_init(m, n, dim, seed, parts, _ptr(W), _ptr(H)),
          "nomad_reference_init")
    return W, H


def write_factors(path, W, H):
    W = np.ascontiguousarray(W, np.float32)
    H = np.ascontiguousarray(H, np.float32)
    check(lib().nomad_io_write_factors(os.fsencode(path), W.shape[0], H.shape[0], W.shape[1],
                                       _ptr(W), _ptr(H)), "nomad_io_write_factors")


def write_checkpoint(path, W, H, epochs_done, lrate=0.0, objective=-1.0):
    """Checkpoint file of factors W[m,dim], H[n,dim] after `epochs_done` passes, with
    the bold driver's learning rate and last objective (0 and -1: none)."""
    W = np.ascontiguousarray(W, np.float32)
    H = np.ascontiguousarray(H, np.float32)
    info = _abi.CheckpointInfo(W.shape[0], H.shape[0], W.shape[1], epochs_done, lrate, objective)
    check(lib().nomad_io_write_checkpoint(os.fsencode(path), ctypes.byref(info), _ptr(W), _ptr(H)),
          "nomad_io_write_checkpoint")


def read_checkpoint(path, with_info=False):
    """(W, H, epochs_done) from a checkpoint file; with_info: (W, H, info dict)."""
    info = _abi.CheckpointInfo()
    check(lib().nomad_io_read_checkpoint_header(os.fsencode(path), ctypes.byref(info)),
          "nomad_io_read_checkpoint_header")
    W = np.empty((info.m, info.dim), np.float32)
    H = np.empty((info.n, info.dim), np.float32)
    check(lib().nomad_io_read_checkpoint(os.fsencode(path), info.m, info.n, info.dim, _ptr(W),
                                         _ptr(H), ctypes.byref(info)), "nomad_io_read_checkpoint")
    if with_info:
        return W, H, {k: getattr(info, k) for k, _ in _abi.CheckpointInfo._fields_}
    return W, H, info.epochs_done


def default_params(**overrides):
    p = _abi.Params()
    check(lib().nomad_gpu_params_default(ctypes.byref(p)), "nomad_gpu_params_default")
    for k, v in overrides.items():
        if k == "mode":
            v = MODES[v] if isinstance(v, str) else v
        elif k == "precision":
            v = PRECISIONS[v] if isinstance(v, str) else v
        elif k == "init":
            v = INITS[v] if isinstance(v, str) else v
        elif k == "lr_strategy":
            v = LR_STRATEGIES[v] if isinstance(v, str) else v
        setattr(p, k, v)
    return p


def device_ok(device=0):
    return bool(lib().nomad_gpu_device_ok(device))


def autotune(train, test=None, epochs=1, W0=None, H0=None, **kw):
    """Measured choice of the ASYNC kernel's runtime configuration for this problem
    (nomad_gpu_autotune): returns (keyword arguments for Nomad with warps_per_block,
    priority_permille and long_visit set, list of the trials with their ms per epoch)."""
    p = default_params(**kw)
    if test is None:
        test = RatingMatrix(train.m, train.n, np.zeros(train.m, np.int32),
                            np.zeros(0, np.int32), np.zeros(0))
    W0 = None if W0 is None else np.ascontiguousarray(W0, np.float32)
    H0 = None if H0 is None else np.ascontiguousarray(H0, np.float32)
    prob = _abi.Problem(train.m, train.n, train._c(), test._c(), _ptr(W0), _ptr(H0))
    trials = (_abi.TuneTrial * 32)()
    n = ctypes.c_int32()
    check(lib().nomad_gpu_autotune(ctypes.byref(prob), ctypes.byref(p), epochs, trials, 32, ctypes.byref(n)),
          "nomad_gpu_autotune")
    best = dict(kw, warps_per_block=p.warps_per_block, priority_permille=p.priority_permille,
                long_visit=p.long_visit)
    return best, [{k: getattr(t, k) for k, _ in _abi.TuneTrial._fields_} for t in trials[:n.value]]


def _batch_problems(problems):
    """ctypes array of nomad_gpu_batch_problem for (train, test, dim[, W0, H0]) tuples, and
    the arrays it points into (keep them alive while the array is used)."""
    arr = (_abi.BatchProblem * len(problems))()
    keep = []
    for i, prob in enumerate(problems):
        train, test, dim = prob[0], prob[1], int(prob[2])
        W0 = H0 = None
        if len(prob) > 3 and prob[3] is not None:
            W0 = np.ascontiguousarray(prob[3], np.float32)
        if len(prob) > 4 and prob[4] is not None:
            H0 = np.ascontiguousarray(prob[4], np.float32)
        keep += [train, test, W0, H0]
        arr[i] = _abi.BatchProblem(train.m, train.n, dim, 0, train._c(), test._c(), _ptr(W0), _ptr(H0))
    return arr, keep


def batch_autotune(problems, epochs=1, **kw):
    """Measured choice of the batched form's large-problem threshold for these problems
    (nomad_gpu_batch_autotune): returns (keyword arguments for Batch with batch_share set,
    list of the trials with their ms per epoch and large-problem counts)."""
    p = default_params(**kw)
    arr, keep = _batch_problems(problems)
    trials = (_abi.BatchTuneTrial * 16)()
    n = ctypes.c_int32()
    check(lib().nomad_gpu_batch_autotune(arr, len(problems), ctypes.byref(p), epochs, trials, 16,
                                         ctypes.byref(n)), "nomad_gpu_batch_autotune")
    del keep
    best = dict(kw, batch_share=p.batch_share)
    return best, [{k: getattr(t, k) for k, _ in _abi.BatchTuneTrial._fields_ if k != "reserved"}
                  for t in trials[:n.value]]


class Nomad:
    """One training context on the GPU (nomad_gpu_ctx)."""

    def __init__(self, train, test=None, W0=None, H0=None, params=None, **kw):
        self._ctx = ctypes.c_void_p()
        p = params if params is not None else default_params(**kw)
        self.params = p
        if test is None:
            test = RatingMatrix(train.m, train.n, np.zeros(train.m, np.int32),
                                np.zeros(0, np.int32), np.zeros(0))
        self.m, self.n, self.dim = train.m, train.n, p.dim
        W0 = None if W0 is None else np.ascontiguousarray(W0, np.float32)
        H0 = None if H0 is None else np.ascontiguousarray(H0, np.float32)
        if W0 is not None:
            assert W0.shape == (self.m, self.dim)
        if H0 is not None:
            assert H0.shape == (self.n, self.dim)
        prob = _abi.Problem(train.m, train.n, train._c(), test._c(), _ptr(W0), _ptr(H0))
        check(lib().nomad_gpu_init(ctypes.byref(self._ctx), ctypes.byref(prob), ctypes.byref(p)),
              "nomad_gpu_init")

    def epoch(self, n_epochs=1):
        st = _abi.EpochStats()
        check(lib().nomad_gpu_epoch(self._ctx, n_epochs, ctypes.byref(st)), "nomad_gpu_epoch")
        return {k: getattr(st, k) for k, _ in _abi.EpochStats._fields_ if k != "reserved0"}

    def sse(self):
        a, c, b, d = ctypes.c_double(), ctypes.c_int64(), ctypes.c_double(), ctypes.c_int64()
        check(lib().nomad_gpu_sse(self._ctx, ctypes.byref(a), ctypes.byref(c), ctypes.byref(b),
                                  ctypes.byref(d)), "nomad_gpu_sse")
        return a.value, c.value, b.value, d.value

    def rmse(self, train=True):
        """(train RMSE, test RMSE); train=False evaluates the test set only (train is None)."""
        a, b = ctypes.c_double(), ctypes.c_double()
        check(lib().nomad_gpu_rmse(self._ctx, ctypes.byref(a) if train else None, ctypes.byref(b)),
              "nomad_gpu_rmse")
        return (a.value if train else None), b.value

    def factors(self):
        W = np.empty((self.m, self.dim), np.float32)
        H = np.empty((self.n, self.dim), np.float32)
        check(lib().nomad_gpu_get_factors(self._ctx, _ptr(W), _ptr(H)), "nomad_gpu_get_factors")
        return W, H

    def set_factors(self, W=None, H=None):
        W = None if W is None else np.ascontiguousarray(W, np.float32)
        H = None if H is None else np.ascontiguousarray(H, np.float32)
        check(lib().nomad_gpu_set_factors(self._ctx, _ptr(W), _ptr(H)), "nomad_gpu_set_factors")

    def objective(self):
        """calobj_mpi of the current factors: SSE + reg * weighted squared norms."""
        o = ctypes.c_double()
        check(lib().nomad_gpu_objective(self._ctx, ctypes.byref(o)), "nomad_gpu_objective")
        return o.value

    def set_epochs_done(self, epochs_done):
        check(lib().nomad_gpu_set_epochs_done(self._ctx, epochs_done), "nomad_gpu_set_epochs_done")

    def save_checkpoint(self, path):
        check(lib().nomad_gpu_save_checkpoint(self._ctx, os.fsencode(path)),
              "nomad_gpu_save_checkpoint")

    def load_checkpoint(self, path):
        check(lib().nomad_gpu_load_checkpoint(self._ctx, os.fsencode(path)),
              "nomad_gpu_load_checkpoint")

    def token_finish_times(self):
        """Seconds from the last ASYNC epoch launch's start to each token's last pass."""
        t = np.zeros(self.n, np.float64)
        check(lib().nomad_gpu_token_finish_times(self._ctx, _ptr(t)),
              "nomad_gpu_token_finish_times")
        return t

    def info(self):
        i = _abi.Info()
        check(lib().nomad_gpu_get_info(self._ctx, ctypes.byref(i)), "nomad_gpu_get_info")
        return {k: getattr(i, k) for k, _ in _abi.Info._fields_}

    def close(self):
        if self._ctx:
            lib().nomad_gpu_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Many independent problems trained together (nomad_gpu_batch): one graph-captured
    persistent launch per epoch; each problem runs the one-worker schedule.

        problems = [ng.synth_batch_problem(i) for i in range(64)]   # (train, test, dim)
        with ng.Batch(problems, lrate=0.002, drate=0.1, reg=0.05) as b:
            b.epoch(30)
            train_rmse, test_rmse = b.rmse()
    """

    def __init__(self, problems, params=None, **kw):
        self._b = ctypes.c_void_p()
        p = params if params is not None else default_params(**kw)
        self.params = p
        self.shapes = [(prob[0].m, prob[0].n, int(prob[2])) for prob in problems]
        arr, self._keep = _batch_problems(problems)
        check(lib().nomad_gpu_batch_init(ctypes.byref(self._b), arr, len(problems), ctypes.byref(p)),
              "nomad_gpu_batch_init")
        self._keep = None  # the library copied the host arrays

    @property
    def count(self):
        return len(self.shapes)

    def epoch(self, n_epochs=1):
        st = _abi.EpochStats()
        check(lib().nomad_gpu_batch_epoch(self._b, n_epochs, ctypes.byref(st)), "nomad_gpu_batch_epoch")
        return {k: getattr(st, k) for k, _ in _abi.EpochStats._fields_ if k != "reserved0"}

    def rmse(self):
        tr = np.zeros(self.count, np.float64)
        te = np.zeros(self.count, np.float64)
        check(lib().nomad_gpu_batch_rmse(self._b, _ptr(tr), _ptr(te)), "nomad_gpu_batch_rmse")
        return tr, te

    def factors(self, problem):
        m, n, dim = self.shapes[problem]
        W = np.empty((m, dim), np.float32)
        H = np.empty((n, dim), np.float32)
        check(lib().nomad_gpu_batch_get_factors(self._b, int(problem), _ptr(W), _ptr(H)),
              "nomad_gpu_batch_get_factors")
        return W, H

    def close(self):
        if self._b:
            lib().nomad_gpu_batch_destroy(self._b)
            self._b = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
