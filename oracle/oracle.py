"""ctypes wrapper of the CPU oracle (TEST INFRASTRUCTURE ONLY).

The oracle restates the reference's hot path on the CPU (see nomad_oracle.h for the
reference lines each function follows).  Only tests/, __graft_entry__.smoke() and the
cpu_baseline / reference leg of bench.py import this module; the product never does.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libnomad_oracle.so")
_lib = None

_i32 = ctypes.c_int32
_i64 = ctypes.c_int64
_u64 = ctypes.c_uint64
_dbl = ctypes.c_double
_ptr = ctypes.c_void_p


def build():
    """Compile the oracle with its Makefile (make is a no-op when up to date)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        L.oracle_step_f32.restype = ctypes.c_float
        L.oracle_step_f32.argtypes = [_dbl, _dbl, _i32]
        L.oracle_step_f64.restype = _dbl
        L.oracle_step_f64.argtypes = [_dbl, _dbl, _i32]
        L.oracle_mt19937_64_10000th.restype = _u64
        L.oracle_init_factors.restype = None
        L.oracle_init_factors.argtypes = [_i32, _i32, _i32, _u64, _i32, _ptr, _ptr]
        for name in ("oracle_replay_f32", "oracle_replay_f64"):
            f = getattr(L, name)
            f.restype = ctypes.c_int
            f.argtypes = [_i32, _i32, _i32, _ptr, _ptr, _ptr, _ptr, _ptr, _i32, _i32,
                          _dbl, _dbl, _dbl, _ptr]
        for name in ("oracle_sse_f32", "oracle_sse_f64"):
            f = getattr(L, name)
            f.restype = ctypes.c_int
            f.argtypes = [_i32, _i32, _i32, _ptr, _ptr, _ptr, _ptr, _ptr, _ptr, _ptr]
        for name in ("oracle_async_f32", "oracle_async_f64"):
            f = getattr(L, name)
            f.restype = ctypes.c_int
            f.argtypes = [_i32, _i32, _i32, _ptr, _ptr, _ptr, _ptr, _ptr, _i32, _i32,
                          _dbl, _dbl, _dbl, _dbl, _u64, _ptr, _ptr, _ptr]
        for name in ("oracle_dsgd_f32", "oracle_dsgd_f64"):
            f = getattr(L, name)
            f.restype = ctypes.c_int
            f.argtypes = [_i32, _i32, _i32, _i64, _ptr, _ptr, _ptr, _ptr, _ptr, _i32,
                          _i32, _i32, _dbl, _dbl, _dbl, _i32]
        for name in ("oracle_dsgd2_f32", "oracle_dsgd2_f64"):
            f = getattr(L, name)
            f.restype = ctypes.c_int
            f.argtypes = [_i32, _i32, _i32, _i64, _ptr, _ptr, _ptr, _ptr, _ptr, _i32,
                          _i32, _i32, _dbl, _dbl, _dbl, _i32, _i32, _i32, _ptr]
        for name in ("oracle_objective_f32", "oracle_objective_f64"):
            f = getattr(L, name)
            f.restype = ctypes.c_int
            f.argtypes = [_i32, _i32, _i32, _i64, _ptr, _ptr, _ptr, _ptr, _ptr, _dbl, _ptr]
        L.oracle_dsgdpp_schedule.restype = ctypes.c_int
        L.oracle_dsgdpp_schedule.argtypes = [_i32, _i32, _i32, _ptr]
        L.oracle_dsgd_schedule.restype = ctypes.c_int
        L.oracle_dsgd_schedule.argtypes = [_i32, _i32, _i32, _ptr]
        L.oracle_row_major_to_csc.restype = ctypes.c_int
        L.oracle_row_major_to_csc.argtypes = [_i32, _i32, _i64, _ptr, _ptr, _ptr, _ptr,
                                              _ptr, _ptr]
        L.oracle_read_header.restype = ctypes.c_int
        L.oracle_read_header.argtypes = [ctypes.c_char_p, _ptr, _ptr, _ptr, _ptr]
        L.oracle_read_matrix.restype = ctypes.c_int
        L.oracle_read_matrix.argtypes = [ctypes.c_char_p, _ptr, _ptr, _ptr]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data if a is not None else None


def _check(rc, what):
    if rc != 0:
        raise RuntimeError(f"{what} failed with status {rc}")


def mt19937_64_10000th():
    return int(lib().oracle_mt19937_64_10000th())


def step(lrate, drate, cnt, dtype=np.float32):
    if np.dtype(dtype) == np.float32:
        return np.float32(lib().oracle_step_f32(lrate, drate, cnt))
    return np.float64(lib().oracle_step_f64(lrate, drate, cnt))


def init_factors(m, n, dim, seed, nthreads=1):
    """Reference init (nb_main.cpp:450-455, :70-98) in double."""
    W = np.empty((m, dim), np.float64)
    H = np.empty((n, dim), np.float64)
    lib().oracle_init_factors(m, n, dim, seed, nthreads, _p(W), _p(H))
    return W, H


def row_major_to_csc(m, n, row_counts, cols, vals):
    row_counts = np.ascontiguousarray(row_counts, np.int32)
    cols = np.ascontiguousarray(cols, np.int32)
    vals = np.ascontiguousarray(vals, np.float64)
    nnz = cols.size
    col_ptr = np.empty(n + 1, np.int64)
    row_idx = np.empty(nnz, np.int32)
    cv = np.empty(nnz, np.float64)
    _check(lib().oracle_row_major_to_csc(m, n, nnz, _p(row_counts), _p(cols), _p(vals),
                                         _p(col_ptr), _p(row_idx), _p(cv)),
           "row_major_to_csc")
    return col_ptr, row_idx, cv


def replay(csc, W, H, first_epoch, n_epochs, lrate, drate, reg):
    """In-place replay on W, H (float32 -> nomad_float, float64 -> nomad_double)."""
    col_ptr, row_idx, vals = csc
    m, dim = W.shape
    n = H.shape[0]
    assert W.flags.c_contiguous and H.flags.c_contiguous and W.dtype == H.dtype
    err = np.zeros(max(n_epochs, 1), np.float64)
    f = lib().oracle_replay_f32 if W.dtype == np.float32 else lib().oracle_replay_f64
    _check(f(m, n, dim, _p(col_ptr), _p(row_idx), _p(vals), _p(W), _p(H), first_epoch,
             n_epochs, lrate, drate, reg, _p(err)), "replay")
    return err[:n_epochs]


def sse(csc, W, H):
    col_ptr, row_idx, vals = csc
    m, dim = W.shape
    n = H.shape[0]
    s = np.zeros(1, np.float64)
    c = np.zeros(1, np.int64)
    f = lib().oracle_sse_f32 if W.dtype == np.float32 else lib().oracle_sse_f64
    _check(f(m, n, dim, _p(col_ptr), _p(row_idx), _p(vals), _p(W), _p(H), _p(s), _p(c)),
           "sse")
    return float(s[0]), int(c[0])


def rmse(csc, W, H):
    s, c = sse(csc, W, H)
    return float(np.sqrt(s / c)) if c else float("nan")


def async_train(csc, W, H, nthreads, n_epochs=0, timeout_sec=0.0, lrate=0.001,
                drate=0.1, reg=1.0, seed=12345):
    col_ptr, row_idx, vals = csc
    m, dim = W.shape
    n = H.shape[0]
    u = np.zeros(1, np.int64)
    fl = np.zeros(1, np.int64)
    t = np.zeros(1, np.float64)
    f = lib().oracle_async_f32 if W.dtype == np.float32 else lib().oracle_async_f64
    _check(f(m, n, dim, _p(col_ptr), _p(row_idx), _p(vals), _p(W), _p(H), nthreads,
             n_epochs, timeout_sec, lrate, drate, reg, seed, _p(u), _p(fl), _p(t)),
           "async")
    return {"updates": int(u[0]), "failures": int(fl[0]), "seconds": float(t[0])}


def dsgd(m, n, row_counts, cols, vals, W, H, nthreads, first_iter, n_iters, lrate,
         decay, reg, stratum_strategy=0):
    row_counts = np.ascontiguousarray(row_counts, np.int32)
    cols = np.ascontiguousarray(cols, np.int32)
    vals = np.ascontiguousarray(vals, np.float64)
    dim = W.shape[1]
    f = lib().oracle_dsgd_f32 if W.dtype == np.float32 else lib().oracle_dsgd_f64
    _check(f(m, n, dim, cols.size, _p(row_counts), _p(cols), _p(vals), _p(W), _p(H),
             nthreads, first_iter, n_iters, lrate, decay, reg, stratum_strategy), "dsgd")


def dsgd2(m, n, row_counts, cols, vals, W, H, nthreads, first_iter, n_iters, lrate, decay, reg,
          stratum_strategy=0, variant=0, lr_strategy=0, lr_state=None):
    """DSGD (variant 0) / DSGD++ (variant 1); lr_strategy 1 = bold driver with
    lr_state = np.array([lrate, objective or -1]) updated in place."""
    row_counts = np.ascontiguousarray(row_counts, np.int32)
    cols = np.ascontiguousarray(cols, np.int32)
    vals = np.ascontiguousarray(vals, np.float64)
    if lr_state is not None:
        assert lr_state.dtype == np.float64 and lr_state.size == 2
    dim = W.shape[1]
    f = lib().oracle_dsgd2_f32 if W.dtype == np.float32 else lib().oracle_dsgd2_f64
    _check(f(m, n, dim, cols.size, _p(row_counts), _p(cols), _p(vals), _p(W), _p(H),
             nthreads, first_iter, n_iters, lrate, decay, reg, stratum_strategy, variant,
             lr_strategy, _p(lr_state) if lr_state is not None else None), "dsgd2")


def objective(m, n, row_counts, cols, vals, W, H, reg):
    row_counts = np.ascontiguousarray(row_counts, np.int32)
    cols = np.ascontiguousarray(cols, np.int32)
    vals = np.ascontiguousarray(vals, np.float64)
    out = np.zeros(1, np.float64)
    f = lib().oracle_objective_f32 if W.dtype == np.float32 else lib().oracle_objective_f64
    _check(f(m, n, W.shape[1], cols.size, _p(row_counts), _p(cols), _p(vals), _p(W), _p(H), reg,
             _p(out)), "objective")
    return float(out[0])


def dsgdpp_schedule(innerB, it, stratum_strategy=0):
    out = np.empty(2 * innerB * innerB, np.int32)
    _check(lib().oracle_dsgdpp_schedule(innerB, it, stratum_strategy, _p(out)),
           "dsgdpp_schedule")
    return out.reshape(2 * innerB, innerB)


def dsgd_schedule(innerB, it, stratum_strategy=0):
    out = np.empty(innerB * innerB, np.int32)
    _check(lib().oracle_dsgd_schedule(innerB, it, stratum_strategy, _p(out)),
           "dsgd_schedule")
    return out.reshape(innerB, innerB)


def read_matrix(path):
    fid = np.zeros(1, np.int32)
    m = np.zeros(1, np.int32)
    n = np.zeros(1, np.int32)
    nnz = np.zeros(1, np.int64)
    bpath = os.fsencode(path)
    _check(lib().oracle_read_header(bpath, _p(fid), _p(m), _p(n), _p(nnz)), "read_header")
    rc = np.empty(int(m[0]), np.int32)
    cols = np.empty(int(nnz[0]), np.int32)
    vals = np.empty(int(nnz[0]), np.float64)
    _check(lib().oracle_read_matrix(bpath, _p(rc), _p(cols), _p(vals)), "read_matrix")
    return {"file_id": int(fid[0]), "m": int(m[0]), "n": int(n[0]),
            "row_counts": rc, "cols": cols, "vals": vals}


# ---- the reference's own updater, compiled from the reference tree -------------------
_REF_LIB_PATH = os.path.join(_HERE, "_ref", "libnomad_ref.so")
_ref_lib = None


def reference_tree():
    """Path of the reference tree when it is present on this machine, else None."""
    d = os.environ.get("NOMAD_REFERENCE_DIR", "/root/reference")
    return d if os.path.isfile(os.path.join(d, "Code", "nomad", "nb_main.cpp")) else None


def build_ref():
    """Compile the reference's updater (oracle/Makefile.ref) when the reference tree is
    present; returns False when it is not (the GPU machine has no reference tree)."""
    d = reference_tree()
    if d is None:
        return False
    subprocess.run(["make", "-s", "-C", _HERE, "-f", "Makefile.ref", "REF_DIR=" + d], check=True)
    return True


def ref_lib():
    global _ref_lib
    if _ref_lib is None:
        if not os.path.exists(_REF_LIB_PATH) and not build_ref():
            raise FileNotFoundError("the reference build oracle/_ref/libnomad_ref.so is absent "
                                    "and the reference tree is not on this machine")
        L = ctypes.CDLL(_REF_LIB_PATH)
        L.ref_replay_f64.restype = ctypes.c_int
        L.ref_replay_f64.argtypes = [ctypes.c_char_p, _i32, _dbl, _dbl, _dbl, _u64, _i32,
                                     ctypes.c_char_p, _ptr, _ptr, _ptr, _ptr, _ptr, _ptr, _ptr]
        _ref_lib = L
    return _ref_lib


def ref_replay(data_dir, n, dim, lrate, drate, reg, seed, epochs, rows_prefix=None):
    """The reference's updater thread (nb_main.cpp:415-710, one rank, one thread) run for
    `epochs` passes on <data_dir>/train.dat from the reference init, then its evaluation
    pass on train.dat and test.dat.  Returns H (n x dim, double), each column's online
    error, the training/test squared-error sums and counts, and the update count."""
    H = np.zeros((n, dim), np.float64)
    col_err = np.zeros(n, np.float64)
    s = np.zeros(2, np.float64)
    c = np.zeros(3, np.int64)
    rc = ref_lib().ref_replay_f64(os.fsencode(data_dir), dim, lrate, drate, reg, seed, epochs,
                                  os.fsencode(rows_prefix) if rows_prefix else None,
                                  _p(H), _p(col_err), s[0:].ctypes.data, c[0:].ctypes.data,
                                  s[1:].ctypes.data, c[1:].ctypes.data, c[2:].ctypes.data)
    _check(rc, "ref_replay_f64")
    return {"H": H, "col_err": col_err, "train_sse": float(s[0]), "train_count": int(c[0]),
            "test_sse": float(s[1]), "test_count": int(c[1]), "updates": int(c[2])}


def write_matrix(path, m, n, row_counts, cols, vals, file_id=1211216):
    """train.dat/test.dat writer for the checks (the format nb_data.cpp:19-176 reads:
    id, m, n, nnz (int32, or int64 under id 1015), row counts, column indices, values)."""
    row_counts = np.ascontiguousarray(row_counts, np.int32)
    cols = np.ascontiguousarray(cols, np.int32)
    vals = np.ascontiguousarray(vals, np.float64)
    with open(path, "wb") as f:
        if file_id == 1015:
            np.array([file_id, m, n], np.int32).tofile(f)
            np.array([cols.size], np.int64).tofile(f)
        else:
            np.array([file_id, m, n, cols.size], np.int32).tofile(f)
        row_counts.tofile(f)
        cols.tofile(f)
        vals.tofile(f)


def async_sim(csc, W, H, P, first_epoch, n_epochs, lrate, drate, reg, seed=12345, partition=1,
              visit_cost=3000.0, rating_cost=400.0, hop_cost=3000.0):
    """P-worker asynchronous NOMAD as a deterministic event simulation (in place on W, H;
    float32 or float64); returns each pass's online squared-error sum."""
    col_ptr, row_idx, vals = csc
    m, dim = W.shape
    n = H.shape[0]
    assert W.flags.c_contiguous and H.flags.c_contiguous and W.dtype == H.dtype
    err = np.zeros(max(n_epochs, 1), np.float64)
    L = lib()
    f = L.oracle_async_sim_f32 if W.dtype == np.float32 else L.oracle_async_sim_f64
    f.restype = ctypes.c_int
    f.argtypes = [_i32, _i32, _i32, _ptr, _ptr, _ptr, _ptr, _ptr, _i32, _i32, _i32, _i32,
                  _dbl, _dbl, _dbl, _u64, _dbl, _dbl, _dbl, _ptr]
    _check(f(m, n, dim, _p(col_ptr), _p(row_idx), _p(vals), _p(W), _p(H), P, partition, first_epoch,
             n_epochs, lrate, drate, reg, seed, visit_cost, rating_cost, hop_cost, _p(err)), "async_sim")
    return err[:n_epochs]


# ---- the seeded workloads, without the GPU library ---------------------------------
_WL_LIB_PATH = os.path.join(_HERE, "_build", "libnomad_workload.so")


def workload(workload_id, **overrides):
    """The library's seeded synthetic workload `workload_id` (nomad_synth_preset /
    nomad_synth_generate), generated by the same host code built on its own
    (oracle/_build/libnomad_workload.so), so that a CPU-only run needs no GPU library.
    Returns (train, test), each a dict of m, n, row_counts, cols, vals."""
    from nomad_gb300 import _abi  # ctypes structures only; loads no library
    if not os.path.exists(_WL_LIB_PATH):
        build()
    L = ctypes.CDLL(_WL_LIB_PATH)
    L.nomad_synth_preset.restype = ctypes.c_int
    L.nomad_synth_preset.argtypes = [_i32, ctypes.POINTER(_abi.SynthSpec)]
    L.nomad_synth_generate.restype = ctypes.c_int
    L.nomad_synth_generate.argtypes = [ctypes.POINTER(_abi.SynthSpec), ctypes.POINTER(_abi.IoMatrix),
                                       ctypes.POINTER(_abi.IoMatrix)]
    L.nomad_io_free.restype = None
    L.nomad_io_free.argtypes = [ctypes.POINTER(_abi.IoMatrix)]
    spec = _abi.SynthSpec()
    _check(L.nomad_synth_preset(int(workload_id), ctypes.byref(spec)), "nomad_synth_preset")
    for k, v in overrides.items():
        setattr(spec, k, v)
    tr, te = _abi.IoMatrix(), _abi.IoMatrix()
    _check(L.nomad_synth_generate(ctypes.byref(spec), ctypes.byref(tr), ctypes.byref(te)), "nomad_synth_generate")
    out = []
    for io in (tr, te):
        d = {"m": io.m, "n": io.n,
             "row_counts": np.ctypeslib.as_array(io.row_counts, (io.m,)).copy() if io.m else np.zeros(0, np.int32),
             "cols": np.ctypeslib.as_array(io.cols, (io.nnz,)).copy() if io.nnz else np.zeros(0, np.int32),
             "vals": np.ctypeslib.as_array(io.vals, (io.nnz,)).copy() if io.nnz else np.zeros(0)}
        L.nomad_io_free(ctypes.byref(io))
        out.append(d)
    return out[0], out[1]
