"""ctypes binding of libnomad_gpu.so (include/nomad_gpu.h, include/nomad_io.h).

The structures below mirror the C headers field by field.  Loading fails loudly: if
the shared library has not been built there is no fallback of any kind.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libnomad_gpu.so")

c_i32 = ctypes.c_int32
c_i64 = ctypes.c_int64
c_u64 = ctypes.c_uint64
c_dbl = ctypes.c_double
c_vp = ctypes.c_void_p

# status codes (enum nomad_gpu_status)
OK = 0
ERR_INVALID_ARG = -1
ERR_CUDA = -2
ERR_OOM = -3
ERR_TIMEOUT = -4
ERR_BOUNDS = -5
ERR_IO = -6
ERR_FORMAT = -7
ERR_NO_DEVICE = -8
ERR_UNSUPPORTED = -9

MODE_ASYNC, MODE_DSGD, MODE_REPLAY, MODE_DSGDPP = 0, 1, 2, 3
LR_FIXED, LR_BOLD_DRIVER = 0, 1
PREC_FP32, PREC_BF16_SR = 0, 1
INIT_REFERENCE, INIT_HASH = 0, 1
FILE_ID_INT, FILE_ID_LONG = 1211216, 1015
SYNTH_UNIFORM, SYNTH_DEGREES = 0, 1
LAW_UNIFORM, LAW_ZIPF, LAW_GEOMETRIC = 0, 1, 2
NOALLOC_MAX_BLOCKS = 2048


class Params(ctypes.Structure):
    _fields_ = [("struct_size", c_i32), ("dim", c_i32), ("lrate", c_dbl), ("drate", c_dbl),
                ("reg", c_dbl), ("seed", c_u64), ("mode", c_i32), ("precision", c_i32),
                ("init", c_i32), ("init_parts", c_i32), ("device", c_i32), ("workers", c_i32),
                ("warps_per_block", c_i32), ("blocks_per_sm", c_i32), ("balance", c_i32),
                ("dsgd_inner_blocks", c_i32), ("dsgd_strategy", c_i32), ("exact", c_i32),
                ("spin_budget_ms", c_i32), ("debug_flags", c_i32), ("long_visit", c_i32),
                ("priority_permille", c_i32), ("lr_strategy", c_i32), ("batch_share", c_i32),
                ("reserved", c_i32 * 4)]


class Matrix(ctypes.Structure):
    _fields_ = [("nnz", c_i64), ("row_counts", c_vp), ("rows", c_vp), ("cols", c_vp),
                ("vals_f64", c_vp), ("vals_f32", c_vp)]


class Problem(ctypes.Structure):
    _fields_ = [("m", c_i32), ("n", c_i32), ("train", Matrix), ("test", Matrix),
                ("W0", c_vp), ("H0", c_vp)]


class BatchProblem(ctypes.Structure):
    _fields_ = [("m", c_i32), ("n", c_i32), ("dim", c_i32), ("reserved", c_i32),
                ("train", Matrix), ("test", Matrix), ("W0", c_vp), ("H0", c_vp)]


class EpochStats(ctypes.Structure):
    _fields_ = [("updates", c_i64), ("hops", c_i64), ("failures", c_i64),
                ("epochs_done", c_i32), ("reserved0", c_i32), ("device_ms", c_dbl),
                ("host_seconds", c_dbl), ("online_sse", c_dbl), ("objective", c_dbl),
                ("lrate", c_dbl)]


class TuneTrial(ctypes.Structure):
    _fields_ = [("warps_per_block", c_i32), ("priority_permille", c_i32), ("long_visit", c_i32),
                ("status", c_i32), ("device_ms", c_dbl)]


class BatchTuneTrial(ctypes.Structure):
    _fields_ = [("batch_share", c_i32), ("status", c_i32), ("device_ms", c_dbl),
                ("large_problems", c_i32), ("reserved", c_i32)]


class CheckpointInfo(ctypes.Structure):
    _fields_ = [("m", c_i32), ("n", c_i32), ("dim", c_i32), ("epochs_done", c_i32),
                ("lrate", c_dbl), ("objective", c_dbl)]


class Info(ctypes.Structure):
    _fields_ = [("m", c_i32), ("n", c_i32), ("dim", c_i32), ("dim_padded", c_i32),
                ("nnz_train", c_i64), ("nnz_test", c_i64), ("workers", c_i32),
                ("active_tokens", c_i32), ("segments", c_i64), ("max_column", c_i64),
                ("grid_blocks", c_i32), ("block_threads", c_i32), ("num_sms", c_i32),
                ("inner_blocks", c_i32), ("device_bytes", c_i64), ("mode", c_i32),
                ("precision", c_i32), ("h2d_bytes", c_i64), ("d2h_bytes", c_i64),
                ("priority_tokens", c_i32), ("reserved0", c_i32)]


class IoMatrix(ctypes.Structure):
    _fields_ = [("file_id", c_i32), ("m", c_i32), ("n", c_i32), ("reserved", c_i32),
                ("nnz", c_i64), ("row_counts", ctypes.POINTER(c_i32)),
                ("cols", ctypes.POINTER(c_i32)), ("vals", ctypes.POINTER(c_dbl))]


class SynthSpec(ctypes.Structure):
    _fields_ = [("struct_size", c_i32), ("m", c_i32), ("n", c_i32), ("positions", c_i32),
                ("nnz_train", c_i64), ("nnz_test", c_i64), ("row_law", c_i32),
                ("col_law", c_i32), ("row_param", c_dbl), ("col_param", c_dbl),
                ("rank", c_i32), ("integer_values", c_i32), ("factor_std", c_dbl),
                ("noise_std", c_dbl), ("offset", c_dbl), ("scale", c_dbl),
                ("clip_lo", c_dbl), ("clip_hi", c_dbl), ("seed", c_u64), ("threads", c_i32),
                ("reserved", c_i32 * 7)]


# name -> (restype, argtypes) for every symbol the headers declare
SIGNATURES = {
    "nomad_gpu_params_default": (ctypes.c_int, [ctypes.POINTER(Params)]),
    "nomad_gpu_init": (ctypes.c_int, [ctypes.POINTER(c_vp), ctypes.POINTER(Problem),
                                      ctypes.POINTER(Params)]),
    "nomad_gpu_epoch": (ctypes.c_int, [c_vp, c_i32, ctypes.POINTER(EpochStats)]),
    "nomad_gpu_sse": (ctypes.c_int, [c_vp, ctypes.POINTER(c_dbl), ctypes.POINTER(c_i64),
                                     ctypes.POINTER(c_dbl), ctypes.POINTER(c_i64)]),
    "nomad_gpu_rmse": (ctypes.c_int, [c_vp, ctypes.POINTER(c_dbl), ctypes.POINTER(c_dbl)]),
    "nomad_gpu_get_factors": (ctypes.c_int, [c_vp, c_vp, c_vp]),
    "nomad_gpu_set_factors": (ctypes.c_int, [c_vp, c_vp, c_vp]),
    "nomad_gpu_get_info": (ctypes.c_int, [c_vp, ctypes.POINTER(Info)]),
    "nomad_gpu_set_epochs_done": (ctypes.c_int, [c_vp, c_i32]),
    "nomad_gpu_objective": (ctypes.c_int, [c_vp, ctypes.POINTER(c_dbl)]),
    "nomad_gpu_save_checkpoint": (ctypes.c_int, [c_vp, ctypes.c_char_p]),
    "nomad_gpu_load_checkpoint": (ctypes.c_int, [c_vp, ctypes.c_char_p]),
    "nomad_gpu_destroy": (None, [c_vp]),
    "nomad_gpu_strerror": (ctypes.c_char_p, [ctypes.c_int]),
    "nomad_gpu_last_error": (ctypes.c_char_p, []),
    "nomad_gpu_device_ok": (ctypes.c_int, [c_i32]),
    "nomad_gpu_token_finish_times": (ctypes.c_int, [c_vp, c_vp]),
    "nomad_gpu_autotune": (ctypes.c_int, [ctypes.POINTER(Problem), ctypes.POINTER(Params), c_i32,
                                          ctypes.POINTER(TuneTrial), c_i32, ctypes.POINTER(c_i32)]),
    "nomad_gpu_batch_autotune": (ctypes.c_int, [ctypes.POINTER(BatchProblem), c_i32, ctypes.POINTER(Params),
                                                c_i32, ctypes.POINTER(BatchTuneTrial), c_i32,
                                                ctypes.POINTER(c_i32)]),
    "nomad_gpu_sse_noalloc": (ctypes.c_int, [c_i32, c_i32, c_i32, c_i32, c_vp, c_vp, c_vp, c_vp,
                                             c_i64, c_i32, c_vp, c_vp]),
    "nomad_gpu_batch_init": (ctypes.c_int, [ctypes.POINTER(c_vp), ctypes.POINTER(BatchProblem), c_i32,
                                            ctypes.POINTER(Params)]),
    "nomad_gpu_batch_epoch": (ctypes.c_int, [c_vp, c_i32, ctypes.POINTER(EpochStats)]),
    "nomad_gpu_batch_rmse": (ctypes.c_int, [c_vp, c_vp, c_vp]),
    "nomad_gpu_batch_get_factors": (ctypes.c_int, [c_vp, c_i32, c_vp, c_vp]),
    "nomad_gpu_batch_destroy": (None, [c_vp]),
    "nomad_synth_batch_problem": (ctypes.c_int, [c_u64, c_i32, ctypes.POINTER(SynthSpec),
                                                 ctypes.POINTER(c_i32)]),
    "nomad_io_read_header": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(c_i32),
                                            ctypes.POINTER(c_i32), ctypes.POINTER(c_i32),
                                            ctypes.POINTER(c_i64)]),
    "nomad_io_read": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(IoMatrix)]),
    "nomad_io_write": (ctypes.c_int, [ctypes.c_char_p, c_i32, c_i32, c_i64, c_vp, c_vp, c_vp,
                                      c_i32]),
    "nomad_io_free": (None, [ctypes.POINTER(IoMatrix)]),
    "nomad_io_write_factors": (ctypes.c_int, [ctypes.c_char_p, c_i32, c_i32, c_i32, c_vp,
                                              c_vp]),
    "nomad_io_write_checkpoint": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(CheckpointInfo),
                                                 c_vp, c_vp]),
    "nomad_io_read_checkpoint_header": (ctypes.c_int, [ctypes.c_char_p,
                                                       ctypes.POINTER(CheckpointInfo)]),
    "nomad_io_read_checkpoint": (ctypes.c_int, [ctypes.c_char_p, c_i32, c_i32, c_i32, c_vp, c_vp,
                                                ctypes.POINTER(CheckpointInfo)]),
    "nomad_reference_init": (ctypes.c_int, [c_i32, c_i32, c_i32, c_u64, c_i32, c_vp, c_vp]),
    "nomad_synth_preset": (ctypes.c_int, [c_i32, ctypes.POINTER(SynthSpec)]),
    "nomad_synth_generate": (ctypes.c_int, [ctypes.POINTER(SynthSpec),
                                            ctypes.POINTER(IoMatrix),
                                            ctypes.POINTER(IoMatrix)]),
}

_lib = None


class NomadError(RuntimeError):
    def __init__(self, status, where, detail=""):
        self.status = status
        msg = f"{where}: status {status}"
        if _lib is not None:
            msg += f" ({_lib.nomad_gpu_strerror(status).decode()})"
        if detail:
            msg += f": {detail}"
        super().__init__(msg)


def lib():
    """The loaded shared library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'` (no CPU fallback exists)")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(status, where):
    if status != OK:
        detail = lib().nomad_gpu_last_error().decode(errors="replace")
        raise NomadError(status, where, detail)
    return status
