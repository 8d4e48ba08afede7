"""nomad_gpu_sse_noalloc: evaluation for callers that cannot allocate device memory.

Some callers of this library cannot let it call cudaMalloc: a host runtime that gives
out device memory only from its own pool, or a tight loop that must not pay for the
device-wide wait of cudaFree.  They hold the inputs and the output in their own device
buffers; the entry point keeps its per-block partial sums in a fixed array inside the
library.  This test gives it buffers owned by the caller (allocated here through
PyTorch, which plays the caller's memory pool), calls it twice in a row through the
C-ABI, and checks both results against the context-based nomad_gpu_sse of the same
factors and ratings, within the 1e-6 relative tolerance of the other evaluation test.

The file name makes pytest collect it last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-6


def _problem(ng):
    return ng.synth(ng.synth_spec(1, m=3000, n=700, nnz_train=80000, nnz_test=8000, seed=99))


def _device_layout(torch, ng, A, W, H, precision):
    """Padded factor storage and the CSC rating pairs, in caller-owned device memory."""
    dim = W.shape[1]
    E = 4 if precision == "fp32" else 8
    kpad = (dim + E - 1) // E * E
    tdt = torch.float32 if precision == "fp32" else torch.bfloat16
    Wp = torch.zeros((W.shape[0], kpad), dtype=tdt)
    Hp = torch.zeros((H.shape[0], kpad), dtype=tdt)
    Wp[:, :dim] = torch.from_numpy(W).to(tdt)
    Hp[:, :dim] = torch.from_numpy(H).to(tdt)
    col_ptr, rows, vals = A.to_csc()
    pairs = np.empty((rows.size, 2), np.int32)
    pairs[:, 0] = rows
    pairs[:, 1] = vals.astype(np.float32).view(np.int32)
    return (Wp.cuda(), Hp.cuda(), torch.from_numpy(pairs).cuda(),
            torch.from_numpy(col_ptr).cuda())


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_noalloc_matches_context_sse_twice(ng, gpu_ok, precision):
    torch = pytest.importorskip("torch")
    train, test = _problem(ng)
    dim = 100
    rng = np.random.default_rng(5)
    W = (rng.standard_normal((train.m, dim)) * 0.1).astype(np.float32)
    H = (rng.standard_normal((train.n, dim)) * 0.1).astype(np.float32)
    with ng.Nomad(train, test, W0=W, H0=H, dim=dim, precision=precision) as nm:
        ref_train, _, ref_test, _ = nm.sse()
    L = ng.lib()
    prec = 0 if precision == "fp32" else 1
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for A, ref in ((train, ref_train), (test, ref_test)):
        Wd, Hd, pairs, col_ptr = _device_layout(torch, ng, A, W, H, precision)
        out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
        got = []
        for _ in range(2):  # the array keeps the previous call's partials
            rc = L.nomad_gpu_sse_noalloc(0, prec, A.n, dim, Wd.data_ptr(), Hd.data_ptr(),
                                         pairs.data_ptr(), col_ptr.data_ptr(), A.nnz, 0,
                                         out.data_ptr(), stream)
            assert rc == 0, L.nomad_gpu_last_error()
            torch.cuda.synchronize()
            got.append(out.item())
        for g in got:
            assert abs(g - ref) <= TOL * ref, (g, ref)
        assert got[0] == got[1]


def test_noalloc_rejects_too_many_blocks(ng, gpu_ok):
    torch = pytest.importorskip("torch")
    train, _ = _problem(ng)
    dim = 8
    W = np.zeros((train.m, dim), np.float32)
    H = np.zeros((train.n, dim), np.float32)
    Wd, Hd, pairs, col_ptr = _device_layout(torch, ng, train, W, H, "fp32")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    L = ng.lib()
    rc = L.nomad_gpu_sse_noalloc(0, 0, train.n, dim, Wd.data_ptr(), Hd.data_ptr(),
                                 pairs.data_ptr(), col_ptr.data_ptr(), train.nnz,
                                 ng._abi.NOALLOC_MAX_BLOCKS + 1, out.data_ptr(), None)
    assert rc == ng._abi.ERR_INVALID_ARG
    assert b"exceeds" in L.nomad_gpu_last_error()
    rc = L.nomad_gpu_sse_noalloc(0, 0, train.n, dim, Wd.data_ptr(), Hd.data_ptr(),
                                 pairs.data_ptr(), col_ptr.data_ptr(), train.nnz,
                                 ng._abi.NOALLOC_MAX_BLOCKS, out.data_ptr(), None)
    assert rc == 0
    torch.cuda.synchronize()
    ref = float(np.sum(train.vals.astype(np.float32).astype(np.float64) ** 2))
    assert abs(out.item() - ref) <= TOL * ref
