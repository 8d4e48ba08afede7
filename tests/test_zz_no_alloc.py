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


def test_noalloc_refuses_misaligned_and_columnless_input(ng, gpu_ok):
    """A view at an odd offset is refused on the host (no kernel runs), and so are
    ratings without any column."""
    torch = pytest.importorskip("torch")
    train, _ = _problem(ng)
    dim = 8
    W = np.zeros((train.m, dim), np.float32)
    H = np.zeros((train.n, dim), np.float32)
    Wd, Hd, pairs, col_ptr = _device_layout(torch, ng, train, W, H, "fp32")
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    L = ng.lib()
    E = ng._abi.ERR_INVALID_ARG
    args = [0, 0, train.n, dim, Wd.data_ptr(), Hd.data_ptr(), pairs.data_ptr(), col_ptr.data_ptr(),
            train.nnz, 0, out.data_ptr(), None]
    for i, off in ((4, 4), (5, 8), (6, 4), (7, 4), (10, 4)):
        bad = list(args)
        bad[i] += off
        assert L.nomad_gpu_sse_noalloc(*bad) == E, i
        assert b"aligned" in L.nomad_gpu_last_error()
    bad = list(args)
    bad[2] = 0
    assert L.nomad_gpu_sse_noalloc(*bad) == E
    torch.cuda.synchronize()
    assert out.abs().sum().item() == 0.0


def test_noalloc_empty_set_and_side_stream(ng, gpu_ok):
    """nnz = 0 writes 0; on a side stream, a call ordered after the kernels that fill
    its inputs on that same stream reads the filled inputs."""
    torch = pytest.importorskip("torch")
    train, test = _problem(ng)
    dim = 64
    rng = np.random.default_rng(8)
    W = (rng.standard_normal((train.m, dim)) * 0.1).astype(np.float32)
    H = (rng.standard_normal((train.n, dim)) * 0.1).astype(np.float32)
    with ng.Nomad(train, test, W0=W, H0=H, dim=dim, precision="fp32") as nm:
        ref, _, _, _ = nm.sse()
    L = ng.lib()
    Wd, Hd, pairs, col_ptr = _device_layout(torch, ng, train, W, H, "fp32")
    out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    rc = L.nomad_gpu_sse_noalloc(0, 0, train.n, dim, Wd.data_ptr(), Hd.data_ptr(), pairs.data_ptr(),
                                 col_ptr.data_ptr(), 0, 0, out.data_ptr(), None)
    assert rc == 0
    torch.cuda.synchronize()
    assert out.item() == 0.0
    side = torch.cuda.Stream()
    W2 = torch.empty_like(Wd)
    H2 = torch.empty_like(Hd)
    torch.cuda.synchronize()
    with torch.cuda.stream(side):
        W2.copy_(Wd)  # producers of the inputs, on the side stream
        H2.copy_(Hd)
        rc = L.nomad_gpu_sse_noalloc(0, 0, train.n, dim, W2.data_ptr(), H2.data_ptr(), pairs.data_ptr(),
                                     col_ptr.data_ptr(), train.nnz, 0, out.data_ptr(),
                                     ctypes.c_void_p(side.cuda_stream))
        assert rc == 0, L.nomad_gpu_last_error()
    side.synchronize()
    assert abs(out.item() - ref) <= TOL * ref, (out.item(), ref)
