"""The asynchronous modes' visit lists built on the device (nomad_gb300/csrc/layout_device.cu)
against the host build (host_layout.cpp: build_async_layout), through the C-ABI.

With debug bit 2 a context builds the layout both ways and refuses (NOMAD_ERR_BOUNDS)
unless the two agree field by field: worker row blocks, every visit {start, len, owner}
in route order, visit offsets, first visits, initial queues and the counts.  Cases: the
pipelined kernel with priority columns (block visits, hierarchical routes) for both row
types and several block sizes, with priority columns off, the exact kernel (shuffled
routes), empty rows and columns, and the 480,189 x 17,770 workload at full size.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def padded(ng, r, extra_rows, extra_cols):
    return ng.RatingMatrix(r.m + extra_rows, r.n + extra_cols,
                           np.concatenate([r.row_counts, np.zeros(extra_rows, np.int32)]), r.cols, r.vals)


@pytest.mark.parametrize("kw", [
    dict(precision="bf16"),
    dict(precision="fp32"),
    dict(precision="bf16", warps_per_block=8, priority_permille=10),
    dict(precision="fp32", priority_permille=-1),
    dict(precision="fp32", exact=1, workers=300),
    dict(precision="bf16", balance=0),
])
def test_device_layout_equals_host(ng, gpu_ok, kw):
    train, test = ng.synth(ng.synth_spec(2, m=20000, n=1500, nnz_train=600000, nnz_test=20000, seed=99))
    train, test = padded(ng, train, 30, 11), padded(ng, test, 30, 11)
    with ng.Nomad(train, test, dim=32, mode="async", debug_flags=4, **kw) as nm:
        st = nm.epoch(1)
    assert st["updates"] == train.nnz


def test_device_layout_full_size(ng, gpu_ok):
    train, test = ng.synth(2)
    with ng.Nomad(train, test, dim=100, mode="async", precision="bf16", debug_flags=4) as nm:
        info = nm.info()
    assert info["segments"] > 0
