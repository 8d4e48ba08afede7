"""train.dat / test.dat format, the --output dump and the reference init (no GPU).

Format (Code/nomad/nb_data.cpp:32-130; writers Scripts/convert.py:99-105 and
Code/nomad/synthgen.cpp:298-311): int32 id (1211216 -> int32 nnz, 1015 -> int64 nnz),
int32 m, int32 n, nnz, int32 row_counts[m], int32 cols[nnz], float64 vals[nnz].
"""
import os
import struct

import numpy as np
import pytest


def _convert_py_style(path, m, n, rows_cols_vals):
    """Bytes exactly as convert.py packs them ("=iiii", "=%si", "=%si", "=%sd")."""
    rows_cols_vals = sorted(rows_cols_vals)
    counts = [0] * m
    for r, _, _ in rows_cols_vals:
        counts[r] += 1
    with open(path, "wb") as f:
        f.write(struct.pack("=iiii", 1211216, m, n, len(rows_cols_vals)))
        f.write(struct.pack("=%si" % m, *counts))
        f.write(struct.pack("=%si" % len(rows_cols_vals), *[c for _, c, _ in rows_cols_vals]))
        f.write(struct.pack("=%sd" % len(rows_cols_vals), *[v for _, _, v in rows_cols_vals]))


def test_read_convert_py_bytes(ng, O, tmp_path):
    p = str(tmp_path / "train.dat")
    entries = [(0, 2, 5.0), (0, 4, 1.5), (2, 0, -1.0), (3, 1, 4.25), (3, 3, 2.0)]
    _convert_py_style(p, 4, 5, entries)
    h = ng.read_header(p)
    assert h == {"file_id": 1211216, "m": 4, "n": 5, "nnz": 5}
    A = ng.RatingMatrix.read(p)
    assert list(A.row_counts) == [2, 0, 1, 2]
    assert list(A.cols) == [2, 4, 0, 1, 3]
    assert list(A.vals) == [5.0, 1.5, -1.0, 4.25, 2.0]
    B = O.read_matrix(p)  # the oracle's restatement of read_data agrees
    assert np.array_equal(B["cols"], A.cols) and np.array_equal(B["vals"], A.vals)


@pytest.mark.parametrize("file_id", [0, 1211216, 1015])
def test_write_read_roundtrip(ng, tmp_path, file_id):
    train, _ = ng.synth(ng.synth_spec(1, m=50, n=40, nnz_train=300, nnz_test=10))
    p = str(tmp_path / "m.dat")
    train.write(p, file_id)
    size = os.path.getsize(p)
    hdr = 20 if file_id == 1015 else 16
    assert size == hdr + 4 * train.m + 12 * train.nnz
    B = ng.RatingMatrix.read(p)
    assert B.file_id == (file_id or 1211216)
    assert np.array_equal(B.row_counts, train.row_counts)
    assert np.array_equal(B.cols, train.cols) and np.array_equal(B.vals, train.vals)


def test_long_header_layout(ng, tmp_path):
    p = str(tmp_path / "l.dat")
    A = ng.RatingMatrix(2, 3, [1, 1], [2, 0], [1.0, 2.0])
    A.write(p, 1015)
    with open(p, "rb") as f:
        fid, m, n = struct.unpack("=iii", f.read(12))
        (nnz,) = struct.unpack("=q", f.read(8))
    assert (fid, m, n, nnz) == (1015, 2, 3, 2)


def test_format_errors(ng, tmp_path):
    bad = tmp_path / "bad.dat"
    bad.write_bytes(struct.pack("=iiii", 42, 1, 1, 0))
    with pytest.raises(ng.NomadError) as e:
        ng.RatingMatrix.read(str(bad))
    assert e.value.status == -7
    short = tmp_path / "short.dat"
    short.write_bytes(struct.pack("=iiii", 1211216, 2, 2, 3) + struct.pack("=ii", 1, 2))
    with pytest.raises(ng.NomadError) as e:
        ng.RatingMatrix.read(str(short))
    assert e.value.status == -7
    mism = tmp_path / "mism.dat"  # row counts do not add up to nnz
    mism.write_bytes(struct.pack("=iiii", 1211216, 2, 2, 3) + struct.pack("=ii", 1, 1) +
                     struct.pack("=iii", 0, 1, 0) + struct.pack("=ddd", 1, 2, 3))
    with pytest.raises(ng.NomadError):
        ng.RatingMatrix.read(str(mism))
    oob = tmp_path / "oob.dat"  # column index out of range
    oob.write_bytes(struct.pack("=iiii", 1211216, 1, 2, 1) + struct.pack("=i", 1) +
                    struct.pack("=i", 5) + struct.pack("=d", 1))
    with pytest.raises(ng.NomadError):
        ng.RatingMatrix.read(str(oob))
    with pytest.raises(ng.NomadError) as e:
        ng.RatingMatrix.read(str(tmp_path / "missing.dat"))
    assert e.value.status == -6


def test_empty_matrix(ng, tmp_path):
    p = str(tmp_path / "e.dat")
    A = ng.RatingMatrix(3, 2, [0, 0, 0], [], [])
    A.write(p)
    B = ng.RatingMatrix.read(p)
    assert B.nnz == 0 and B.m == 3 and B.n == 2


def test_factor_dump_format(ng, tmp_path):
    p = str(tmp_path / "out0")
    W = np.array([[0.5, 0.25], [1.0 / 3.0, 2.0]], np.float32)
    H = np.array([[1e-7, 123456.789]], np.float32)
    ng.write_factors(p, W, H)
    lines = open(p).read().splitlines()
    # ostream default format: %g with 6 significant digits (nb_main.cpp:696-698)
    assert lines[0] == "row,0,0.5,0.25"
    assert lines[1] == "row,1,0.333333,2"
    assert lines[2] == "column,0,1e-07,123457"


def test_reference_init_matches_oracle(ng, O):
    # small and large parts (the values come 312 to a twist), dim 1 (bound 1.0), more parts
    # than rows, a seed above 2^63
    for m, n, dim, seed, parts in [(37, 11, 10, 12345, 1), (100, 7, 33, 99, 4),
                                   (5, 5, 100, 0, 16), (3000, 700, 100, 12345, 16),
                                   (480, 17, 1, 5, 7), (1, 2000, 64, 2**63 + 5, 3)]:
        W, H = ng.reference_init(m, n, dim, seed, parts)
        Wd, Hd = O.init_factors(m, n, dim, seed, parts)
        assert np.array_equal(W, Wd.astype(np.float32))
        assert np.array_equal(H, Hd.astype(np.float32))
