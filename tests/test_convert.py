"""The python3 converter (nomad_gb300/convert.py) of the reference's Scripts/convert.py:
tab-separated text -> train.dat/test.dat and the id maps.

The id order is the reference script's under Python 2.7: its ids pass through a
Python 2 set and Python 2's random.shuffle after random.seed(12345).  The pieces are
pinned by known answers of CPython 2.7 (64-bit): hash('a') = 12416037344,
hash('abc') = 1453079729188098211, and set(['a', 'b', 'c']) iterates a, c, b."""
import os
import random
import re
import subprocess

import numpy as np
import pytest

from nomad_gb300 import convert as C

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "nomad_gb300", "_build", "nomad_gpu")


def test_python2_hash_known_answers():
    assert C.py2_str_hash(b"") == 0
    assert C.py2_str_hash(b"a") == 12416037344
    assert C.py2_str_hash(b"abc") == 1453079729188098211


def test_python2_set_order_known_answer():
    s = C.Py2StrSet()
    for k in (b"a", b"b", b"c", b"a"):
        s.add(k)
    assert s.in_order() == [b"a", b"c", b"b"]


def test_python2_set_grows_and_keeps_every_key():
    """Past the table's resizes (8 -> 32 -> 128 -> ... slots) every key is listed once."""
    s = C.Py2StrSet()
    keys = [str(i).encode() for i in range(5000)]
    for k in keys + keys[:100]:
        s.add(k)
    got = s.in_order()
    assert sorted(got) == sorted(keys) and s.mask + 1 >= 3 * len(keys) // 2


def test_python2_shuffle_loop():
    """2.7's loop: for i from n-1 down to 1, j = int(random() * (i + 1)), swap."""
    class Fixed:
        def __init__(self, xs):
            self.xs = list(xs)

        def random(self):
            return self.xs.pop(0)
    items = list("abcd")
    C.py2_shuffle(items, Fixed([0.0, 0.99, 0.5]))  # i=3 -> j=0, i=2 -> j=2, i=1 -> j=1
    assert items == list("dbca")
    # the stream python3 gives for an int seed is Python 2's (init_by_array, genrand_res53)
    a, b = random.Random(12345), random.Random(12345)
    assert [a.random() for _ in range(3)] == [b.random() for _ in range(3)]


TRAIN_TXT = b"alice\tdune\t5\nbob\tdune\t3\t978300760\nalice\temma\t4\nalice\tdune\t1\ncarol\tfargo\t2.5\n"
TEST_TXT = b"bob\temma\t2\ndave\tdune\t4\n"


def _convert(tmp_path, train=TRAIN_TXT, test=TEST_TXT):
    tr, te = tmp_path / "train.txt", tmp_path / "test.txt"
    tr.write_bytes(train)
    te.write_bytes(test)
    out = tmp_path / "out"
    info = C.convert(str(tr), str(te), str(out))
    return out, info


def test_fixture_bytes(tmp_path):
    """A hand-checked case: ids of both files index both matrices; (alice, dune) appears
    twice and is summed; a fourth column (timestamp) is ignored; dave has no training
    rating; columns ascend inside a row."""
    out, info = _convert(tmp_path)
    assert info == {"m": 4, "n": 3, "train_nnz": 4, "test_nnz": 2}
    assert (out / "user_ids.txt").read_bytes() == b"dave\nalice\ncarol\nbob\n"
    assert (out / "item_ids.txt").read_bytes() == b"emma\ndune\nfargo\n"
    hdr = lambda nnz: np.array([1211216, 4, 3, nnz], "<i4").tobytes()  # noqa: E731
    train = (hdr(4) + np.array([0, 2, 1, 1], "<i4").tobytes() + np.array([0, 1, 2, 1], "<i4").tobytes()
             + np.array([4.0, 6.0, 2.5, 3.0], "<f8").tobytes())
    test = (hdr(2) + np.array([1, 0, 0, 1], "<i4").tobytes() + np.array([1, 0], "<i4").tobytes()
            + np.array([4.0, 2.0], "<f8").tobytes())
    assert (out / "train.dat").read_bytes() == train
    assert (out / "test.dat").read_bytes() == test


def _text_from_matrix(rng, m, n, nnz, dup=0):
    users = [f"u{rng.integers(1 << 40)}".encode() for _ in range(m)]
    items = [f"i{rng.integers(1 << 40)}".encode() for _ in range(n)]
    cells = rng.choice(m * n, nnz, replace=False)
    r, c = np.divmod(cells, n)
    v = rng.integers(1, 6, nnz).astype(float)
    lines = [b"%s\t%s\t%g\n" % (users[a], items[b], x) for a, b, x in zip(r, c, v)]
    lines += lines[:dup]
    order = rng.permutation(len(lines))
    return b"".join(lines[i] for i in order), users, items


def _parse(text):
    acc = {}
    for line in text.splitlines():
        u, i, x = line.split(b"\t")[:3]
        acc[(u, i)] = acc.get((u, i), 0.0) + float(x)
    return acc


def test_round_trip_through_the_readers(ng, O, tmp_path):
    """Converted files read back (the library's reader and the oracle's restatement of
    nb_data.cpp) give the text's ratings, repeated pairs summed, through the id maps."""
    rng = np.random.default_rng(3)
    train_txt, _, _ = _text_from_matrix(rng, 300, 90, 3000, dup=40)
    test_txt, _, _ = _text_from_matrix(rng, 250, 80, 400)
    out, info = _convert(tmp_path, train_txt, test_txt)
    uids = (out / "user_ids.txt").read_bytes().split(b"\n")[:-1]
    iids = (out / "item_ids.txt").read_bytes().split(b"\n")[:-1]
    assert len(uids) == info["m"] and len(iids) == info["n"]
    assert len(set(uids)) == len(uids) and len(set(iids)) == len(iids)
    for fname, text in (("train.dat", train_txt), ("test.dat", test_txt)):
        lib_m = ng.RatingMatrix.read(str(out / fname))
        orc = O.read_matrix(str(out / fname))
        assert (lib_m.m, lib_m.n) == (info["m"], info["n"]) == (orc["m"], orc["n"])
        assert np.array_equal(lib_m.cols, orc["cols"]) and np.array_equal(lib_m.vals, orc["vals"])
        rows = lib_m.rows()
        got = {(uids[a], iids[b]): x for a, b, x in zip(rows, lib_m.cols, lib_m.vals)}
        assert got == _parse(text)
        for a in range(lib_m.m):  # columns ascending inside each row
            cs = lib_m.cols[lib_m.row_counts[:a].sum():lib_m.row_counts[:a + 1].sum()]
            assert np.all(np.diff(cs) > 0)


def test_reference_loader_reads_converted_files(O, tmp_path):
    """The reference's own read_data (built from the reference tree) trains on the
    converted files and evaluates every rating."""
    if O.reference_tree() is None:
        pytest.skip("the reference tree is not on this machine")
    rng = np.random.default_rng(4)
    train_txt, _, _ = _text_from_matrix(rng, 200, 60, 1500)
    test_txt, _, _ = _text_from_matrix(rng, 200, 60, 150)
    out, info = _convert(tmp_path, train_txt, test_txt)
    res = O.ref_replay(str(out), info["n"], 8, 0.01, 0.1, 0.05, 12345, 2)
    assert res["train_count"] == info["train_nnz"] and res["test_count"] == info["test_nnz"]
    assert res["updates"] == 2 * info["train_nnz"]


def test_command_line(tmp_path):
    (tmp_path / "a.txt").write_bytes(TRAIN_TXT)
    (tmp_path / "b.txt").write_bytes(TEST_TXT)
    r = subprocess.run(["python3", "-m", "nomad_gb300.convert", str(tmp_path / "a.txt"), str(tmp_path / "b.txt"),
                        str(tmp_path / "o")], capture_output=True, text=True, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    assert "1st pass training: 0" in r.stderr and (tmp_path / "o" / "train.dat").exists()
    (tmp_path / "bad.txt").write_bytes(b"just one column\n")
    r = subprocess.run(["python3", "-m", "nomad_gb300.convert", str(tmp_path / "bad.txt"), str(tmp_path / "b.txt"),
                        str(tmp_path / "o2")], capture_output=True, text=True, cwd=ROOT)
    assert r.returncode == 1 and "expected user<TAB>item<TAB>rating" in r.stderr


@pytest.mark.gpu
def test_nomad_gpu_trains_on_converted_files(ng, gpu_ok, tmp_path):
    """Text -> convert -> nomad_gpu --path: the run reads the files and reports the
    reference's statistics over every converted rating."""
    rng = np.random.default_rng(5)
    train_txt, _, _ = _text_from_matrix(rng, 500, 150, 8000)
    test_txt, _, _ = _text_from_matrix(rng, 500, 150, 800)
    out, info = _convert(tmp_path, train_txt, test_txt)
    r = subprocess.run([CLI, "--path", str(out), "--dim", "16", "--lrate", "0.01", "--timeout", "0.3"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    m = re.search(r"detail: train: s=([0-9.e+]+), c=(\d+); test: s=([0-9.e+]+), c=(\d+)", r.stdout)
    assert m and int(m.group(2)) == info["train_nnz"] and int(m.group(4)) == info["test_nnz"]
