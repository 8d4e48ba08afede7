"""Text ratings to train.dat / test.dat: the reference's Scripts/convert.py for python3.

    python -m nomad_gb300.convert TRAIN_TXT TEST_TXT OUTPUT_DIR

Reads two tab-separated files of `user<TAB>item<TAB>rating[<TAB>...]` lines and writes,
into OUTPUT_DIR, the binary matrices the trainer reads and the id maps:

  train.dat, test.dat   header (1211216, m, n, nnz) as four int32, then the row counts
                        (int32[m]), the column index of every entry (int32[nnz]) and its
                        value (float64[nnz]), rows in order, columns ascending inside a
                        row, repeated (user, item) pairs summed into one entry
                        (Scripts/convert.py:75-95, 97-106, the csr_matrix it builds);
  user_ids.txt,         line k holds the original id of row k / column k
  item_ids.txt          (Scripts/convert.py:143-160).

Ids of both files index both matrices: m and n count every user and item seen in
either file.  Row and column indices are the positions of the ids in a shuffled list,
and the shuffle is the reference's own: the ids are collected in a Python 2 `set`, listed
in that set's iteration order, and shuffled by Python 2's `random.shuffle` after
`random.seed(12345)` (Scripts/convert.py:9, 21-52).  Both steps are restated here --
CPython 2.7's string hash and set table (Objects/stringobject.c string_hash,
Objects/setobject.c set_add_key / set_lookkey_string / set_table_resize), and 2.7's
shuffle loop `j = int(random() * (i + 1))`, driven by the same Mersenne Twister stream
that python3's `random.Random(12345).random()` produces -- so that a text file converts
to the same bytes and the same id maps as the reference script gives under Python 2.7
(64-bit build, hash randomisation off, its default).
"""
import argparse
import os
import random
import sys

import numpy as np

MAT_FILE_CLASSID = 1211216   # Code/nomad/nb_data.cpp:14; Scripts/convert.py:101
LONG_FILE_CLASSID = 1015     # Code/nomad/nb_data.cpp:15 (int64 nnz; read, not written here)

_M64 = (1 << 64) - 1
_PERTURB_SHIFT = 5
_SET_MINSIZE = 8


def py2_str_hash(b):
    """CPython 2.7's hash of a byte string on a 64-bit build (string_hash with a zero
    hash secret): x = b[0] << 7; x = (1000003 * x) ^ c for every byte c; x ^= len."""
    if not b:
        return 0
    x = (b[0] << 7) & _M64
    for c in b:
        x = ((1000003 * x) & _M64) ^ c
    x ^= len(b)
    if x >= 1 << 63:
        x -= 1 << 64
    return -2 if x == -1 else x


class Py2StrSet:
    """Insertion into, and iteration order of, a CPython 2.7 `set` of str.

    Open addressing over a power-of-two table: slot hash & mask, then the probe
    i = 5 i + perturb + 1 with perturb = hash >> 5 per step; after an insertion that
    fills two thirds of the table, the table grows to the smallest power of two above
    4 x used (2 x used beyond 50,000 entries) and the entries are re-inserted in slot
    order.  Iteration visits the slots in order."""

    def __init__(self):
        self.mask = _SET_MINSIZE - 1
        self.keys = [None] * _SET_MINSIZE
        self.hashes = [0] * _SET_MINSIZE
        self.used = 0
        self.members = set()

    def _probe(self, h):
        mask = self.mask
        perturb = h & _M64
        i = h & _M64
        while True:
            yield i & mask
            i = (i * 5 + perturb + 1) & _M64
            perturb >>= _PERTURB_SHIFT

    def add(self, key):
        if key in self.members:
            return
        h = py2_str_hash(key)
        for slot in self._probe(h):
            if self.keys[slot] is None:
                break
        self.keys[slot] = key
        self.hashes[slot] = h
        self.used += 1
        self.members.add(key)
        if self.used * 3 >= (self.mask + 1) * 2:   # fill == used: nothing is ever deleted
            self._resize(self.used * 2 if self.used > 50000 else self.used * 4)

    def _resize(self, minused):
        size = _SET_MINSIZE
        while size <= minused:
            size <<= 1
        old = [(k, h) for k, h in zip(self.keys, self.hashes) if k is not None]
        self.mask = size - 1
        self.keys = [None] * size
        self.hashes = [0] * size
        for k, h in old:
            for slot in self._probe(h):
                if self.keys[slot] is None:
                    break
            self.keys[slot] = k
            self.hashes[slot] = h

    def in_order(self):
        return [k for k in self.keys if k is not None]


def py2_shuffle(items, rng):
    """Python 2.7's random.shuffle (in place) with `rng.random()` as its random()."""
    for i in range(len(items) - 1, 0, -1):
        j = int(rng.random() * (i + 1))
        items[i], items[j] = items[j], items[i]


def _lines(path):
    with open(path, "rb") as f:
        for lineno, line in enumerate(f, 1):
            tokens = line.split(b"\t")
            if len(tokens) < 3:
                raise ValueError(f"{path}:{lineno}: expected user<TAB>item<TAB>rating, got {line!r}")
            yield tokens


def _matrix(pairs, m, n):
    """(row counts, column indices, values) of the csr_matrix the reference builds:
    entries sorted by (row, column), repeated pairs summed in file order."""
    rows = np.asarray(pairs[0], np.int64)
    cols = np.asarray(pairs[1], np.int64)
    vals = np.asarray(pairs[2], np.float64)
    if rows.size == 0:
        return np.zeros(m, np.int32), np.zeros(0, np.int32), np.zeros(0, np.float64)
    key = rows * n + cols
    order = np.argsort(key, kind="stable")
    key, vals = key[order], vals[order]
    first = np.ones(key.size, bool)
    first[1:] = key[1:] != key[:-1]
    starts = np.flatnonzero(first)
    summed = np.add.reduceat(vals, starts)
    ukey = key[starts]
    r, c = np.divmod(ukey, n)
    counts = np.bincount(r, minlength=m).astype(np.int32)
    return counts, c.astype(np.int32), summed


def write_matrix(path, m, n, row_counts, cols, vals):
    """train.dat layout: int32 (1211216, m, n, nnz), int32 row counts, int32 column
    indices, float64 values (Scripts/convert.py:101-104)."""
    if cols.size >= 1 << 31:
        raise ValueError("more than 2^31 - 1 entries do not fit the 1211216 header")
    with open(path, "wb") as f:
        np.array([MAT_FILE_CLASSID, m, n, cols.size], "<i4").tofile(f)
        np.ascontiguousarray(row_counts, "<i4").tofile(f)
        np.ascontiguousarray(cols, "<i4").tofile(f)
        np.ascontiguousarray(vals, "<f8").tofile(f)


def convert(train_path, test_path, output_path, seed=12345, log=None):
    """Convert the two text files; returns {"m", "n", "train_nnz", "test_nnz"}."""
    say = log or (lambda *a: None)
    users, items = Py2StrSet(), Py2StrSet()
    for name, path in (("training", train_path), ("test", test_path)):
        for index, tokens in enumerate(_lines(path)):
            if index % 1000000 == 0:
                say(f"1st pass {name}: {index}")
            users.add(tokens[0])
            items.add(tokens[1])
    rng = random.Random(seed)
    user_list, item_list = users.in_order(), items.in_order()
    py2_shuffle(user_list, rng)
    py2_shuffle(item_list, rng)
    user_index = {k: i for i, k in enumerate(user_list)}
    item_index = {k: i for i, k in enumerate(item_list)}
    m, n = len(user_list), len(item_list)
    os.makedirs(output_path, exist_ok=True)
    out = {"m": m, "n": n}
    for name, path, fname in (("training", train_path, "train.dat"), ("test", test_path, "test.dat")):
        ui, ii, vv = [], [], []
        for index, tokens in enumerate(_lines(path)):
            if index % 1000000 == 0:
                say(f"2nd pass {name}: {index}")
            ui.append(user_index[tokens[0]])
            ii.append(item_index[tokens[1]])
            vv.append(float(tokens[2]))
        counts, cols, vals = _matrix((ui, ii, vv), m, n)
        write_matrix(os.path.join(output_path, fname), m, n, counts, cols, vals)
        out["train_nnz" if fname == "train.dat" else "test_nnz"] = int(cols.size)
    for fname, ids in (("user_ids.txt", user_list), ("item_ids.txt", item_list)):
        with open(os.path.join(output_path, fname), "wb") as f:
            for k in ids:
                f.write(k + b"\n")
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(
        prog="python -m nomad_gb300.convert",
        description="tab-separated ratings -> train.dat/test.dat and id maps (Scripts/convert.py)")
    ap.add_argument("train_filename")
    ap.add_argument("test_filename")
    ap.add_argument("output_path")
    ap.add_argument("--seed", type=int, default=12345, help="random.seed of the id shuffle (12345)")
    ap.add_argument("--quiet", action="store_true")
    a = ap.parse_args(argv)
    log = None if a.quiet else (lambda *x: print(*x, file=sys.stderr, flush=True))
    try:
        info = convert(a.train_filename, a.test_filename, a.output_path, a.seed, log)
    except (OSError, ValueError, KeyError) as e:
        print(f"convert: {e}", file=sys.stderr)
        return 1
    if log:
        log(f"m={info['m']} n={info['n']} train nnz={info['train_nnz']} test nnz={info['test_nnz']}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
