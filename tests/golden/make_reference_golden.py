"""Golden outputs of the reference's own updater, for pinning the oracle.

Builds the reference's unmodified Code/nomad/nb_main.cpp, nb_data.cpp and pool.cpp
against the stand-in headers in oracle/refshim (oracle/Makefile.ref), writes each case's
train.dat/test.dat, runs the reference updater thread for the case's epochs on one rank
with one thread (deterministic: columns round-robin in index order), and stores inputs
and outputs in tests/golden/reference_replay.npz:

  H          every column's values after the last epoch (double, bit for bit)
  train_sse, test_sse, train_count, test_count   the reference's evaluation pass
  updates    the updater's update counter (u=)
  col_err    each column token's accumulated online error

Needs the reference tree (NOMAD_REFERENCE_DIR, default /root/reference).
Run:  python tests/golden/make_reference_golden.py
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402

OUT = os.path.join(HERE, "reference_replay.npz")


def case_uniform():
    """300 x 80, 4,000 distinct cells drawn uniformly, integer ratings 1-5, 10% test."""
    rng = np.random.default_rng(5)
    m, n = 300, 80
    cells = np.sort(rng.choice(m * n, 4000, replace=False))
    r, c = np.divmod(cells, n)
    v = rng.integers(1, 6, r.size).astype(np.float64)
    test = rng.random(r.size) < 0.1
    return dict(m=m, n=n, dim=16, lrate=0.01, drate=0.1, reg=0.05, seed=12345, epochs=3,
                file_id=1211216, r=r, c=c, v=v, test=test)


def case_ragged():
    """120 x 50 with empty rows and columns, a one-rating column, a column rated by most
    rows, real-valued ratings, an odd dimension and the long-nnz file header (id 1015)."""
    rng = np.random.default_rng(11)
    m, n = 120, 50
    mask = rng.random((m, n)) < 0.08
    mask[:, 7] = False                      # empty column
    mask[:, 9] = rng.random(m) < 0.9        # dense column
    mask[:, 13] = False
    mask[17, 13] = True                     # one rating
    mask[40:45, :] = False                  # empty rows
    r, c = np.nonzero(mask)
    v = rng.normal(0.0, 1.0, r.size)
    test = rng.random(r.size) < 0.15
    return dict(m=m, n=n, dim=7, lrate=0.02, drate=0.05, reg=0.1, seed=777, epochs=4,
                file_id=1015, r=r, c=c, v=v, test=test)


CASES = {"uniform": case_uniform, "ragged": case_ragged}


def split(cs):
    """Row-major (row counts, column indices, values) of the training and test parts."""
    out = []
    for sel in (~cs["test"], cs["test"]):
        r, c, v = cs["r"][sel], cs["c"][sel], cs["v"][sel]
        order = np.lexsort((c, r))
        out.append((np.bincount(r, minlength=cs["m"]).astype(np.int32), c[order].astype(np.int32), v[order]))
    return out


def run_reference(cs, rows_prefix=None):
    (tr, te) = split(cs)
    d = tempfile.mkdtemp(prefix="nomad_ref_")
    O.write_matrix(os.path.join(d, "train.dat"), cs["m"], cs["n"], *tr, file_id=cs["file_id"])
    O.write_matrix(os.path.join(d, "test.dat"), cs["m"], cs["n"], *te, file_id=cs["file_id"])
    res = O.ref_replay(d, cs["n"], cs["dim"], cs["lrate"], cs["drate"], cs["reg"], cs["seed"], cs["epochs"],
                       rows_prefix=os.path.join(d, rows_prefix) if rows_prefix else None)
    return d, res


def main():
    if not O.build_ref():
        raise SystemExit("the reference tree is not on this machine")
    arrays = {}
    for name, make in CASES.items():
        cs = make()
        _, res = run_reference(cs)
        (tr, te) = split(cs)
        for k in ("m", "n", "dim", "lrate", "drate", "reg", "seed", "epochs", "file_id"):
            arrays[f"{name}.{k}"] = np.array(cs[k])
        for part, (rc, cols, vals) in (("train", tr), ("test", te)):
            arrays[f"{name}.{part}.row_counts"] = rc
            arrays[f"{name}.{part}.cols"] = cols
            arrays[f"{name}.{part}.vals"] = vals
        for k in ("H", "col_err", "train_sse", "test_sse", "train_count", "test_count", "updates"):
            arrays[f"{name}.out.{k}"] = np.array(res[k])
        print(name, "train RMSE", np.sqrt(res["train_sse"] / res["train_count"]),
              "test RMSE", np.sqrt(res["test_sse"] / max(res["test_count"], 1)))
    np.savez_compressed(OUT, **arrays)


if __name__ == "__main__":
    main()
