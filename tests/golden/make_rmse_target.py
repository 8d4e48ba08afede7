"""FP64 oracle trajectory of the 480,189 x 17,770 workload (bench.py's time-to-target).

Runs the oracle's nomad_double replay (one worker, columns in index order; the
reference's schedule with --nthreads 1) from the reference init for EPOCHS epochs and
records the test RMSE after each, with a checksum of the generated workload so that a
run on another machine can tell whether it trained on the same data.

Run:  python tests/golden/make_rmse_target.py [epochs]
"""
import json
import os
import sys
import time
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import nomad_gb300 as ng  # noqa: E402
from oracle import oracle as O  # noqa: E402

HP = dict(dim=100, lrate=0.002, drate=0.05, reg=0.05)


def workload_checksum(train, test):
    c = 0
    for a in (train.row_counts, train.cols, train.vals, test.row_counts, test.cols, test.vals):
        c = zlib.crc32(np.ascontiguousarray(a).view(np.uint8), c)
    return c


def main():
    epochs = int(sys.argv[1]) if len(sys.argv) > 1 else 20
    train, test = ng.synth(2)
    csc = O.row_major_to_csc(train.m, train.n, train.row_counts, train.cols, train.vals)
    tcsc = O.row_major_to_csc(test.m, test.n, test.row_counts, test.cols, test.vals)
    W, H = O.init_factors(train.m, train.n, HP["dim"], 12345, 16)
    out = {"workload": 2, "init_parts": 16, "mode": "replay (nomad_double)", **HP,
           "checksum": workload_checksum(train, test), "test_rmse": [], "train_online_rmse": []}
    for e in range(epochs):
        t = time.time()
        err = O.replay(csc, W, H, e, 1, HP["lrate"], HP["drate"], HP["reg"])
        out["test_rmse"].append(O.rmse(tcsc, W, H))
        out["train_online_rmse"].append(float(np.sqrt(err[0] / train.nnz)))
        print(f"epoch {e}: test RMSE {out['test_rmse'][-1]:.6f} ({time.time() - t:.1f} s)",
              flush=True)
        with open(os.path.join(HERE, "workload2_fp64_rmse.json"), "w") as f:
            json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
