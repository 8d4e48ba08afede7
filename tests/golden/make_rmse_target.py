"""FP64 oracle trajectories of the large workloads (bench.py's time-to-target and gaps).

Trains the oracle in double precision from the reference init for EPOCHS epochs and
records the test RMSE after each, with a checksum of the generated workload so that a
run on another machine can tell whether it trained on the same data.  Two oracles:

  replay  nomad_double with one worker: columns in index order (the reference's
          schedule with --nthreads 1; the oracle equals the reference's own updater bit
          for bit on this schedule, tests/test_reference_pin.py);
  async   nomad_double with P workers (the reference with --nthreads P): the oracle's
          deterministic event simulation, rows in P parts of about nnz/P ratings, each
          column's route its mt19937_64(seed + 137) permutation of the workers.

Workloads: 2 = 480,189 x 17,770 (lrate 0.002), 3 = 1,000,990 x 624,961 (lrate 0.0005);
drate 0.05, reg 0.05, k = 100 for both.

Run:  python tests/golden/make_rmse_target.py --workload 2 --mode replay --epochs 20
      python tests/golden/make_rmse_target.py --workload 2 --mode async --workers 1824
"""
import argparse
import json
import os
import sys
import time
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402

HP = {2: dict(dim=100, lrate=0.002, drate=0.05, reg=0.05),
      3: dict(dim=100, lrate=0.0005, drate=0.05, reg=0.05)}
# the event simulation's time units: a visit costs VISIT + RATING * len, a hop HOP
VISIT, RATING, HOP = 3000.0, 400.0, 3000.0


def workload_checksum(train, test):
    c = 0
    for a in (train["row_counts"], train["cols"], train["vals"], test["row_counts"], test["cols"], test["vals"]):
        c = zlib.crc32(np.ascontiguousarray(a).view(np.uint8), c)
    return c


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", type=int, default=2, choices=(2, 3))
    ap.add_argument("--mode", default="replay", choices=("replay", "async"))
    ap.add_argument("--workers", type=int, default=1824)
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--out", default=None)
    a = ap.parse_args()
    hp = HP[a.workload]
    name = f"workload{a.workload}_fp64_rmse.json" if a.mode == "replay" else f"workload{a.workload}_async_fp64_rmse.json"
    out_path = a.out or os.path.join(HERE, name)
    train, test = O.workload(a.workload)
    m, n = train["m"], train["n"]
    csc = O.row_major_to_csc(m, n, train["row_counts"], train["cols"], train["vals"])
    tcsc = O.row_major_to_csc(m, n, test["row_counts"], test["cols"], test["vals"])
    W, H = O.init_factors(m, n, hp["dim"], 12345, 16)
    out = {"workload": a.workload, "init_parts": 16, **hp, "checksum": workload_checksum(train, test),
           "test_rmse": [], "train_online_rmse": []}
    if a.mode == "replay":
        out["mode"] = "replay (nomad_double, one worker)"
    else:
        out["mode"] = (f"async (nomad_double, {a.workers} workers, deterministic event simulation: visit "
                       f"{VISIT:g} + {RATING:g}/rating, hop {HOP:g}; rows in parts of equal rating counts)")
        out["workers"] = a.workers
    nnz = int(train["cols"].size)
    del train, test
    for e in range(a.epochs):
        t = time.time()
        if a.mode == "replay":
            err = O.replay(csc, W, H, e, 1, hp["lrate"], hp["drate"], hp["reg"])
        else:
            err = O.async_sim(csc, W, H, a.workers, e, 1, hp["lrate"], hp["drate"], hp["reg"], seed=12345,
                              partition=1, visit_cost=VISIT, rating_cost=RATING, hop_cost=HOP)
        out["test_rmse"].append(O.rmse(tcsc, W, H))
        out["train_online_rmse"].append(float(np.sqrt(err[0] / nnz)))
        print(f"epoch {e}: test RMSE {out['test_rmse'][-1]:.6f} ({time.time() - t:.1f} s)", flush=True)
        with open(out_path, "w") as f:
            json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
