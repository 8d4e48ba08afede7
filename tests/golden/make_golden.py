"""Generate the golden fixtures of tests/golden/ from independent pure-Python
restatements (no C++ involved), so that the C++ oracle is pinned against them.

  init_seed12345.json   first values of the reference init (Code/nomad/nb_main.cpp:
                        450-455 rows, :70-92 columns): MT19937-64 (Matsumoto &
                        Nishimura's published parameters) feeding libstdc++'s
                        generate_canonical<double, 53> and uniform_real_distribution.
  replay_small.npz      a 30 x 12 problem trained 3 epochs by the one-worker schedule,
                        every float32 / float64 operation rounded one at a time in numpy
                        (nb_main.cpp:513-542; float semantics of nomad_body.hpp:324-357).

Run:  python tests/golden/make_golden.py
"""
import json
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


class MT19937_64:
    """The 64-bit Mersenne Twister (Matsumoto & Nishimura 2000) as std::mt19937_64."""

    N, M = 312, 156
    A = 0xB5026F5AA96619E9
    UPPER, LOWER = 0xFFFFFFFF80000000, 0x7FFFFFFF
    MASK = (1 << 64) - 1

    def __init__(self, seed=5489):
        self.mt = [0] * self.N
        self.mt[0] = seed & self.MASK
        for i in range(1, self.N):
            prev = self.mt[i - 1]
            self.mt[i] = (6364136223846793005 * (prev ^ (prev >> 62)) + i) & self.MASK
        self.idx = self.N

    def _twist(self):
        mt = self.mt
        for i in range(self.N):
            x = (mt[i] & self.UPPER) | (mt[(i + 1) % self.N] & self.LOWER)
            xa = x >> 1
            if x & 1:
                xa ^= self.A
            mt[i] = mt[(i + self.M) % self.N] ^ xa
        self.idx = 0

    def __call__(self):
        if self.idx >= self.N:
            self._twist()
        y = self.mt[self.idx]
        self.idx += 1
        y ^= (y >> 29) & 0x5555555555555555
        y ^= (y << 17) & 0x71D67FFFEDA60000
        y ^= (y << 37) & 0xFFF7EEE000000000
        y ^= y >> 43
        return y & self.MASK


def uniform(rng, b):
    """uniform_real_distribution<double>(0, b) over generate_canonical<double, 53>:
    one 64-bit draw, converted to double and divided by 2^64 (clamped below 1)."""
    u = float(rng()) / 18446744073709551616.0
    if u >= 1.0:
        u = math.nextafter(1.0, 0.0)
    return u * b + 0.0


def reference_init(m, n, dim, seed, nthreads):
    b = 1.0 / math.sqrt(dim)
    W = np.empty(m * dim)
    per = m // nthreads + (1 if m % nthreads else 0)
    for t in range(nthreads):
        lo, hi = min(per * t, m), min(per * (t + 1), m)
        rng = MT19937_64(seed + t + 1)
        for i in range(lo * dim, hi * dim):
            W[i] = uniform(rng, b)
    rng = MT19937_64(seed + 139)
    H = np.array([uniform(rng, b) for _ in range(n * dim)])
    return W.reshape(m, dim), H.reshape(n, dim)


def step_size(lr, dr, cnt, dt):
    if dt == np.float32:
        lr, dr = float(np.float32(lr)), float(np.float32(dr))
    return dt(lr * 1.5 / (1.0 + dr * (cnt + 1) ** 1.5))


def replay(col_ptr, row_idx, vals, W, H, epochs, lr, dr, reg, dt):
    lam = dt(reg)
    v = vals.astype(dt)
    for ep in range(epochs):
        step = step_size(lr, dr, ep, dt)
        for j in range(H.shape[0]):
            col = H[j]
            for o in range(col_ptr[j], col_ptr[j + 1]):
                row = W[row_idx[o]]
                cur = dt(-v[o])
                for i in range(col.size):
                    cur = dt(cur + dt(col[i] * row[i]))
                for i in range(col.size):
                    tmp = row[i]
                    row[i] = dt(row[i] - dt(step * dt(dt(cur * col[i]) + dt(lam * tmp))))
                    col[i] = dt(col[i] - dt(step * dt(dt(cur * tmp) + dt(lam * col[i]))))


def main():
    assert MT19937_64()() == 14514284786278117030  # first output of the default seed
    g = MT19937_64()
    for _ in range(9999):
        g()
    assert g() == 9981545732273789042  # ISO C++ [rand.predef]

    m, n, dim, seed, nthreads = 7, 5, 6, 12345, 3
    W, H = reference_init(m, n, dim, seed, nthreads)
    with open(os.path.join(HERE, "init_seed12345.json"), "w") as f:
        json.dump({"m": m, "n": n, "dim": dim, "seed": seed, "nthreads": nthreads,
                   "W_head": W.ravel()[:24].tolist(), "H_head": H.ravel()[:24].tolist()},
                  f, indent=1)

    rng = np.random.default_rng(20240601)
    m, n, dim, epochs = 30, 12, 8, 3
    cells = rng.choice(m * n, 110, replace=False)
    rows, cols = (cells // n).astype(np.int32), (cells % n).astype(np.int32)
    vals = np.round(rng.normal(0, 1, cells.size), 3)
    order = np.lexsort((rows, cols))
    rows, cols, vals = rows[order], cols[order], vals[order]
    col_ptr = np.zeros(n + 1, np.int64)
    np.cumsum(np.bincount(cols, minlength=n), out=col_ptr[1:])
    W0, H0 = reference_init(m, n, dim, 12345, 1)
    lr, dr, reg = 0.05, 0.1, 0.05
    out = {"col_ptr": col_ptr, "row_idx": rows, "vals": vals, "W0": W0, "H0": H0,
           "epochs": epochs, "lrate": lr, "drate": dr, "reg": reg}
    for kind, dt in (("f32", np.float32), ("f64", np.float64)):
        W, H = W0.astype(dt), H0.astype(dt)
        replay(col_ptr, rows, vals, W, H, epochs, lr, dr, reg, dt)
        out["W_" + kind], out["H_" + kind] = W, H
    np.savez(os.path.join(HERE, "replay_small.npz"), **out)
    print("wrote", os.listdir(HERE))


if __name__ == "__main__":
    main()
