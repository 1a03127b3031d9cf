"""Known-answer fixtures for fromfile1, in the reference's file formats.

Writes <name>.in (n, then the n rows of A, then the n rows of B), <name>.correct
(the n rows of C = A * B, exact) and <name>.params (every valid one-GPU
`fromfile1 -b bs -r r` line), the formats of the reference's tests/ directory
(generateTest.py:56-99 describes them; fromfile1.cpp:45-57 reads them).  Entries
are integers in [lo, hi], so the exact product is known and Strassen must
reproduce it bit for bit.  numpy does the product in int64, so sizes in the
thousands take seconds.

    python caps_gb300/drivers/generate_test.py 448 tests_out/test448 [--lo 1 --hi 5 --seed 0]
"""
from __future__ import annotations

import argparse
import os

import numpy as np


def valid_params(n: int):
    """(bs, r) pairs fromfile1 accepts on one GPU: n % (2^r * bs) == 0."""
    out = []
    r = 0
    while n % (1 << r) == 0:
        m = n >> r
        for bs in range(1, m + 1):
            if m % bs == 0:
                out.append((bs, r))
        r += 1
    return out


def write_matrix(f, M: np.ndarray) -> None:
    for row in M:
        f.write(" ".join(str(int(v)) for v in row))
        f.write("\n")


def generate(n: int, base: str, lo: int = 1, hi: int = 5, seed: int = 0):
    rng = np.random.default_rng(seed)
    A = rng.integers(lo, hi + 1, (n, n), dtype=np.int64)
    B = rng.integers(lo, hi + 1, (n, n), dtype=np.int64)
    C = A @ B
    d = os.path.dirname(base)
    if d:
        os.makedirs(d, exist_ok=True)
    with open(base + ".in", "w") as f:
        f.write("%d\n" % n)
        write_matrix(f, A)
        write_matrix(f, B)
    with open(base + ".correct", "w") as f:
        write_matrix(f, C)
    name = os.path.basename(base)
    with open(base + ".params", "w") as f:
        for bs, r in valid_params(n):
            f.write("./fromfile1 -i %s.in -b %d -r %d -c %s.correct\n" % (name, bs, r, name))
    return A, B, C


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("n", type=int)
    ap.add_argument("base", help="output path without extension")
    ap.add_argument("--lo", type=int, default=1)
    ap.add_argument("--hi", type=int, default=5)
    ap.add_argument("--seed", type=int, default=0)
    a = ap.parse_args()
    generate(a.n, a.base, a.lo, a.hi, a.seed)


if __name__ == "__main__":
    main()
