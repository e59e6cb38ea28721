"""Fill the tuner table for a set of tournament shapes and write it to a file
that ``icm_init(path)`` / ``icm_gb300.tuner_load(path)`` reads.

    python -m icm_gb300.tune --out icm_tuner.txt                 # the bench shapes
    python -m icm_gb300.tune --n 50000 --k 5000 --out t.txt      # one shape

Each shape is timed on synthetic stacks of the requested distribution (the
table is keyed by size class only; stacks change the zero-prefix pruning, so
tune on stacks like the production ones)."""
from __future__ import annotations

import argparse

import numpy as np

import icm_gb300 as icm
from icm_gb300 import workloads as W

SHAPES = [("drop-in n=k=65536", lambda: W.dropin()[:2]),
          ("n=16384 k=2000", lambda: W.vjp()[:2]),
          ("n=2000 k=300", lambda: W.batched(count=1, n_lo=2000, n_hi=2000)[0]),
          ("n=200 k=30", lambda: W.batched(count=1, n_lo=200, n_hi=200)[0])]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--n", type=int, default=0)
    ap.add_argument("--k", type=int, default=0)
    ap.add_argument("--Q", type=int, default=256)
    ap.add_argument("--runs", type=int, default=2)
    args = ap.parse_args()
    icm.init()
    shapes = SHAPES
    if args.n:
        k = args.k or args.n
        shapes = [(f"n={args.n} k={k}", lambda: (1e4 * np.exp(np.random.default_rng(1).standard_normal(args.n)),
                                                 W.geometric_payout(k, 0.97)))]
    for name, make in shapes:
        S, P = make()
        b, f, ms = icm.autotune(S, P, Q=args.Q, runs=args.runs)
        print(f"{name}: block_size {b}, fft_min_degree {f}, {ms:.3f} ms")
    print(f"{icm.tuner_save(args.out)} entries written to {args.out}")


if __name__ == "__main__":
    main()
