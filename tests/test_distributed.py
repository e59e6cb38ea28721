"""The node-range split of the quadrature over torch.distributed ranks
(icm_gb300/distributed.py), on CPU: world_size 2 over gloo, each rank's part
computed by a numpy restatement of the per-node sum at the oracle's nodes
(test infrastructure standing in for the GPU plan), then one all-reduce.
Checks the ranges, that every rank gets the full equities, and that they
match the oracle's whole-Q solve.  Tolerance 1e-12 relative (rounding of
the restatement against the oracle's FFT tree)."""
import os
import socket

import numpy as np
import pytest
from numpy.polynomial import polynomial as Pm

from icm_gb300.distributed import node_ranges


def test_node_ranges():
    for Q in (1, 2, 7, 256, 257):
        for W in (1, 2, 3, 8):
            r = node_ranges(Q, W)
            assert len(r) == W and r[0][0] == 0 and r[-1][1] == Q
            assert all(a[1] == b[0] for a, b in zip(r, r[1:]))
            sizes = [e - b for b, e in r]
            assert max(sizes) - min(sizes) <= 1 and sizes == sorted(sizes, reverse=True)
    with pytest.raises(ValueError):
        node_ranges(0, 2)


def test_weighted_node_ranges():
    rng = np.random.default_rng(11)
    for Q in (1, 5, 256):
        w = rng.integers(0, 1000, Q).astype(float)
        for W in (1, 2, 3, 8):
            r = node_ranges(Q, W, w)
            assert len(r) == W and r[0][0] == 0 and r[-1][1] == Q
            assert all(a[1] == b[0] and a[0] <= a[1] for a, b in zip(r, r[1:]))
            sums = [w[b:e].sum() for b, e in r]
            assert max(sums) - w.sum() / W <= w.max() + 1e-9    # within one node's weight of an equal share
    assert node_ranges(4, 2, [0, 0, 0, 0]) == [(0, 0), (0, 4)]
    with pytest.raises(ValueError):
        node_ranges(4, 2, [1.0, 2.0])


def test_node_work_counts_players_outside_the_zero_prefix(oracle):
    """icm_gb300_node_work: n - (players with S logv < -700) per node of the
    rule, 0 for weight-0 nodes; the oracle's nodes give the same counts."""
    from icm_gb300 import workloads as W
    from icm_gb300.distributed import node_work
    S, _, _ = W.dropin(n=5000)
    Q = 256
    work = node_work(S, Q)
    logv, w = oracle.nodes(Q, float(S.max()))
    ref = np.array([0 if w[q] == 0.0 else int(np.sum(S * logv[q] >= -700.0)) for q in range(Q)])
    assert np.array_equal(work, ref)
    assert work.min() < work.max() == len(S)      # the spread stacks give uneven nodes


def partial_restated(oracle_path, stacks, payouts, Q, qb, qe):
    """sum over nodes q in [qb, qe) with w_q != 0 of w_q S_i a_i / v_q
    <payout, prod_{j != i} (a_j + (1 - a_j) x) mod x^k> (a = 0 when S logv < -700)."""
    from oracle.oracle import Oracle
    orc = Oracle(oracle_path)
    logv, w = orc.nodes(Q, float(np.max(stacks)))
    S, P = np.asarray(stacks), np.asarray(payouts)
    n, k = len(S), len(P)
    E = np.zeros(n)
    for q in range(qb, qe):
        if w[q] == 0.0:
            continue
        arg = S * logv[q]
        a = np.where(arg < -700.0, 0.0, np.exp(arg))
        for i in range(n):
            poly = np.array([1.0])
            for j in range(n):
                if j != i:
                    poly = Pm.polymul(poly, [a[j], 1.0 - a[j]])[:k]
            pw = w[q] * S[i] * a[i] * np.exp(-logv[q])
            if np.isfinite(pw):
                E[i] += pw * np.dot(P[: len(poly)], poly)
    return E


def _rank(rank, world, port, stacks, payouts, Q, oracle_path, out_dir):
    import torch.distributed as dist
    from icm_gb300 import distributed as D
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        E = D.equity(stacks, payouts, Q=Q,
                     partial=lambda S, P, Qq, b, e: partial_restated(oracle_path, S, P, Qq, b, e))
        np.save(os.path.join(out_dir, f"rank{rank}.npy"), E)
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_node_split_gloo_world2(oracle, tmp_path):
    import torch.multiprocessing as mp
    rng = np.random.default_rng(5)
    S = 10.0 ** (3 * rng.random(7))
    P = np.array([0.5, 0.3, 0.2])
    Q = 48
    mp.spawn(_rank, args=(2, _free_port(), S, P, Q, None, str(tmp_path)), nprocs=2, join=True)
    r0, r1 = np.load(tmp_path / "rank0.npy"), np.load(tmp_path / "rank1.npy")
    assert np.array_equal(r0, r1)
    ref = oracle.equity(S, P, Q=Q)
    assert np.max(np.abs(r0 - ref) / np.abs(ref)) < 1e-12
