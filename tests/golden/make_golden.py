"""Regenerate the golden fixtures in tests/golden/ (run in a tree where the
reference is available; the GPU host never runs this).

Writes:
  web_reference.json   the reference's own golden vectors
                       (web/verify/reference.json): equities only, at all
                       indices for n <= 300 and at 120 sampled indices above;
                       inputs are rebuilt by webgen.py, which is checked here
                       against the JSON bit for bit.
  ref_workloads.json   equities from the reference's src/cpu/icm.c (compiled
                       unmodified into oracle/_ref) on seeded workloads of the
                       shapes the benchmarks use, at sizes the CPU finishes in
                       minutes, plus the full-size drop-in workload's subset.
  closed_form.json     exact closed-form equities (no quadrature) for the
                       full-size drop-in workload's 64 subset targets:
                       payout (k-j+1)^2 with k = n gives E = 2 V2 + 3 V1 - 2
                       (unnormalised), from oracle V1/V2.
  ref_gpu_scale_geometric.json  the reference's own icm_equity_subset on the
                       GPU-only scale workload with geometric payouts (n = 2^20,
                       k = 1000, Q = 256) at 16 seeded targets (minutes on the
                       CPU: the full field would take hours).
  vjp_fd_reference.json  directional derivatives of L = <cot, equity> taken
                       by central finite differences of the reference's own
                       icm_equity (oracle/_ref): along stacks S -> S (1 + h u)
                       at h = 1e-6 and a Richardson pair h = 1e-4 / 5e-5, with
                       u = 0 on stacks within 1% of the largest so that the
                       quadrature nodes (which depend on max S) stay fixed;
                       and along a payout
                       direction v, where L is linear: <cot, icm_equity(S, v)>.

Usage:  python tests/golden/make_golden.py [--skip-large] [--only NAME]
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from icm_gb300 import workloads as W  # noqa: E402
from oracle.oracle import Oracle, ReferenceLib, build  # noqa: E402
from tests.golden.webgen import all_cases  # noqa: E402

REF_JSON = os.path.join(os.environ.get("ICM_REFERENCE_DIR", "/root/reference"),
                        "web", "verify", "reference.json")


def sample_idx(n: int, count: int, S: np.ndarray | None = None) -> np.ndarray:
    if n <= count:
        return np.arange(n)
    idx = set(np.linspace(0, n - 1, count - 2).astype(int).tolist())
    if S is not None:
        idx.add(int(np.argmin(S)))
        idx.add(int(np.argmax(S)))
    return np.array(sorted(idx))


def fl(a):
    return [float(x) for x in a]


def web_fixture():
    ref = json.load(open(REF_JSON))
    out = []
    for (name, n, k, Q, S, P), c in zip(all_cases(), ref):
        assert c["name"] == name and c["n"] == n and c["k"] == k and c["Q"] == Q
        assert np.array_equal(S, np.array(c["stacks"])), name
        assert np.array_equal(P, np.array(c["payouts"])), name
        E = np.array(c["equity"])
        idx = np.arange(n) if n <= 300 else sample_idx(n, 120, S)
        out.append({"name": name, "n": n, "k": k, "Q": Q,
                    "idx": idx.tolist(), "equity": fl(E[idx])})
    return {"source": "web/verify/reference.json (reference native build)", "cases": out}


def workload_fixture(ref: ReferenceLib, skip_large: bool):
    cases = []

    def add(name, S, P, Q=256, targets=None, count=256, meta=None):
        t0 = time.time()
        E = ref.equity(S, P, Q=Q)
        rec = {"name": name, "n": len(S), "k": len(P), "Q": Q,
               "sum_S": float(S.sum()), "sum_P": float(P.sum()), **(meta or {})}
        idx = sample_idx(len(S), count, S)
        rec["idx"] = idx.tolist()
        rec["equity"] = fl(E[idx])
        if targets is not None:
            Es = ref.equity(S, P, Q=Q, targets=targets)
            rec["targets"] = [int(t) for t in targets]
            rec["subset_equity"] = fl(Es[targets])
            rec["full_at_targets"] = fl(E[targets])
        print(f"  {name}: n={len(S)} k={len(P)} {time.time() - t0:.1f}s", flush=True)
        cases.append(rec)

    S, P = W.plain_small()
    add("plain_small", S, P, count=1024, meta={"gen": "plain_small()"})
    S, P, T = W.dropin(n=4096)
    add("dropin_4096", S, P, targets=T, meta={"gen": "dropin(n=4096)"})
    S, P, T = W.dropin(n=3000, k=3000, n_targets=17)
    add("dropin_3000_ragged", S, P, targets=T, meta={"gen": "dropin(n=3000, k=3000, n_targets=17)"})
    S, P = W.gpu_scale(n=8192, shape="linear")
    add("gpu_scale_8192_linear", S, P, meta={"gen": "gpu_scale(n=8192, shape='linear')"})
    S, P = W.gpu_scale(n=8192, shape="geometric")
    add("gpu_scale_8192_geometric", S, P, meta={"gen": "gpu_scale(n=8192, shape='geometric')"})
    for i, (S, P) in enumerate(W.batched(count=24, n_hi=3000)):
        add(f"batched_small_{i}", S, P, count=32, meta={"gen": "batched(count=24, n_hi=3000)", "member": i})
    for shape in ("linear", "quadratic"):
        S, P, _ = W.vjp(n=2048, k=256, payout=shape)
        add(f"vjp_2048_{shape}", S, P, count=128, meta={"gen": f"vjp(n=2048, k=256, payout='{shape}')"})
    if not skip_large:
        S, P, T = W.dropin()
        add("dropin_65536", S, P, targets=T, count=128, meta={"gen": "dropin()"})
    return {"source": "reference src/cpu/icm.c via oracle/_ref (FFTW shim, devices/generic, OpenMP)",
            "cases": cases}


def closed_form_fixture(orc: Oracle):
    S, P, T = W.dropin()
    n = len(S)
    t0 = time.time()
    v1 = orc.v1(S, idx=T)
    v2 = orc.v2(S, idx=T)
    r = np.arange(n, dtype=np.float64)[::-1]            # r = n-1-m
    norm = float(np.sum((r + 1.0) ** 2))
    exact = (2.0 * v2 + 3.0 * v1 - 2.0) / norm
    print(f"  closed form n={n}: {time.time() - t0:.1f}s", flush=True)
    return {"source": "oracle V1/V2 closed forms, E = (2 V2 + 3 V1 - 2) / sum (n-m)^2",
            "gen": "dropin()", "n": n, "targets": [int(t) for t in T], "equity": fl(exact)}


# the VJP cases: (name, generator call, directions); stacks, payouts and the
# cotangent come from icm_gb300.workloads, directions from splitmix64 normals
VJP_CASES = [
    ("vjp_16384_linear", "vjp(payout='linear')", 3),
    ("vjp_16384_quadratic", "vjp(payout='quadratic')", 3),
    ("dropin_2048_kn", "dropin(n=2048)", 3),
]


def vjp_inputs(gen: str, seed: int):
    """(S, P, cot) of a VJP fixture case; the drop-in shape (k = n) gets a
    splitmix64 N(0, 1) cotangent from `seed`."""
    out = eval("W." + gen)   # noqa: S307 -- generator calls of this module's own table
    if gen.startswith("vjp("):
        return out
    S, P, _ = out
    return S, P, W.SplitMix64(seed).normal(len(S))


def stack_direction(S, seed: int):
    """A splitmix64 N(0, 1) direction that keeps max S (and with it the
    quadrature nodes) fixed: stacks within 1% of the largest are not moved,
    so no step changes which player sets the nodes."""
    u = W.SplitMix64(seed).normal(len(S))
    u[S > 0.99 * np.max(S)] = 0.0
    return u


def vjp_fd_fixture(ref: ReferenceLib):
    cases = []
    for name, gen, ndir in VJP_CASES:
        t0 = time.time()
        S, P, cot = vjp_inputs(gen, 9001)

        def loss(x, pay=P):
            return float(np.dot(cot, ref.equity(x, pay)))

        dirs = []
        for d in range(ndir):
            seed = 7000 + d
            u = stack_direction(S, seed)
            fd = {}
            for h in (1e-6, 1e-4, 5e-5):
                fd[h] = (loss(S * (1.0 + h * u)) - loss(S * (1.0 - h * u))) / (2.0 * h)
            rich = (4.0 * fd[5e-5] - fd[1e-4]) / 3.0
            dirs.append({"seed": seed, "fd_1e-6": fd[1e-6], "fd_richardson": rich})
        v = W.SplitMix64(8000).normal(len(P))
        rec = {"name": name, "gen": gen, "cot_seed": 9001, "n": len(S), "k": len(P), "Q": 256,
               "L": loss(S), "stack_directions": dirs,
               "payout_direction": {"seed": 8000, "derivative": loss(S, v)}}
        print(f"  {name}: n={len(S)} k={len(P)} {time.time() - t0:.1f}s", flush=True)
        cases.append(rec)
    return {"source": "central differences of the reference's src/cpu/icm.c icm_equity (oracle/_ref, OpenMP), "
                      "Q = 256", "cases": cases}


def scale_geometric_fixture(ref: ReferenceLib):
    S, P = W.gpu_scale(shape="geometric")
    T = np.sort(np.random.default_rng(20).choice(len(S), 16, replace=False)).astype(np.int32)
    t0 = time.time()
    E = ref.equity(S, P, Q=256, targets=T)
    print(f"  gpu_scale geometric n={len(S)} k={len(P)}: {time.time() - t0:.1f}s", flush=True)
    return {"source": "reference src/cpu/icm.c icm_equity_subset via oracle/_ref (FFTW shim, devices/generic, OpenMP)",
            "gen": "gpu_scale(shape='geometric')", "n": len(S), "k": len(P), "Q": 256,
            "targets": [int(t) for t in T], "subset_equity": fl(E[T])}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--skip-large", action="store_true")
    ap.add_argument("--only", choices=["vjp_fd", "scale_geometric"], default=None,
                    help="regenerate only this fixture")
    args = ap.parse_args()
    build()
    ref = ReferenceLib(openmp=True)
    orc = Oracle()
    if args.only == "scale_geometric":
        print("ref_gpu_scale_geometric.json")
        json.dump(scale_geometric_fixture(ref), open(os.path.join(HERE, "ref_gpu_scale_geometric.json"), "w"))
        return
    if args.only == "vjp_fd":
        print("vjp_fd_reference.json")
        json.dump(vjp_fd_fixture(ref), open(os.path.join(HERE, "vjp_fd_reference.json"), "w"), indent=1)
        return
    print("web_reference.json")
    json.dump(web_fixture(), open(os.path.join(HERE, "web_reference.json"), "w"))
    print("ref_workloads.json")
    json.dump(workload_fixture(ref, args.skip_large), open(os.path.join(HERE, "ref_workloads.json"), "w"))
    if not args.skip_large:
        print("closed_form.json")
        json.dump(closed_form_fixture(orc), open(os.path.join(HERE, "closed_form.json"), "w"))
    print("vjp_fd_reference.json")
    json.dump(vjp_fd_fixture(ref), open(os.path.join(HERE, "vjp_fd_reference.json"), "w"), indent=1)
    if not args.skip_large:
        print("ref_gpu_scale_geometric.json")
        json.dump(scale_geometric_fixture(ref), open(os.path.join(HERE, "ref_gpu_scale_geometric.json"), "w"))


if __name__ == "__main__":
    main()
