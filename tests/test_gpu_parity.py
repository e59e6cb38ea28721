"""Parity of the GB300 engine (through the C ABI) with the oracle, the
reference's golden vectors, the reference library's outputs and the exact
closed forms.  Tolerances: 1e-8 relative against the reference (its own
GPU-vs-CPU gate, bench/bench_gpu.cu:157) and 1e-9 against the closed forms,
as the engine's accuracy target states; tighter where the case allows."""
import json
import os

import numpy as np
import pytest

from tests.conftest import GOLDEN, max_rel
from tests.golden.webgen import all_cases
from tests.test_oracle import _regen
from icm_gb300 import workloads as W

pytestmark = pytest.mark.gpu

WEB = json.load(open(os.path.join(GOLDEN, "web_reference.json")))
REFW = json.load(open(os.path.join(GOLDEN, "ref_workloads.json")))
CLOSED = json.load(open(os.path.join(GOLDEN, "closed_form.json")))
WEB_INPUTS = {name: (n, k, Q, S, P) for name, n, k, Q, S, P in all_cases()}

TOL_REF = 1e-8
TOL_EXACT = 1e-9


@pytest.fixture(autouse=True)
def default_config(gpu_icm):
    gpu_icm.configure()
    yield
    gpu_icm.configure()


@pytest.mark.parametrize("case", WEB["cases"], ids=lambda c: c["name"])
def test_reference_golden_vectors(gpu_icm, case):
    n, k, Q, S, P = WEB_INPUTS[case["name"]]
    E = gpu_icm.equity(S, P, Q=Q)
    idx = np.array(case["idx"])
    assert max_rel(E[idx], case["equity"]) < TOL_REF


@pytest.mark.parametrize("case", REFW["cases"], ids=lambda c: c["name"])
def test_reference_library_workloads(gpu_icm, case):
    S, P = _regen(case)
    E = gpu_icm.equity(S, P, Q=case["Q"])
    idx = np.array(case["idx"])
    assert max_rel(E[idx], case["equity"]) < TOL_REF
    if "targets" in case:
        T = case["targets"]
        Es = gpu_icm.equity_subset(S, P, T, Q=case["Q"])
        assert max_rel(Es[T], case["subset_equity"]) < TOL_REF
        assert np.count_nonzero(np.delete(Es, T)) == 0


def test_dropin_full_size_against_closed_form(gpu_icm):
    """n = k = 65536, stacks log-uniform over [1, 1e9], payout (k-j+1)^2:
    the 64 subset targets against E = 2 V2 + 3 V1 - 2 (exact)."""
    S, P, T = W.dropin()
    assert list(T) == CLOSED["targets"]
    Es = gpu_icm.equity_subset(S, P, T)
    assert max_rel(Es[T], CLOSED["equity"]) < TOL_EXACT
    E = gpu_icm.equity(S, P)
    assert max_rel(E[T], CLOSED["equity"]) < TOL_EXACT
    assert max_rel(E[T], Es[T]) < 1e-12
    assert abs(E.sum() - 1.0) < 1e-9


def _stacks(rng, n, dist):
    if dist == "uniform":
        return 1 + 99 * rng.random(n)
    if dist == "loguniform":
        return 10.0 ** (9 * rng.random(n))
    if dist == "equal":
        return np.full(n, 100.0)
    if dist == "adversarial":
        S = np.ones(n)
        S[0] = 1e4
        return S
    S = np.ones(n)        # adv_1e9 (bench/bench.c:83-86)
    S[0] = 1e9
    return S


@pytest.mark.parametrize("n", [1, 2, 3, 7, 8, 9, 16, 17, 33, 100, 257, 1000, 3001])
@pytest.mark.parametrize("dist", ["uniform", "loguniform", "equal", "adversarial"])
def test_against_oracle_shapes(gpu_icm, oracle, n, dist):
    rng = np.random.default_rng(n * 7 + len(dist))
    S = _stacks(rng, n, dist)
    for k in sorted({1, min(3, n), max(1, n // 2), n}):
        P = np.sort(rng.random(k))[::-1] + 0.01
        E = gpu_icm.equity(S, P, Q=128)
        R = oracle.equity(S, P, Q=128, B=8, fft_min_deg=64)
        assert max_rel(E, R, floor=1e-300) < 1e-9, (n, k, dist)


@pytest.mark.parametrize("B", [4, 8, 16, 32])
@pytest.mark.parametrize("fft_min", [4, 16, 64, 1 << 20])
def test_block_size_and_fft_crossover(gpu_icm, oracle, B, fft_min):
    """Every tree level forced through the FFT path, or through schoolbook."""
    gpu_icm.configure(block_size=B, fft_min_degree=fft_min)
    rng = np.random.default_rng(B + fft_min)
    S = 1 + 999 * rng.random(1500)
    for k in (1500, 200, 5):
        P = (k - np.arange(k)).astype(float)
        E = gpu_icm.equity(S, P, Q=64)
        R = oracle.equity(S, P, Q=64, B=B)
        assert max_rel(E, R) < 1e-10, (B, fft_min, k)


@pytest.mark.parametrize("n,dist", [(64, "uniform"), (256, "adversarial"), (1024, "uniform"),
                                    (4096, "adversarial"), (16384, "uniform"), (256, "adv_1e9")])
def test_closed_form_v1(gpu_icm, oracle, n, dist):
    """payout[m] = n - m, k = n: equity = V1 (reference bench/bench.c:699-723)."""
    S = _stacks(np.random.default_rng(42), n, dist)
    P = (n - np.arange(n)).astype(float)
    E = gpu_icm.equity(S, P)
    tol = 1e-9 if dist == "adv_1e9" else 5e-12
    assert max_rel(E, oracle.v1(S)) < tol


def test_closed_form_v2(gpu_icm, oracle):
    """payout C(n-1-m, 2): equity = V2 (reference bench/bench.c:769-798)."""
    n = 200
    S = 1 + 99 * np.random.default_rng(5).random(n)
    r = n - 1 - np.arange(n)
    P = np.where(r >= 2, r * (r - 1) / 2.0, 0.0)
    assert max_rel(gpu_icm.equity(S, P), oracle.v2(S)) < 5e-12


def test_properties(gpu_icm):
    """Reference python/tests/test_icm.py: sums, symmetry, k = 1 closed form."""
    eq = gpu_icm.equity([1000, 1000, 1000], [0.5, 0.3, 0.2])
    assert max_rel(eq, np.full(3, 1 / 3)) < 1e-12
    S = np.array([100.0 * (i + 1) for i in range(10)])
    assert max_rel(gpu_icm.equity(S, [1.0]), S / S.sum()) < 1e-10
    S = 10.0 ** (6 * np.random.default_rng(1).random(5000))
    P = W.geometric_payout(700, 0.9)
    assert abs(gpu_icm.equity(S, P).sum() - 1.0) < 1e-9
    eq = gpu_icm.equity([500, 1000, 1500, 2000, 5000], [0.40, 0.25, 0.18, 0.10, 0.07])
    assert np.all(np.diff(eq) > 0)


def test_subset(gpu_icm, oracle):
    S, P = W.plain_small()
    T = [0, 7, 42, 100, 255, 500, 777, 900, 999, 1023]
    full = gpu_icm.equity(S, P)
    sub = gpu_icm.equity_subset(S, P, T)
    assert max_rel(sub[T], full[T]) < 1e-13
    assert np.count_nonzero(np.delete(sub, T)) == 0
    sub2 = gpu_icm.gpu_equity_subset(S, P, [3])
    assert max_rel(sub2[[3]], full[[3]]) < 1e-13


def test_plan_reuse_and_stats(gpu_icm):
    S, P, _ = W.dropin(n=5000)
    plan = gpu_icm.GpuPlan(S, len(P))
    a, st = plan.equity(P, return_stats=True)
    b = plan.equity(P * 2.0)
    assert max_rel(b, 2.0 * a) < 1e-14
    assert st["total_ns"] > 0 and st["engine"] == 1
    s = plan.summary()
    assert s["n"] == 5000 and s["n_levels"] >= 2
    plan.close()
    assert max_rel(gpu_icm.equity(S, P), a) < 1e-14


def test_batched_matches_single(gpu_icm):
    ts = W.batched(count=12, n_hi=2000)
    res = gpu_icm.equity_batched(ts)
    for (S, P), E in zip(ts, res):
        assert max_rel(E, gpu_icm.equity(S, P)) < 1e-13


def test_deterministic_repeat(gpu_icm):
    S, P, _ = W.dropin(n=20000)
    a = gpu_icm.equity(S, P)
    b = gpu_icm.equity(S, P)
    assert np.array_equal(a, b)


def test_probes(gpu_icm):
    assert gpu_icm.measure_fp64_gflops() > 100.0
    assert gpu_icm.measure_hbm_gbps() > 1000.0


@pytest.mark.parametrize("n", [300, 1025, 4096, 20000])
@pytest.mark.parametrize("kfrac", [1.0, 0.3, 0.01])
def test_spectral_levels_match_coefficient_levels(gpu_icm, n, kfrac):
    """Spectral tree levels (nodes carried as spectra) against the
    coefficient FFT path and the oracle, ragged trees and truncated k included."""
    rng = np.random.default_rng(n)
    S = 10.0 ** (4 * rng.random(n))
    k = max(1, int(kfrac * n))
    P = np.sort(rng.random(k))[::-1] + 0.01
    T = sorted(rng.choice(n, size=min(5, n), replace=False).tolist())
    outs = {}
    for coeff in (False, True):
        gpu_icm.configure(fft_min_degree=16, coefficient_fft_only=coeff)
        outs[coeff] = (gpu_icm.equity(S, P, Q=64), gpu_icm.equity_subset(S, P, T, Q=64))
    assert max_rel(outs[False][0], outs[True][0]) < 1e-11
    assert max_rel(outs[False][1][T], outs[True][0][T]) < 1e-11
    assert np.count_nonzero(np.delete(outs[False][1], T)) == 0


@pytest.mark.parametrize("wl", ["lognormal", "loguniform", "adv_1e9", "batched"])
def test_zero_prefix_pruning_matches_full_tree(gpu_icm, oracle, wl):
    """Tree nodes whose players all have a leaf factor of exactly 0 at a node
    are written as monomials / skipped; equities equal the full tree's to
    rounding, spectral and coefficient levels, single and batched."""
    rng = np.random.default_rng(17)
    if wl == "batched":
        ts = W.batched(count=24)
        outs = []
        for zp in (True, False):
            gpu_icm.configure(zero_prefix=zp)
            outs.append(gpu_icm.equity_batched(ts))
        for a, b in zip(*outs):
            assert max_rel(a, b, floor=1e-300) < 1e-11
        return
    n = 30000
    if wl == "lognormal":
        S, P = W.gpu_scale(n=n, shape="linear")
    elif wl == "loguniform":
        S, P, _ = W.dropin(n=n)
    else:
        S = np.ones(n)
        S[:50] = 1e9
        P = (n - np.arange(n)).astype(float)
    for coeff in (False, True):
        res = []
        for zp in (True, False):
            gpu_icm.configure(zero_prefix=zp, coefficient_fft_only=coeff)
            res.append(gpu_icm.equity(S, P))
        assert max_rel(res[0], res[1], floor=1e-300) < 1e-11, coeff
    if wl == "lognormal":   # k = n linear: closed form
        idx = rng.choice(n, 32, replace=False)
        ref = oracle.v1(S, idx=idx) * (P[0] / n)
        assert max_rel(res[0][idx], ref) < 1e-9


def test_autotune_and_table(gpu_icm, oracle, tmp_path):
    """The search returns a candidate, records it for the size class, plans
    of that class use it, and results stay on the oracle."""
    gpu_icm.tuner_clear()
    S, P = W.batched(count=1, n_lo=3000, n_hi=3000)[0]
    b, f, ms = gpu_icm.autotune(S, P, Q=64, runs=1)
    assert b in (4, 8, 16) and f in (16, 32, 64, 128) and ms > 0
    assert gpu_icm.tuner_lookup(len(S), len(P)) == (b, f)
    path = tmp_path / "tuner.txt"
    saved = gpu_icm.tuner_save(path)   # the class entry and any per-level entries
    assert saved >= 1
    gpu_icm.tuner_clear()
    assert gpu_icm.tuner_load(path) == saved
    plan = gpu_icm.GpuPlan(S, len(P))
    assert plan.summary()["B"] == b
    E = plan.equity(P, Q=64)
    plan.close()
    assert max_rel(E, oracle.equity(S, P, Q=64, B=8, fft_min_deg=64), floor=1e-300) < 1e-9
    gpu_icm.tuner_clear()


def test_per_level_tuning_stable_and_close(gpu_icm, tmp_path):
    """Per-level tuner entries (a level kept on coefficients, other points per
    CTA) change the plan's kernels, not its result beyond rounding: a tuned
    plan repeats itself bit for bit and stays within 1e-12 of the default
    plan (normwise, and per player above 1e-12 of the largest equity)."""
    gpu_icm.tuner_clear()
    S, P, _ = W.dropin(n=16384)
    plan = gpu_icm.GpuPlan(S, len(P))
    E0 = plan.equity(P)
    plan.close()
    path = tmp_path / "levels.txt"
    path.write_text("tune_level 14 3 5 0 0 1.0\ntune_level 14 3 7 1 1024 1.0\ntune_level 14 3 9 1 8192 1.0\n")
    assert gpu_icm.tuner_load(path) == 3
    assert gpu_icm.tuner_lookup_level(len(S), len(P), 5) == (0, 0)
    plan = gpu_icm.GpuPlan(S, len(P))
    E1, E2 = plan.equity(P), plan.equity(P)
    plan.close()
    assert np.array_equal(E1, E2)
    scale = float(np.abs(E0).max())
    assert float(np.abs(E1 - E0).max()) <= 1e-12 * scale
    assert max_rel(E1, E0, floor=1e-12 * scale) < 1e-12
    # the search itself: every level entry it records names a spectral level
    gpu_icm.tuner_clear()
    b, f, ms = gpu_icm.autotune(S, P, Q=32, runs=1)
    plan = gpu_icm.GpuPlan(S, len(P))
    E3, E4 = plan.equity(P), plan.equity(P)
    plan.close()
    assert np.array_equal(E3, E4)
    assert max_rel(E3, E0, floor=1e-11 * scale) < 1e-11
    for lev in range(1, 15):
        e = gpu_icm.tuner_lookup_level(len(S), len(P), lev)
        assert e is None or (e[0] in (0, 1) and e[1] in (0, 1024, 2048, 8192))
    gpu_icm.tuner_clear()


def test_plan_targets_match_one_shot_subset(gpu_icm):
    """A resident plan's subset state gives the one-shot subset query's
    equities bit for bit, and clearing it the full field's."""
    S, P, T = W.dropin(n=20000, n_targets=40)
    full = gpu_icm.gpu_equity(S, P)
    sub = gpu_icm.gpu_equity_subset(S, P, T)
    plan = gpu_icm.GpuPlan(S, len(P))
    plan.set_targets(T)
    assert np.array_equal(plan.equity(P), sub)
    plan.set_targets(None)
    assert np.array_equal(plan.equity(P), full)
    with pytest.raises(gpu_icm.ICMError):
        plan.set_targets([0, len(S)])
    plan.close()


def test_quadrature_ladder(gpu_icm, oracle):
    """Q doubles until successive rules agree; the result is the oracle's at that Q."""
    S, P, _ = W.vjp(n=4096, k=600)
    E, Q, err = gpu_icm.equity_adaptive(S, P, tol=1e-9, Q0=128, Qmax=8192)
    assert Q > 128 and err <= 1e-9
    assert max_rel(E, oracle.equity(S, P, Q=Q), floor=1e-12 * np.abs(E).max()) < 1e-9
    E2, Q2, err2 = gpu_icm.equity_adaptive(S, P, tol=1e-30, Q0=128, Qmax=512)   # capped
    assert Q2 == 512 and err2 > 0


@pytest.mark.parametrize("B,fft_min", [(4, 128), (8, 64), (16, 1 << 20), (32, 64), (8, 8)])
def test_subtree_kernels_equal_level_by_level(gpu_icm, B, fft_min):
    """Leaf blocks and bottom schoolbook levels fused per direction: the same
    arithmetic as the level-by-level kernels, so bitwise equal results (full
    query, subset, batched)."""
    rng = np.random.default_rng(B + fft_min)
    S = 10.0 ** (5 * rng.random(7001))
    P = np.sort(rng.random(900))[::-1]
    T = sorted(rng.choice(len(S), size=9, replace=False).tolist())
    ts = W.batched(count=10)
    out = []
    for sub in (True, False):
        gpu_icm.configure(block_size=B, fft_min_degree=fft_min, subtree=sub)
        out.append((gpu_icm.equity(S, P, Q=64), gpu_icm.equity_subset(S, P, T, Q=64),
                    gpu_icm.equity_batched(ts, Q=32)))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])
    for a, b in zip(out[0][2], out[1][2]):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("n,k", [(40, 40), (3000, 450), (20000, 20000)])
def test_plan_graph_replay(gpu_icm, n, k):
    """IcmGpuOptions.enable_graphs: the run is captured once per node count and
    replayed; results equal the direct launches bit for bit (small path, tree
    levels, new payouts and node counts)."""
    from icm_gb300._lib import IcmGpuOptions
    rng = np.random.default_rng(n)
    S = 1e4 * np.exp(rng.standard_normal(n))
    P1, P2 = 0.8 ** np.arange(k), np.linspace(1.0, 0.1, k)
    direct = gpu_icm.GpuPlan(S, k)
    graphed = gpu_icm.GpuPlan(S, k, IcmGpuOptions(enable_graphs=1))
    for P, Q in [(P1, 256), (P2, 256), (P1, 128), (P2, 256)]:
        a, b = direct.equity(P, Q=Q), graphed.equity(P, Q=Q)
        assert np.array_equal(a, b), (n, k, Q)
    direct.close()
    graphed.close()


def test_verbose_stage_times(gpu_icm):
    """IcmGpuOptions.verbose: per-stage device times in IcmGpuRunStats (block
    build, tree build, propagate, leaf extraction), as the reference's
    instrumented path reports them; the results do not change."""
    from icm_gb300._lib import IcmGpuOptions
    rng = np.random.default_rng(31)
    S = 1e4 * np.exp(rng.standard_normal(20000))
    P = 0.8 ** np.arange(3000)
    gpu_icm.configure(q_chunk=100)   # three chunks: stage times add up over chunks
    plain = gpu_icm.GpuPlan(S, len(P))
    verbose = gpu_icm.GpuPlan(S, len(P), IcmGpuOptions(verbose=1))
    a = plain.equity(P)
    b, st = verbose.equity(P, return_stats=True)
    gpu_icm.configure()
    assert np.array_equal(a, b)
    stages = [st["block_build_ns"], st["tree_build_ns"], st["tree_propagate_cached_ns"], st["leaf_extract_ns"]]
    assert all(x > 0 for x in stages), stages
    assert sum(stages) <= st["total_ns"]
    plain.close()
    verbose.close()


def test_one_shot_plan_reuse(gpu_icm):
    """Repeated one-shot calls of one shape reuse the thread's last plan with
    new stacks; results equal fresh plans bit for bit, and a configuration
    change is not served by a plan built under the old one."""
    rng = np.random.default_rng(77)
    n, k = 3000, 450
    P = 0.9 ** np.arange(k)
    stacks = [1e4 * np.exp(s * rng.standard_normal(n)) for s in (1.0, 2.0, 0.5, 1.0)]

    def fresh(S):
        p = gpu_icm.GpuPlan(S, k)
        e = p.equity(P)
        p.close()
        return e
    for S in stacks:
        assert np.array_equal(gpu_icm.gpu_equity(S, P), fresh(S))
    gpu_icm.configure(block_size=16, fft_min_degree=32)
    try:
        for S in stacks[:2]:
            assert np.array_equal(gpu_icm.gpu_equity(S, P), fresh(S))
    finally:
        gpu_icm.configure()
    assert np.array_equal(gpu_icm.gpu_equity(stacks[0], P), fresh(stacks[0]))


def test_one_shot_subset_reuses_plan(gpu_icm):
    """Subset queries take the thread's cached plan too and set their targets
    for that run only: subset and full one-shot calls of one shape, in any
    order, with new stacks and with captured graphs, equal the same queries
    on fresh plans (the subset's non-targets stay 0, a full call after a
    subset call is not pruned)."""
    from icm_gb300._lib import IcmGpuOptions, lib
    import ctypes
    rng = np.random.default_rng(78)
    n, k = 6000, 600
    P = 0.9 ** np.arange(k)
    T = np.array([0, 5, 2999, 5999], dtype=np.int32)
    stacks = [1e4 * np.exp(s * rng.standard_normal(n)) for s in (1.0, 2.0)]
    dp, ip = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)

    def subset(S, opts):
        out = np.zeros(n)
        assert lib().icm_gpu_equity_subset(n, S.ctypes.data_as(dp), 256, P.ctypes.data_as(dp), k,
                                           out.ctypes.data_as(dp), T.ctypes.data_as(ip), len(T),
                                           ctypes.byref(opts) if opts else None, None) == 0
        return out

    def full(S, opts):
        out = np.zeros(n)
        assert lib().icm_gpu_equity(n, S.ctypes.data_as(dp), 256, P.ctypes.data_as(dp), k,
                                    out.ctypes.data_as(dp), ctypes.byref(opts) if opts else None, None) == 0
        return out

    def evict():   # another shape replaces the cached plan
        gpu_icm.gpu_equity(np.linspace(1.0, 2.0, 2500), np.ones(3))

    sub_ref, full_ref = [], []
    for S in stacks:
        evict()
        sub_ref.append(subset(S, None))   # on a fresh plan
        plan = gpu_icm.GpuPlan(S, k)
        full_ref.append(plan.equity(P))
        plan.close()
        assert np.count_nonzero(np.delete(sub_ref[-1], T)) == 0
    for opts in (None, IcmGpuOptions(enable_graphs=1)):
        evict()
        for j in (0, 1, 0, 1):
            assert np.array_equal(subset(stacks[j], opts), sub_ref[j])
            assert np.array_equal(full(stacks[j], opts), full_ref[j])
            assert np.array_equal(subset(stacks[j], opts), sub_ref[j])
