"""Concurrent host threads (ctypes releases the GIL during calls): one-shot
solves on the small path and the plan path, reused plans, batches and VJPs
from several threads at once give the same bits as the same calls made one
after another; errors stay with the thread that made them."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _jobs(gpu_icm, seed):
    rng = np.random.default_rng(seed)
    small = (1e3 * np.exp(rng.standard_normal(37)), 0.8 ** np.arange(9))
    mid = (1e4 * np.exp(rng.standard_normal(3000)), 0.9 ** np.arange(400))
    ts = [(1e3 * np.exp(rng.standard_normal(n)), 0.8 ** np.arange(max(1, n // 5))) for n in (20, 700, 2500)]
    cot = rng.standard_normal(len(mid[0]))

    def run():
        out = [gpu_icm.gpu_equity(*small), gpu_icm.gpu_equity(*mid)]
        plan = gpu_icm.GpuPlan(mid[0], len(mid[1]))
        out += [plan.equity(mid[1]), plan.equity(mid[1])]
        plan.close()
        out += gpu_icm.equity_batched(ts)
        out += list(gpu_icm.equity_vjp(mid[0], mid[1], cot))
        return out
    return run


def test_concurrent_threads_match_serial(gpu_icm):
    jobs = [_jobs(gpu_icm, s) for s in range(4)]
    serial = [job() for job in jobs]
    results, errors = [None] * len(jobs), []

    def worker(i):
        try:
            for _ in range(3):
                results[i] = jobs[i]()
        except Exception as e:   # reported below
            errors.append(repr(e))
    threads = [threading.Thread(target=worker, args=(i,)) for i in range(len(jobs))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    for got, ref in zip(results, serial):
        assert len(got) == len(ref)
        for a, b in zip(got, ref):
            assert np.array_equal(a, b)


def test_errors_stay_with_their_thread(gpu_icm):
    from icm_gb300._lib import lib
    msgs = {}

    def bad():
        lib().icm_gpu_equity(3, None, 256, None, 5, None, None, None)   # invalid: k > n, null arrays
        msgs["bad"] = lib().icm_gpu_last_error()

    def good():
        gpu_icm.gpu_equity(np.array([1.0, 2.0, 3.0]), np.array([0.6, 0.4]))
        msgs["good"] = lib().icm_gpu_last_error()
    t1, t2 = threading.Thread(target=bad), threading.Thread(target=good)
    t1.start(); t2.start(); t1.join(); t2.join()
    assert b"invalid" in msgs["bad"]
    assert b"invalid" not in msgs["good"]


def test_large_one_shot_plans_from_threads(gpu_icm):
    """One-shot solves whose plans (several GB of arena each) are kept per
    thread while the process-wide budget allows: three threads solving
    drop-in fields twice each give the serial results bit for bit, whichever
    of their plans were kept."""
    from icm_gb300 import workloads as W
    fields = [W.dropin(n=40000 + 1000 * i)[:2] for i in range(3)]
    serial = [gpu_icm.equity(S, P) for S, P in fields]
    results, errors = [None] * 3, []

    def worker(i):
        try:
            for _ in range(2):
                results[i] = gpu_icm.equity(*fields[i])
        except Exception as e:   # reported below
            errors.append(repr(e))
    threads = [threading.Thread(target=worker, args=(i,)) for i in range(3)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    for got, ref in zip(results, serial):
        assert np.array_equal(got, ref)
