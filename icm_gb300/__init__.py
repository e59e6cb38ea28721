"""GB300-native ICM equity engine (sm_103a), Python binding.

Drop-in for the reference's ``icm`` package (python/icm/__init__.py): the same
``init``, ``equity``, ``equity_subset`` and ``ICMError`` with the same argument
checks and messages, reaching ``libicm_gb300.so`` through ctypes.  The
computation runs on the GPU; if the library or a GPU is missing the calls
raise ``ICMError`` (there is no CPU fallback).

Additions: ``gpu_equity`` (with run statistics), ``GpuPlan`` (reusable
tournament plan), ``equity_batched`` (many tournaments), ``configure``
(block size / FFT crossover / chunking) and the FP64 peak probe.

Example::

    import icm_gb300 as icm
    icm.init()
    eq = icm.equity([1000, 2000, 3000], [0.5, 0.3, 0.2])
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from ._lib import (IcmGb300Config, IcmGpuOptions, IcmGpuPlanSummary, IcmGpuRunStats, ICMError, lib,
                   library_path)

__all__ = ["init", "equity", "equity_subset", "ICMError", "gpu_equity", "gpu_equity_subset", "GpuPlan",
           "equity_batched", "GpuBatch", "GpuVjpBatch", "player_order", "equity_vjp", "equity_vjp_batched", "VjpPlan", "autotune", "tuner_load",
           "tuner_save", "tuner_clear", "tuner_lookup", "equity_adaptive", "configure", "measure_fp64_gflops", "measure_hbm_gbps", "library_path",
           "last_launch_count"]

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def _to_double_array(data, name):
    arr = np.ascontiguousarray(data, dtype=np.float64)
    if arr.ndim != 1:
        raise ValueError(f"{name} must be a 1-D array, got shape {arr.shape}")
    if arr.size == 0:
        raise ValueError(f"{name} must not be empty")
    return arr


def _to_int_array(data, name):
    arr = np.ascontiguousarray(data, dtype=np.int32)
    if arr.ndim != 1:
        raise ValueError(f"{name} must be a 1-D array, got shape {arr.shape}")
    if arr.size == 0:
        raise ValueError(f"{name} must not be empty")
    return arr


def _d(a):
    return a.ctypes.data_as(_dp)


def _check(n, k, Q):
    if k < 1 or k > n:
        raise ValueError(f"payouts length k={k} must satisfy 1 <= k <= n={n}")
    if Q < 1:
        raise ValueError(f"Q must be positive, got {Q}")


_initialized = False


def init(wisdom_path=None):
    """Initialise the library (selects GPU 0 unless ``icm_gpu_init`` chose one).

    ``wisdom_path`` names an optional tuner table (text lines ``block_size 8``,
    ``fft_min_degree 64``, ``q_chunk 64``), the analogue of the reference's
    FFTW wisdom file.
    """
    global _initialized
    L = lib()
    L.icm_init(wisdom_path.encode() if isinstance(wisdom_path, str) else wisdom_path)
    _initialized = True


def _auto_init():
    if not _initialized:
        init()


def _raise_if_failed(what):
    if lib().icm_last_status() != 0:
        raise ICMError(f"{what} failed: {lib().icm_gpu_last_error().decode(errors='replace')}")


def equity(stacks, payouts, Q=256):
    """ICM equities for all players (reference ``icm.equity``)."""
    stacks_arr = _to_double_array(stacks, "stacks")
    payouts_arr = _to_double_array(payouts, "payouts")
    n, k = len(stacks_arr), len(payouts_arr)
    _check(n, k, Q)
    _auto_init()
    out = np.zeros(n, dtype=np.float64)
    lib().icm_equity(n, _d(stacks_arr), int(Q), _d(payouts_arr), k, _d(out))
    _raise_if_failed("icm_equity")
    return out


def equity_subset(stacks, payouts, targets, Q=256):
    """Equities for the target players only; other entries are 0
    (reference ``icm.equity_subset``)."""
    stacks_arr = _to_double_array(stacks, "stacks")
    payouts_arr = _to_double_array(payouts, "payouts")
    targets_arr = _to_int_array(targets, "targets")
    n, k, nt = len(stacks_arr), len(payouts_arr), len(targets_arr)
    _check(n, k, Q)
    if nt < 1:
        raise ValueError("targets must not be empty")
    if np.any(targets_arr < 0) or np.any(targets_arr >= n):
        raise ValueError(f"target indices must be in [0, {n-1}]")
    _auto_init()
    out = np.zeros(n, dtype=np.float64)
    lib().icm_equity_subset(n, _d(stacks_arr), int(Q), _d(payouts_arr), k, _d(out),
                            targets_arr.ctypes.data_as(_ip), nt)
    _raise_if_failed("icm_equity_subset")
    return out


def _stats_dict(st):
    return {name: getattr(st, name) for name, _ in IcmGpuRunStats._fields_}


def gpu_equity(stacks, payouts, Q=256, return_stats=False):
    """``icm_gpu_equity``: like ``equity`` but returns run statistics too."""
    S = _to_double_array(stacks, "stacks")
    P = _to_double_array(payouts, "payouts")
    _check(len(S), len(P), Q)
    _auto_init()
    out = np.zeros(len(S))
    st = IcmGpuRunStats()
    if lib().icm_gpu_equity(len(S), _d(S), int(Q), _d(P), len(P), _d(out), None, ctypes.byref(st)) != 0:
        raise ICMError(lib().icm_gpu_last_error().decode(errors="replace"))
    return (out, _stats_dict(st)) if return_stats else out


def gpu_equity_subset(stacks, payouts, targets, Q=256):
    S = _to_double_array(stacks, "stacks")
    P = _to_double_array(payouts, "payouts")
    T = _to_int_array(targets, "targets")
    _check(len(S), len(P), Q)
    if np.any(T < 0) or np.any(T >= len(S)):
        raise ValueError(f"target indices must be in [0, {len(S)-1}]")
    _auto_init()
    out = np.zeros(len(S))
    if lib().icm_gpu_equity_subset(len(S), _d(S), int(Q), _d(P), len(P), _d(out), T.ctypes.data_as(_ip),
                                   len(T), None, None) != 0:
        raise ICMError(lib().icm_gpu_last_error().decode(errors="replace"))
    return out


class GpuPlan:
    """Reusable plan for one tournament (``IcmGpuPlan``): sorted stacks, tree
    geometry and device buffers are set up once; ``equity`` runs the
    quadrature for any payout vector of length k."""

    def __init__(self, stacks, k, options: IcmGpuOptions | None = None):
        _auto_init()
        self.S = _to_double_array(stacks, "stacks")
        self.n, self.k = len(self.S), int(k)
        _check(self.n, self.k, 1)
        self._p = lib().icm_gpu_plan_create(self.n, _d(self.S), self.k,
                                            ctypes.byref(options) if options else None)
        if not self._p:
            raise ICMError(lib().icm_gpu_last_error().decode(errors="replace"))

    def equity(self, payouts, Q=256, return_stats=False, nodes=None):
        """Equities for ``payouts`` (length k).  ``nodes=(q_begin, q_end)``
        sums only the rule's nodes q_begin <= q < q_end of Q (a part of the
        quadrature; the parts of a partition of [0, Q) add up to the full
        equities, to rounding)."""
        P = _to_double_array(payouts, "payouts")
        if len(P) != self.k:
            raise ValueError(f"payouts length {len(P)} != plan k={self.k}")
        out = np.zeros(self.n)
        st = IcmGpuRunStats()
        if nodes is None:
            rc = lib().icm_gpu_equity_with_plan(self._p, int(Q), _d(P), _d(out), ctypes.byref(st))
        else:
            qb, qe = (int(x) for x in nodes)
            rc = lib().icm_gb300_plan_equity_nodes(self._p, int(Q), _d(P), qb, qe, _d(out), ctypes.byref(st))
        if rc != 0:
            raise ICMError(lib().icm_gpu_last_error().decode(errors="replace"))
        return (out, _stats_dict(st)) if return_stats else out

    def equity_device(self, payout_ptr, equity_ptr, stream=0, Q=256):
        """Stream-ordered run on device memory (icm_gb300_plan_equity_dev):
        ``payout_ptr`` (k doubles) and ``equity_ptr`` (n doubles) are device
        addresses (e.g. a CUDA tensor's ``data_ptr()``), ``stream`` the
        caller's cudaStream_t as an integer (0 = the legacy default stream).
        Returns once the work is queued; the stream's later work sees the
        equities."""
        if lib().icm_gb300_plan_equity_dev(self._p, int(Q), ctypes.c_void_p(int(payout_ptr)),
                                           ctypes.c_void_p(int(equity_ptr)), ctypes.c_void_p(int(stream))) != 0:
            raise ICMError(lib().icm_gpu_last_error().decode(errors="replace"))

    def set_targets(self, targets=None):
        """Later equity() calls compute only these players' equities (others
        0), pruning the propagate as equity_subset does; None or an empty
        list returns the plan to full-field runs."""
        if targets is None or len(targets) == 0:
            rc = lib().icm_gb300_plan_set_targets(self._p, None, 0)
        else:
            t = _to_int_array(targets, "targets")
            rc = lib().icm_gb300_plan_set_targets(self._p, t.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), len(t))
        if rc != 0:
            raise ICMError(lib().icm_gpu_last_error().decode(errors="replace"))

    def summary(self):
        s = IcmGpuPlanSummary()
        lib().icm_gpu_plan_summary(self._p, ctypes.byref(s))
        return {name: getattr(s, name) for name, _ in IcmGpuPlanSummary._fields_}

    def close(self):
        if getattr(self, "_p", None):
            lib().icm_gpu_plan_destroy(self._p)
            self._p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _batch_arrays(tournaments, Q):
    Ss = [_to_double_array(s, "stacks") for s, _ in tournaments]
    Ps = [_to_double_array(p, "payouts") for _, p in tournaments]
    if not Ss:
        raise ValueError("tournaments must not be empty")
    ns = np.array([len(s) for s in Ss], dtype=np.int32)
    ks = np.array([len(p) for p in Ps], dtype=np.int32)
    for n, k in zip(ns, ks):
        _check(int(n), int(k), Q)
    return ns, ks, np.ascontiguousarray(np.concatenate(Ss)), np.ascontiguousarray(np.concatenate(Ps))


def equity_batched(tournaments, Q=256, return_stats=False):
    """Equities of many independent tournaments: ``tournaments`` is a list of
    (stacks, payouts).  Every tree-level step of all tournaments runs as one
    work-list launch; results equal single-tournament solves bit for bit.
    Returns a list of arrays."""
    ns, ks, S, P = _batch_arrays(tournaments, Q)
    _auto_init()
    out = np.zeros(len(S))
    st = IcmGpuRunStats()
    if lib().icm_gpu_equity_batched(len(ns), ns.ctypes.data_as(_ip), ks.ctypes.data_as(_ip), _d(S), _d(P),
                                    int(Q), _d(out), ctypes.byref(st)) != 0:
        raise ICMError(lib().icm_gpu_last_error().decode(errors="replace"))
    res = np.split(out, np.cumsum(ns)[:-1])
    return (res, _stats_dict(st)) if return_stats else res


class GpuBatch:
    """Reusable batch of tournaments: sorts, geometry, device buffers and the
    work lists are built once from the stacks; ``equity(payouts)`` uploads the
    payouts and replays the captured CUDA graph of the launch sequence."""

    _create = "icm_gb300_batch_create"

    def __init__(self, stacks_list, ks):
        Ss = [_to_double_array(s, "stacks") for s in stacks_list]
        self.ns = np.array([len(s) for s in Ss], dtype=np.int32)
        self.ks = np.array([int(k) for k in ks], dtype=np.int32)
        if len(self.ks) != len(self.ns):
            raise ValueError("one k per tournament")
        for n, k in zip(self.ns, self.ks):
            _check(int(n), int(k), 1)
        _auto_init()
        S = np.ascontiguousarray(np.concatenate(Ss))
        self._h = getattr(lib(), self._create)(len(Ss), self.ns.ctypes.data_as(_ip), self.ks.ctypes.data_as(_ip),
                                               _d(S))
        if not self._h:
            raise ICMError(lib().icm_gpu_last_error().decode(errors="replace"))
        self._splits = np.cumsum(self.ns)[:-1]

    def _concat(self, xs, what, size):
        if isinstance(xs, (list, tuple)):
            X = np.ascontiguousarray(np.concatenate([_to_double_array(x, what) for x in xs]))
        else:
            X = _to_double_array(xs, what)
        if X.size != size:
            raise ValueError(f"{what}: expected {size} values, got {X.size}")
        return X

    def equity(self, payouts, Q=256, return_stats=False, split=True):
        """``payouts``: list of arrays (one per tournament) or their
        concatenation.  Returns the list of equity arrays (or the
        concatenation with ``split=False``)."""
        P = self._concat(payouts, "payouts", int(self.ks.sum()))
        if Q < 1:
            raise ValueError(f"Q must be >= 1, got Q={Q}")
        out = np.zeros(int(self.ns.sum()))
        st = IcmGpuRunStats()
        if lib().icm_gb300_batch_run(self._h, int(Q), _d(P), _d(out), ctypes.byref(st)) != 0:
            raise ICMError(lib().icm_gpu_last_error().decode(errors="replace"))
        res = np.split(out, self._splits) if split else out
        return (res, _stats_dict(st)) if return_stats else res

    def set_options(self, graphs=True, profiling=None):
        prof = -1 if profiling is None else int(bool(profiling))
        lib().icm_gb300_batch_set_options(self._h, int(bool(graphs)), prof)

    def info(self):
        m, fb, pl = ctypes.c_long(), ctypes.c_long(), ctypes.c_long()
        qc, ms, nb = ctypes.c_int(), ctypes.c_double(), ctypes.c_size_t()
        lib().icm_gb300_batch_info(self._h, ctypes.byref(m), ctypes.byref(fb), ctypes.byref(pl), ctypes.byref(qc),
                                   ctypes.byref(ms), ctypes.byref(nb))
        return {"members": m.value, "fallbacks": fb.value, "players": pl.value, "q_chunk": qc.value,
                "device_ms": ms.value, "device_bytes": nb.value}

    def kernel_stats(self):
        L = lib()
        cnt = L.icm_gb300_batch_kernel_stats(self._h, -1, None, 0, None, None, None)
        out = []
        for i in range(max(cnt, 0)):
            name = ctypes.create_string_buffer(64)
            ms, fl, ln = ctypes.c_double(), ctypes.c_double(), ctypes.c_long()
            L.icm_gb300_batch_kernel_stats(self._h, i, name, 64, ctypes.byref(ms), ctypes.byref(ln), ctypes.byref(fl))
            out.append({"name": name.value.decode(), "ms": ms.value, "launches": ln.value, "flops": fl.value})
        return out

    def close(self):
        if getattr(self, "_h", None):
            lib().icm_gb300_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GpuVjpBatch(GpuBatch):
    """Reusable batched VJP: the forward and adjoint passes of every
    tournament as work-list launches, replayed as one CUDA graph.
    ``vjp(payouts, cotangents)`` returns (grad_stacks, grad_payouts) lists
    (or the concatenations with ``split=False``)."""

    _create = "icm_gb300_vjp_batch_create"

    def equity(self, *a, **kw):
        raise ICMError("a VJP batch computes gradients: use vjp()")

    def vjp(self, payouts, cotangents, Q=256, node_terms=False, return_stats=False, split=True):
        P = self._concat(payouts, "payouts", int(self.ks.sum()))
        C = self._concat(cotangents, "cotangent", int(self.ns.sum()))
        if Q < 1:
            raise ValueError(f"Q must be >= 1, got Q={Q}")
        gS, gP = np.zeros(C.size), np.zeros(P.size)
        st = IcmGpuRunStats()
        if lib().icm_gb300_vjp_batch_run(self._h, int(Q), _d(P), _d(C), _d(gS), _d(gP), int(bool(node_terms)),
                                         ctypes.byref(st)) != 0:
            raise ICMError(lib().icm_gpu_last_error().decode(errors="replace"))
        res = (list(zip(np.split(gS, self._splits), np.split(gP, np.cumsum(self.ks)[:-1]))) if split else (gS, gP))
        return (res, _stats_dict(st)) if return_stats else res


def equity_vjp(stacks, payouts, cotangent, Q=256, node_terms=False):
    """dL/dS and dL/dpayout of L = sum_i cot_i equity_i(S, payout), through
    the GPU adjoint passes.  Returns (grad_stacks, grad_payouts).
    ``node_terms`` also differentiates the quadrature nodes' dependence on
    max S (the exact derivative of the Q-node formula)."""
    S = _to_double_array(stacks, "stacks")
    P = _to_double_array(payouts, "payouts")
    C = _to_double_array(cotangent, "cotangent")
    n, k = len(S), len(P)
    _check(n, k, Q)
    if len(C) != n:
        raise ValueError(f"cotangent: expected {n} values, got {len(C)}")
    _auto_init()
    gS, gP = np.zeros(n), np.zeros(k)
    if lib().icm_gb300_equity_vjp(n, _d(S), int(Q), _d(P), k, _d(C), _d(gS), _d(gP), int(bool(node_terms))) != 0:
        raise ICMError(lib().icm_gpu_last_error().decode(errors="replace"))
    return gS, gP


def equity_vjp_batched(tournaments, cotangents, Q=256, node_terms=False):
    """VJPs of many tournaments: lists of (stacks, payouts) and cotangents.
    Returns a list of (grad_stacks, grad_payouts)."""
    ns, ks, S, P = _batch_arrays(tournaments, Q)
    C = np.ascontiguousarray(np.concatenate([_to_double_array(c, "cotangent") for c in cotangents]))
    if C.size != S.size:
        raise ValueError("one cotangent value per player")
    _auto_init()
    gS, gP = np.zeros(S.size), np.zeros(P.size)
    if lib().icm_gb300_equity_vjp_batched(len(ns), ns.ctypes.data_as(_ip), ks.ctypes.data_as(_ip), _d(S), _d(P),
                                          int(Q), _d(C), _d(gS), _d(gP), int(bool(node_terms))) != 0:
        raise ICMError(lib().icm_gpu_last_error().decode(errors="replace"))
    return list(zip(np.split(gS, np.cumsum(ns)[:-1]), np.split(gP, np.cumsum(ks)[:-1])))


class VjpPlan:
    """Reusable VJP plan for one set of stacks (sort, geometry and buffers
    once); ``run(payouts, cotangent)`` returns (grad_stacks, grad_payouts)."""

    def __init__(self, stacks, k):
        S = _to_double_array(stacks, "stacks")
        self.n, self.k = len(S), int(k)
        _check(self.n, self.k, 1)
        _auto_init()
        self._h = lib().icm_gb300_vjp_create(self.n, _d(S), self.k)
        if not self._h:
            raise ICMError(lib().icm_gpu_last_error().decode(errors="replace"))

    def run(self, payouts, cotangent, Q=256, return_stats=False, node_terms=False):
        P = _to_double_array(payouts, "payouts")
        C = _to_double_array(cotangent, "cotangent")
        if len(P) != self.k or len(C) != self.n:
            raise ValueError("payouts must have k values and cotangent n values")
        gS, gP = np.zeros(self.n), np.zeros(self.k)
        st = IcmGpuRunStats()
        if lib().icm_gb300_vjp_run(self._h, int(Q), _d(P), _d(C), _d(gS), _d(gP), int(bool(node_terms)),
                                   ctypes.byref(st)) != 0:
            raise ICMError(lib().icm_gpu_last_error().decode(errors="replace"))
        return ((gS, gP), _stats_dict(st)) if return_stats else (gS, gP)

    def run_device(self, payout_ptr, cot_ptr, grad_s_ptr, grad_p_ptr, stream=0, Q=256, node_terms=False):
        """Stream-ordered VJP on device memory (icm_gb300_vjp_run_dev); the
        pointers are device addresses (k, n, n and k doubles), ``stream`` the
        caller's cudaStream_t as an integer."""
        vp = ctypes.c_void_p
        if lib().icm_gb300_vjp_run_dev(self._h, int(Q), vp(int(payout_ptr)), vp(int(cot_ptr)), vp(int(grad_s_ptr)),
                                       vp(int(grad_p_ptr)), int(bool(node_terms)), vp(int(stream))) != 0:
            raise ICMError(lib().icm_gpu_last_error().decode(errors="replace"))

    def device_ms(self):
        return lib().icm_gb300_vjp_device_ms(self._h)

    def close(self):
        if getattr(self, "_h", None):
            lib().icm_gb300_vjp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def autotune(stacks, payouts, Q=256, runs=2):
    """Time every (block size, FFT crossover) candidate on these stacks and
    payouts, record the fastest in the tuner table for their size class, then
    time each spectral level's alternatives (points per CTA, coefficients)
    and record those faster by more than 1% (tuner_lookup_level); return
    (block_size, fft_min_degree, best_ms)."""
    S = _to_double_array(stacks, "stacks")
    P = _to_double_array(payouts, "payouts")
    _check(len(S), len(P), Q)
    _auto_init()
    b, f, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
    if lib().icm_gb300_autotune(len(S), _d(S), int(Q), _d(P), len(P), int(runs), ctypes.byref(b), ctypes.byref(f),
                                ctypes.byref(ms)) != 0:
        raise ICMError(lib().icm_gpu_last_error().decode(errors="replace"))
    return b.value, f.value, ms.value


def tuner_load(path):
    """Load a tuner table file; returns the number of size-class entries read."""
    r = lib().icm_gb300_tuner_load(os.fsencode(path))
    if r < 0:
        raise ICMError(lib().icm_gpu_last_error().decode(errors="replace"))
    return r


def tuner_save(path):
    """Write the tuner table; returns the number of size-class entries."""
    r = lib().icm_gb300_tuner_save(os.fsencode(path))
    if r < 0:
        raise ICMError(lib().icm_gpu_last_error().decode(errors="replace"))
    return r


def tuner_clear():
    lib().icm_gb300_tuner_clear()


def tuner_lookup(n, k):
    """(block_size, fft_min_degree) the table holds for (n, k)'s class, or None."""
    b, f = ctypes.c_int(), ctypes.c_int()
    if lib().icm_gb300_tuner_lookup(int(n), int(k), ctypes.byref(b), ctypes.byref(f)) == 1:
        return b.value, f.value
    return None


def tuner_lookup_level(n, k, level):
    """(spectral, cta_points) the table holds for tree level `level` of
    (n, k)'s class, or None."""
    sp, pts = ctypes.c_int(), ctypes.c_int()
    if lib().icm_gb300_tuner_lookup_level(int(n), int(k), int(level), ctypes.byref(sp), ctypes.byref(pts)) == 1:
        return sp.value, pts.value
    return None


def equity_adaptive(stacks, payouts, tol=1e-9, Q0=256, Qmax=4096):
    """Equities with Q doubled from Q0 until two successive node counts agree
    to `tol` per player.  Returns (equity, Q_used, estimated_error)."""
    S = _to_double_array(stacks, "stacks")
    P = _to_double_array(payouts, "payouts")
    _check(len(S), len(P), Q0)
    _auto_init()
    out = np.zeros(len(S))
    qu, est = ctypes.c_int(), ctypes.c_double()
    if lib().icm_gb300_equity_adaptive(len(S), _d(S), _d(P), len(P), int(Q0), float(tol), int(Qmax), _d(out),
                                       ctypes.byref(qu), ctypes.byref(est)) != 0:
        raise ICMError(lib().icm_gpu_last_error().decode(errors="replace"))
    return out, qu.value, est.value


def configure(block_size=0, fft_min_degree=0, q_chunk=0, max_device_bytes=0, coefficient_fft_only=False,
              zero_prefix=True, subtree=False, small_max_n=0, engine="auto", quadrature="erfc", chunk_streams=0,
              cta_points=0, tma=True, vjp_spectral_min_degree=0):
    """Process-wide engine settings for plans created afterwards (0 = default).

    coefficient_fft_only=True keeps every FFT tree level on coefficients
    (no spectral levels), for comparison and testing; zero_prefix=False
    computes tree nodes whose players all have a leaf factor of exactly 0 at
    a quadrature node instead of writing them as monomials / skipping them;
    subtree=True runs the leaf blocks and bottom schoolbook levels in one
    kernel per direction (same results; measured slightly slower);
    small_max_n sets the largest n of the one-CTA-per-node small path
    (0 = default k-dependent limit, -1 = never); engine is "auto", "tree"
    or "linear" (the O(n k) linear engine, one warp per node, k <= 256);
    quadrature is "erfc" (the reference's erfc-trapezoid rule) or "tanh_sinh";
    chunk_streams spreads a tree plan's node chunks over that many streams
    (0 = default: 4 from n = 6000, else 2; 1 = one stream; at most 4; same
    results); cta_points sets the complex points per CTA of the spectral
    levels' one-CTA FFT steps (1024, 2048, 4096 or 8192; 0 = the tuner
    table's per-level choice, else 4096; same results); tma=False makes the
    four-step column pass of the largest levels gather its tile with ordinary
    loads instead of a TMA tensor copy (same results);
    vjp_spectral_min_degree: levels of a VJP (single or batched) whose
    children have at least this degree run spectrally in the forward and
    adjoint passes
    (0 = every level a forward plan would make spectral, -1 = all on
    coefficients; results agree to rounding)."""
    engines = {"auto": 0, "tree": 1, "linear": 2}
    rules = {"erfc": 0, "tanh_sinh": 1}
    if engine not in engines:
        raise ValueError(f"engine must be one of {sorted(engines)}, got {engine!r}")
    if quadrature not in rules:
        raise ValueError(f"quadrature must be one of {sorted(rules)}, got {quadrature!r}")
    cfg = IcmGb300Config(block_size, fft_min_degree, q_chunk, 1 if coefficient_fft_only else 0, max_device_bytes,
                         0 if zero_prefix else 1, 1 if subtree else 0, int(small_max_n), engines[engine],
                         rules[quadrature], int(chunk_streams), int(cta_points), 0 if tma else 1,
                         int(vjp_spectral_min_degree))
    lib().icm_gb300_set_config(ctypes.byref(cfg))


def measure_fp64_gflops():
    _auto_init()
    v = ctypes.c_double()
    if lib().icm_gpu_measure_fp64_gflops(ctypes.byref(v)) != 1:
        raise ICMError(lib().icm_gpu_last_error().decode(errors="replace"))
    return v.value


def measure_hbm_gbps():
    _auto_init()
    v = ctypes.c_double()
    if lib().icm_gpu_measure_hbm_bandwidth_gbps(ctypes.byref(v)) != 1:
        raise ICMError(lib().icm_gpu_last_error().decode(errors="replace"))
    return v.value


def last_launch_count():
    return int(lib().icm_gpu_last_launch_count())


def player_order(stacks):
    """The engine's player order (host only): indices by stack, descending,
    ties by index."""
    S = _to_double_array(stacks, "stacks")
    perm = np.zeros(len(S), dtype=np.int32)
    if len(S) == 0 or lib().icm_gb300_player_order(len(S), _d(S), perm.ctypes.data_as(_ip)) != 0:
        raise ICMError(lib().icm_gpu_last_error().decode(errors="replace") if len(S) else "empty stacks")
    return perm
