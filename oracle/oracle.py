"""ctypes front end for the CPU oracle (test infrastructure only).

Two checkers live here:

* ``Oracle`` wraps ``liboracle.so``: this project's C restatement of the
  reference's quadrature engine (``icm_oracle.c``; each function cites the
  reference lines it follows) plus the closed-form V1 / V2 equities.
* ``ReferenceLib`` wraps ``_ref/libicm_ref*.so``: the reference's own
  ``src/cpu/icm.c``, compiled unmodified against the FFTW-API shim.  It only
  exists where the reference sources were present at build time.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import
this module.  The product package never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def build(ref: str | None = None, quiet: bool = True) -> None:
    """Compile liboracle.so (and oracle/_ref when the reference tree exists)."""
    out = subprocess.DEVNULL if quiet else None
    subprocess.run(["make", "-C", HERE, "liboracle.so"], check=True, stdout=out)
    ref = ref or os.environ.get("ICM_REFERENCE_DIR", "/root/reference")
    if os.path.isfile(os.path.join(ref, "src", "cpu", "icm.c")):
        subprocess.run(["make", "-C", HERE, "ref", f"REF={ref}"], check=True, stdout=out)


class Oracle:
    """The C restatement (icm_oracle.c)."""

    def __init__(self, path: str | None = None):
        path = path or os.path.join(HERE, "liboracle.so")
        if not os.path.isfile(path):
            build()
        lib = ctypes.CDLL(path)
        lib.oracle_equity.argtypes = [ctypes.c_int, _dp, ctypes.c_int, _dp, ctypes.c_int,
                                      ctypes.c_int, ctypes.c_int, _ip, ctypes.c_int,
                                      ctypes.c_int, _dp]
        lib.oracle_equity.restype = ctypes.c_int
        lib.oracle_equity_naive.argtypes = [ctypes.c_int, _dp, ctypes.c_int, _dp, ctypes.c_int, _dp]
        lib.oracle_equity_naive.restype = ctypes.c_int
        lib.oracle_make_nodes.argtypes = [ctypes.c_int, ctypes.c_double, _dp, _dp]
        lib.oracle_make_nodes.restype = None
        lib.oracle_sort_desc.argtypes = [ctypes.c_int, _dp, _ip]
        lib.oracle_sort_desc.restype = None
        for fn in (lib.oracle_v1, lib.oracle_v2):
            fn.argtypes = [ctypes.c_int, _dp, ctypes.c_int, _ip, _dp, ctypes.c_int]
            fn.restype = None
        self.lib = lib

    def equity(self, S, payout, Q=256, B=16, fft_min_deg=0, targets=None, threads=None):
        S = np.ascontiguousarray(S, dtype=np.float64)
        P = np.ascontiguousarray(payout, dtype=np.float64)
        n, k = len(S), len(P)
        out = np.zeros(n)
        threads = threads or os.cpu_count() or 1
        if targets is not None:
            t = np.ascontiguousarray(targets, dtype=np.int32)
            rc = self.lib.oracle_equity(n, _d(S), Q, _d(P), k, B, fft_min_deg, _i(t), len(t),
                                        threads, _d(out))
        else:
            rc = self.lib.oracle_equity(n, _d(S), Q, _d(P), k, B, fft_min_deg, None, 0,
                                        threads, _d(out))
        if rc != 0:
            raise ValueError("oracle_equity rejected its arguments")
        return out

    def equity_naive(self, S, payout, Q=256):
        S = np.ascontiguousarray(S, dtype=np.float64)
        P = np.ascontiguousarray(payout, dtype=np.float64)
        out = np.zeros(len(S))
        if self.lib.oracle_equity_naive(len(S), _d(S), Q, _d(P), len(P), _d(out)) != 0:
            raise ValueError("oracle_equity_naive rejected its arguments")
        return out

    def nodes(self, Q, Smax):
        lv, w = np.zeros(Q), np.zeros(Q)
        self.lib.oracle_make_nodes(Q, float(Smax), _d(lv), _d(w))
        return lv, w

    def sort_desc(self, S):
        S = np.ascontiguousarray(S, dtype=np.float64)
        perm = np.zeros(len(S), dtype=np.int32)
        self.lib.oracle_sort_desc(len(S), _d(S), _i(perm))
        return perm

    def _closed(self, fn, S, idx, threads):
        S = np.ascontiguousarray(S, dtype=np.float64)
        threads = threads or os.cpu_count() or 1
        if idx is None:
            out = np.zeros(len(S))
            fn(len(S), _d(S), 0, None, _d(out), threads)
        else:
            idx = np.ascontiguousarray(idx, dtype=np.int32)
            out = np.zeros(len(idx))
            fn(len(S), _d(S), len(idx), _i(idx), _d(out), threads)
        return out

    def v1(self, S, idx=None, threads=None):
        """Closed-form equity for payout[m] = n - m."""
        return self._closed(self.lib.oracle_v1, S, idx, threads)

    def v2(self, S, idx=None, threads=None):
        """Closed-form equity for payout[m] = C(n-1-m, 2)."""
        return self._closed(self.lib.oracle_v2, S, idx, threads)


class ReferenceLib:
    """The reference's own icm.c built against the FFTW shim (oracle/_ref)."""

    def __init__(self, openmp: bool = False):
        name = "libicm_ref_omp.so" if openmp else "libicm_ref.so"
        path = os.path.join(HERE, "_ref", name)
        if not os.path.isfile(path):
            raise FileNotFoundError(path)
        lib = ctypes.CDLL(path, mode=ctypes.RTLD_LOCAL)
        lib.icm_init.argtypes = [ctypes.c_char_p]
        lib.icm_equity.argtypes = [ctypes.c_int, _dp, ctypes.c_int, _dp, ctypes.c_int, _dp]
        lib.icm_equity.restype = None
        lib.icm_equity_subset.argtypes = [ctypes.c_int, _dp, ctypes.c_int, _dp, ctypes.c_int,
                                          _dp, _ip, ctypes.c_int]
        lib.icm_equity_subset.restype = None
        lib.icm_v1_exact.argtypes = [ctypes.c_int, _dp, _dp]
        lib.icm_v2_exact.argtypes = [ctypes.c_int, _dp, _dp]
        lib.icm_init(os.path.join(HERE, "_ref", "no_wisdom.dat").encode())
        self.lib = lib

    @staticmethod
    def available(openmp: bool = False) -> bool:
        name = "libicm_ref_omp.so" if openmp else "libicm_ref.so"
        return os.path.isfile(os.path.join(HERE, "_ref", name))

    def equity(self, S, payout, Q=256, targets=None):
        S = np.ascontiguousarray(S, dtype=np.float64)
        P = np.ascontiguousarray(payout, dtype=np.float64)
        out = np.zeros(len(S))
        if targets is None:
            self.lib.icm_equity(len(S), _d(S), Q, _d(P), len(P), _d(out))
        else:
            t = np.ascontiguousarray(targets, dtype=np.int32)
            self.lib.icm_equity_subset(len(S), _d(S), Q, _d(P), len(P), _d(out), _i(t), len(t))
        return out
