"""ctypes front end for the CPU oracle (test infrastructure only).

Two checkers live here:

* ``Oracle`` wraps ``liboracle.so``: this project's C restatement of the
  reference's quadrature engine (``icm_oracle.c``; each function cites the
  reference lines it follows) plus the closed-form V1 / V2 equities.
* ``ReferenceLib`` wraps ``_ref/libicm_ref*.so``: the reference's own
  ``src/cpu/icm.c``, compiled unmodified against the FFTW-API shim (serial
  and OpenMP builds).
* ``ReferenceGpu`` wraps ``_ref/libicm_ref_gpu.so``: the reference's own GPU
  library (``src/gpu/*.cu``, cuFFT tier), a timing comparison on the same GPU.

The reference libraries exist where the reference sources were present at
build time: the reference tree itself, or the git-ignored staged copy of its
few files under ``_ref/tree`` (oracle/Makefile, target ``stage``).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg and
reference arm import this module.  The product package never does.
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


STAGE = os.path.join(HERE, "_ref", "tree")


def _make(targets, quiet):
    """Run oracle/Makefile; ICM_REFERENCE_DIR, when set, names the reference
    tree to stage from (the Makefile's own default otherwise)."""
    cmd = ["make", "-C", HERE, *targets]
    if os.environ.get("ICM_REFERENCE_DIR"):
        cmd.append(f"REF={os.environ['ICM_REFERENCE_DIR']}")
    subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL if quiet else None)


def build(quiet: bool = True, gpu: bool = False) -> None:
    """Compile liboracle.so and, where the reference's sources are present
    (its tree, or the staged copy under _ref/tree), the reference's own CPU
    library (_ref/libicm_ref*.so); with gpu=True also its GPU library
    (_ref/libicm_ref_gpu.so)."""
    _make(["liboracle.so", "ref"] + (["-j8", "ref-gpu"] if gpu else []), quiet)


def staged(relpath: str) -> str | None:
    """Path of a staged reference file (by its path in the reference tree),
    or None where nothing was staged."""
    p = os.path.join(STAGE, relpath)
    return p if os.path.isfile(p) else None


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
    """The reference's own icm.c built against the FFTW shim (oracle/_ref):
    libicm_ref.so is the serial build (the reference Makefile's `make`),
    libicm_ref_omp.so the OpenMP build (`make parallel`; its thread count
    follows OMP_NUM_THREADS, read when the library starts its first parallel
    region)."""

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


class _GpuOptions(ctypes.Structure):
    """IcmGpuOptions, layout of the reference's src/gpu/icm_gpu.h:12-34."""
    _fields_ = [(f, ctypes.c_int) for f in (
        "device_id", "use_cufftdx", "enable_graphs", "enable_q_pipeline", "memory_strategy",
        "force_uncached_fused_levels", "force_uncached_cufft_levels", "fast_mode", "verbose")]


class _GpuRunStats(ctypes.Structure):
    """IcmGpuRunStats, layout of the reference's src/gpu/icm_gpu.h:36-50."""
    _fields_ = [(f, ctypes.c_double) for f in (
        "total_ns", "sort_ns", "quadrature_overhead_ns", "block_build_ns", "tree_build_ns",
        "tree_propagate_cached_ns", "tree_propagate_recomputed_ns", "leaf_extract_ns")] + [
        ("peak_vram_bytes", ctypes.c_size_t)] + [(f, ctypes.c_int) for f in (
            "engine", "B", "uncached_fused_levels", "uncached_cufft_levels")]


class ReferenceGpu:
    """The reference's own GPU library (oracle/_ref/libicm_ref_gpu.so: its
    src/gpu/*.cu with the cuFFT tier, B200 calibration data), a comparison
    arm for timing on the same GPU.  Entry points as src/gpu/icm_gpu.h:66-104:
    icm_gpu_init returns 1 on success, the others 0 / -1."""

    PATH = os.path.join(HERE, "_ref", "libicm_ref_gpu.so")

    def __init__(self, device: int = 0):
        if not os.path.isfile(self.PATH):
            raise FileNotFoundError(self.PATH)
        lib = ctypes.CDLL(self.PATH, mode=ctypes.RTLD_LOCAL)
        vp = ctypes.c_void_p
        lib.icm_gpu_init.argtypes = [ctypes.c_int]
        lib.icm_gpu_last_error.restype = ctypes.c_char_p
        lib.icm_gpu_plan_create.argtypes = [ctypes.c_int, _dp, ctypes.c_int, ctypes.POINTER(_GpuOptions)]
        lib.icm_gpu_plan_create.restype = vp
        lib.icm_gpu_plan_destroy.argtypes = [vp]
        lib.icm_gpu_equity_with_plan.argtypes = [vp, ctypes.c_int, _dp, _dp, ctypes.POINTER(_GpuRunStats)]
        lib.icm_gpu_equity.argtypes = [ctypes.c_int, _dp, ctypes.c_int, _dp, ctypes.c_int, _dp,
                                       ctypes.POINTER(_GpuOptions), ctypes.POINTER(_GpuRunStats)]
        lib.icm_gpu_shutdown.restype = None
        if lib.icm_gpu_init(device) != 1:
            raise RuntimeError("reference icm_gpu_init failed: " + (lib.icm_gpu_last_error() or b"").decode())
        self.lib = lib

    @staticmethod
    def available() -> bool:
        return os.path.isfile(ReferenceGpu.PATH)

    def error(self) -> str:
        return (self.lib.icm_gpu_last_error() or b"").decode()

    @staticmethod
    def options():
        """The options the reference's own benchmarks pass
        (tools/heatmap_gpu.cu:79-85, bench/bench_gpu.cu:214-220)."""
        o = _GpuOptions()
        o.use_cufftdx, o.enable_graphs, o.enable_q_pipeline, o.memory_strategy = 1, 0, 1, 0
        o.force_uncached_fused_levels = o.force_uncached_cufft_levels = -1
        return o

    def equity(self, S, payout, Q=256):
        """One-shot icm_gpu_equity (plan set-up inside); returns (equity,
        total_ns as the library reports it)."""
        S = np.ascontiguousarray(S, dtype=np.float64)
        P = np.ascontiguousarray(payout, dtype=np.float64)
        out = np.zeros(len(S))
        st = _GpuRunStats()
        opts = self.options()
        if self.lib.icm_gpu_equity(len(S), _d(S), Q, _d(P), len(P), _d(out), ctypes.byref(opts),
                                   ctypes.byref(st)) != 0:
            raise RuntimeError("reference icm_gpu_equity failed: " + self.error())
        return out, st.total_ns

    def plan(self, S, k):
        S = np.ascontiguousarray(S, dtype=np.float64)
        opts = self.options()
        p = self.lib.icm_gpu_plan_create(len(S), _d(S), int(k), ctypes.byref(opts))
        if not p:
            raise RuntimeError("reference icm_gpu_plan_create failed: " + self.error())
        return p

    def equity_with_plan(self, plan, n, payout, Q=256):
        P = np.ascontiguousarray(payout, dtype=np.float64)
        out = np.zeros(n)
        st = _GpuRunStats()
        if self.lib.icm_gpu_equity_with_plan(plan, Q, _d(P), _d(out), ctypes.byref(st)) != 0:
            raise RuntimeError("reference icm_gpu_equity_with_plan failed: " + self.error())
        return out, st.total_ns

    def destroy(self, plan):
        self.lib.icm_gpu_plan_destroy(plan)
