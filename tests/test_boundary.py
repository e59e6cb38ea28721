"""The drop-in boundary, checked without a GPU: the C-ABI library builds for
sm_103a, loads, and exports every function include/*.h declares; the Python
binding rejects bad arguments exactly as the reference's package does
(python/tests/test_icm.py:183-208)."""
import ctypes
import os
import re

import numpy as np
import pytest

from tests.conftest import ROOT

HEADERS = [os.path.join(ROOT, "include", h) for h in ("icm.h", "icm_gpu.h", "icm_gb300.h")]


def declared_functions():
    names = set()
    for h in HEADERS:
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"typedef[^;]*;", "", text, flags=re.S)
        for m in re.finditer(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", text):
            name = m.group(1)
            if name.startswith("icm_"):
                names.add(name)
    return names


@pytest.fixture(scope="module")
def built_lib():
    from icm_gb300 import build
    path = build.build()
    return ctypes.CDLL(path)


def test_headers_declare_the_reference_api():
    names = declared_functions()
    # every entry point of the reference's src/cpu/icm.h and src/gpu/icm_gpu.h
    ref = {"icm_equity", "icm_equity_subset", "icm_init", "icm_tree_ctx_create", "icm_hybrid_ctx_create",
           "icm_linear_ctx_create", "icm_ctx_destroy", "icm_engine_tree", "icm_engine_hybrid",
           "icm_engine_linear", "icm_run_engine", "icm_run_linear_batched", "icm_select_engine",
           "icm_select_best_B", "icm_v1_exact", "icm_v2_exact", "icm_gpu_init", "icm_gpu_shutdown",
           "icm_gpu_last_error", "icm_gpu_release_pooled_memory", "icm_gpu_plan_create",
           "icm_gpu_plan_destroy", "icm_gpu_plan_summary", "icm_gpu_equity_with_plan", "icm_gpu_equity",
           "icm_gpu_equity_subset", "icm_gpu_measure_hbm_bandwidth_gbps", "icm_gpu_measure_fused_pair_ns",
           "icm_gpu_measure_fused_r2c_pair_ns"}
    assert ref <= names


def test_library_exports_every_declared_symbol(built_lib):
    missing = [n for n in sorted(declared_functions()) if not hasattr(built_lib, n)]
    assert not missing, missing


def test_python_signatures_cover_the_headers():
    from icm_gb300._lib import SIGNATURES
    engine_api = {"icm_tree_ctx_create", "icm_hybrid_ctx_create", "icm_linear_ctx_create", "icm_ctx_destroy",
                  "icm_engine_tree", "icm_engine_hybrid", "icm_engine_linear", "icm_run_engine",
                  "icm_run_linear_batched"}
    assert declared_functions() - engine_api <= set(SIGNATURES)


def test_struct_layouts_match_reference_sizes():
    from icm_gb300._lib import IcmGpuOptions, IcmGpuPlanSummary, IcmGpuRunStats
    assert ctypes.sizeof(IcmGpuOptions) == 9 * 4
    assert ctypes.sizeof(IcmGpuRunStats) == 8 * 8 + 8 + 4 * 4
    assert ctypes.sizeof(IcmGpuPlanSummary) == 9 * 4 + 4 + 8


def test_closed_forms_on_host(built_lib):
    """icm_v1_exact / icm_v2_exact run on the host and need no GPU."""
    import icm_gb300._lib as L
    lib = L.lib()
    rng = np.random.default_rng(0)
    S = 1 + 99 * rng.random(30)
    v1 = np.zeros(30)
    v2 = np.zeros(30)
    dp = ctypes.POINTER(ctypes.c_double)
    lib.icm_v1_exact(30, S.ctypes.data_as(dp), v1.ctypes.data_as(dp))
    lib.icm_v2_exact(30, S.ctypes.data_as(dp), v2.ctypes.data_as(dp))
    ref1 = np.array([1 + sum(S[i] / (S[i] + S[j]) for j in range(30) if j != i) for i in range(30)])
    assert np.allclose(v1, ref1, rtol=1e-14)
    # sum over players of V2 equals the total quadratic payout sum_m C(n-1-m, 2)
    assert abs(v2.sum() - sum((30 - 1 - m) * (30 - 2 - m) / 2 for m in range(30))) < 1e-9


class TestInputValidation:
    """Same checks and messages as the reference binding."""

    def test_empty_stacks(self):
        import icm_gb300 as icm
        with pytest.raises(ValueError, match="must not be empty"):
            icm.equity([], [0.5, 0.3, 0.2])

    def test_empty_payouts(self):
        import icm_gb300 as icm
        with pytest.raises(ValueError, match="must not be empty"):
            icm.equity([1000, 2000], [])

    def test_k_greater_than_n(self):
        import icm_gb300 as icm
        with pytest.raises(ValueError, match="k=3 must satisfy 1 <= k <= n=2"):
            icm.equity([1000, 2000], [0.5, 0.3, 0.2])

    def test_invalid_target_index(self):
        import icm_gb300 as icm
        with pytest.raises(ValueError, match="target indices"):
            icm.equity_subset([1000, 2000, 3000], [0.5, 0.3], targets=[5])

    def test_negative_target_index(self):
        import icm_gb300 as icm
        with pytest.raises(ValueError, match="target indices"):
            icm.equity_subset([1000, 2000, 3000], [0.5, 0.3], targets=[-1])

    def test_invalid_Q(self):
        import icm_gb300 as icm
        with pytest.raises(ValueError, match="Q must be positive"):
            icm.equity([1000, 2000, 3000], [0.5, 0.3, 0.2], Q=0)

    def test_two_dimensional_stacks(self):
        import icm_gb300 as icm
        with pytest.raises(ValueError, match="1-D"):
            icm.equity([[1.0, 2.0]], [1.0])


def test_missing_library_fails_loudly(tmp_path, monkeypatch):
    """No silent CPU fallback: a missing library raises ICMError."""
    import importlib
    import icm_gb300._lib as L
    monkeypatch.setenv("ICM_GB300_LIB", str(tmp_path / "absent.so"))
    monkeypatch.setattr(L, "_lib", None)
    with pytest.raises(L.ICMError):
        L.lib()
    monkeypatch.delenv("ICM_GB300_LIB")
    monkeypatch.setattr(L, "_lib", None)
    importlib.reload(L)


def _stacks(dist, n, rng):
    if dist == "mixed":                                             # many ties beside extreme magnitudes
        S = rng.integers(1, 50, n).astype(float)
        if n > 3:
            S[: n // 3] = 10.0 ** rng.uniform(-300, 300, n // 3)
            S[1] = np.nextafter(S[0], 0.0)                          # neighbours in the last bit
        return S
    if dist == "loguniform":
        return 10.0 ** rng.uniform(0, 9, n)
    if dist == "lognormal":
        return 1e4 * np.exp(1.5 * rng.standard_normal(n))
    if dist == "ints100":
        return rng.integers(1, 101, n).astype(float)
    if dist == "equal":
        return np.full(n, 2500.0)
    S = np.full(n, 100.0)                                           # one far outlier, near-equal rest
    S[::7] = np.nextafter(100.0, 200.0)
    S[n // 2] = 1e9
    return S


@pytest.mark.parametrize("dist", ["mixed", "loguniform", "lognormal", "ints100", "equal", "outlier"])
@pytest.mark.parametrize("n", [1, 2, 7, 4096, 4097, 20000, 70000, 300000])
def test_player_order_host(built_lib, n, dist):
    """The engine's player order (host only): stacks descending, ties by index,
    for the comparison sort (n <= 4096), the bucket sort on one thread and on
    several (n >= 16384), and its LSD fallback (one bucket would hold most
    players: equal stacks, a far outlier, ties beside extreme magnitudes)."""
    import icm_gb300 as icm
    S = _stacks(dist, n, np.random.default_rng(n))
    ref = np.lexsort((np.arange(n), -S))
    assert np.array_equal(icm.player_order(S), ref)
    with pytest.raises(icm.ICMError):
        icm.player_order(np.array([1.0, -2.0]))


def test_plan_geometry_invariants(built_lib):
    """Host-only sweep of the planner: for every size class, truncation, block
    size and FFT crossover (and the VJP's coefficient-only geometry), the FFT
    sizes cover every product and correlation, spectral levels sit over
    untruncated children, lengths and strides are consistent."""
    from icm_gb300._lib import lib
    L = lib()
    why = ctypes.create_string_buffer(256)
    ns = sorted({1, 2, 3, 5, 7, 8, 9, 31, 33, 100, 255, 257, 1000, 4095, 4097, 9999, 16385, 65536, 65537,
                 100003, 262144, 1 << 20, (1 << 21) + 3})
    checked = 0
    for n in ns:
        ks = sorted({k for k in (1, 2, 7, 100, n // 7, n // 2, n - 1, n, 1000, 8193, 16385) if 1 <= k <= n})
        big = n >= (1 << 18)   # fewer combinations where each geometry costs a sort of n players
        for k in ks:
            for B in ((8, 32) if big else (4, 8, 16, 32)):
                for fm in ((16, 512) if big else (8, 16, 64, 512)):
                    for flags in (0, 1, 2):
                        rc = L.icm_gb300_check_geometry(n, k, B, fm, flags, why, 256)
                        assert rc == 0, (n, k, B, fm, flags, why.value.decode())
                        checked += 1
    assert checked > 2250
    assert L.icm_gb300_check_geometry(5, 6, 8, 64, 0, why, 256) == -1


@pytest.mark.filterwarnings("ignore:This process .* is multi-threaded")
def test_player_order_concurrent_and_forked(built_lib):
    """The sort's worker pool serves one call at a time: concurrent callers
    (ctypes releases the GIL) get threads of their own, and a forked child,
    which has none of the parent's workers, sorts with fresh threads."""
    import os
    import threading
    import icm_gb300 as icm
    rng = np.random.default_rng(3)
    cases = [10.0 ** rng.uniform(0, 9, n) for n in (70000, 150000, 40000, 90000)]
    refs = [np.lexsort((np.arange(len(S)), -S)) for S in cases]
    assert np.array_equal(icm.player_order(cases[0]), refs[0])   # the pool exists
    bad = []

    def worker(j):
        for _ in range(5):
            if not np.array_equal(icm.player_order(cases[j]), refs[j]):
                bad.append(j)

    th = [threading.Thread(target=worker, args=(j,)) for j in range(len(cases))]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert not bad
    pid = os.fork()
    if pid == 0:   # child: exit status 0 only for the right order
        ok = np.array_equal(icm.player_order(cases[1]), refs[1])
        os._exit(0 if ok else 1)
    _, status = os.waitpid(pid, 0)
    assert os.WIFEXITED(status) and os.WEXITSTATUS(status) == 0


def test_player_order_many_threads(built_lib):
    """Sixteen host threads sorting fields of every size class at once (the
    worker pool serves one of them, the others spawn their own threads, small
    fields sort on the caller): every order is right."""
    import threading
    import icm_gb300 as icm
    rng = np.random.default_rng(11)
    cases = [10.0 ** rng.uniform(0, 9, n) for n in (100, 5000, 17000, 40000, 70000, 130000)]
    refs = [np.lexsort((np.arange(len(S)), -S)) for S in cases]
    bad = []

    def worker(w):
        for r in range(6):
            j = (w + r) % len(cases)
            if not np.array_equal(icm.player_order(cases[j]), refs[j]):
                bad.append((w, j))

    th = [threading.Thread(target=worker, args=(w,)) for w in range(16)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert not bad


def test_config_struct_layout_matches_header(tmp_path):
    """IcmGb300Config as the C compiler lays it out (include/icm_gb300.h)
    equals the ctypes mirror field by field."""
    import shutil
    import subprocess
    from icm_gb300._lib import IcmGb300Config
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    names = [f for f, _ in IcmGb300Config._fields_]
    src = tmp_path / "layout.c"
    src.write_text("#include <stdio.h>\n#include <stddef.h>\n#include \"icm_gb300.h\"\nint main(void) {\n"
                   "  printf(\"%zu\\n\", sizeof(IcmGb300Config));\n" +
                   "".join(f"  printf(\"%zu\\n\", offsetof(IcmGb300Config, {f}));\n" for f in names) +
                   "  return 0;\n}\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    vals = [int(x) for x in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    assert vals[0] == ctypes.sizeof(IcmGb300Config)
    assert vals[1:] == [getattr(IcmGb300Config, f).offset for f in names]
