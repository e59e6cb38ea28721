"""Tuner table file (the analogue of FFTW wisdom): parsing, size classes and
round trip, on the CPU (no GPU call)."""
import pytest

from icm_gb300._lib import lib, ICMError


@pytest.fixture()
def L():
    try:
        L = lib()
    except ICMError as e:
        pytest.skip(str(e))
    L.icm_gb300_tuner_clear()
    yield L
    L.icm_gb300_tuner_clear()


def _lookup(L, n, k):
    import ctypes
    b, f = ctypes.c_int(), ctypes.c_int()
    r = L.icm_gb300_tuner_lookup(n, k, ctypes.byref(b), ctypes.byref(f))
    return (b.value, f.value) if r == 1 else None


def test_load_lookup_save_roundtrip(L, tmp_path):
    p = tmp_path / "t.txt"
    p.write_text("# comment\ntune 16 3 8 64 20.3\ntune 11 1 4 32 0.5  # trailing comment\n"
                 "tune 11 9 4 32 1.0\ntune 12 0 5 32 1.0\nbogus line\n")
    assert L.icm_gb300_tuner_load(str(p).encode()) == 2          # bucket 9 and B = 5 rejected
    assert _lookup(L, 65536, 65536) == (8, 64)
    assert _lookup(L, 40000, 60000 // 2) == (8, 64)               # ceil log2 40000 = 16, k/n > 1/2
    assert _lookup(L, 2000, 200) == (4, 32)                        # 11, k/n in (1/64, 1/8]
    assert _lookup(L, 2000, 2000) is None
    out = tmp_path / "o.txt"
    assert L.icm_gb300_tuner_save(str(out).encode()) == 2
    L.icm_gb300_tuner_clear()
    assert _lookup(L, 65536, 65536) is None
    assert L.icm_gb300_tuner_load(str(out).encode()) == 2
    assert _lookup(L, 65536, 65536) == (8, 64) and _lookup(L, 2000, 200) == (4, 32)


def test_missing_file(L, tmp_path):
    assert L.icm_gb300_tuner_load(str(tmp_path / "none.txt").encode()) == -1
    assert b"cannot open" in L.icm_gpu_last_error()


def test_later_entry_replaces_earlier(L, tmp_path):
    p = tmp_path / "t.txt"
    p.write_text("tune 10 2 4 16 1\ntune 10 2 16 128 2\n")
    assert L.icm_gb300_tuner_load(str(p).encode()) == 2
    assert _lookup(L, 1000, 300) == (16, 128)
