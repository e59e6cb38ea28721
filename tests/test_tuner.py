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


def _lookup_level(L, n, k, level):
    import ctypes
    sp, pts = ctypes.c_int(), ctypes.c_int()
    r = L.icm_gb300_tuner_lookup_level(n, k, level, ctypes.byref(sp), ctypes.byref(pts))
    return (sp.value, pts.value) if r == 1 else None


def test_level_entries_roundtrip(L, tmp_path):
    p = tmp_path / "t.txt"
    p.write_text("tune 16 3 4 64 16.8\n"
                 "tune_level 16 3 7 1 2048 16.7\n"
                 "tune_level 16 3 9 0 0 16.6\n"
                 "tune_level 16 3 9 2 0 1.0\n"          # spectral must be 0 or 1
                 "tune_level 16 3 10 1 3000 1.0\n"      # points per CTA: 1024, 2048, 4096 or 8192 (0 = default)
                 "tune_level 16 3 99 1 1024 1.0\n")     # level out of range
    assert L.icm_gb300_tuner_load(str(p).encode()) == 3
    assert _lookup_level(L, 65536, 65536, 7) == (1, 2048)
    assert _lookup_level(L, 65536, 65536, 9) == (0, 0)
    assert _lookup_level(L, 65536, 65536, 8) is None
    assert _lookup_level(L, 65536, 1000, 7) is None      # another k/n bucket
    out = tmp_path / "o.txt"
    assert L.icm_gb300_tuner_save(str(out).encode()) == 3
    L.icm_gb300_tuner_clear()
    assert _lookup_level(L, 65536, 65536, 7) is None
    assert L.icm_gb300_tuner_load(str(out).encode()) == 3
    assert _lookup_level(L, 65536, 65536, 7) == (1, 2048) and _lookup_level(L, 65536, 65536, 9) == (0, 0)


def test_level_entry_keeps_a_level_on_coefficients(L, tmp_path):
    """A spectral level that the table keeps on coefficients is planned as a
    coefficient-FFT level; the geometry invariants still hold for it and for
    the levels above it (host-side check, no GPU)."""
    import ctypes
    n = k = 16384
    buf = ctypes.create_string_buffer(256)
    assert L.icm_gb300_check_geometry(n, k, 8, 64, 0, buf, 256) == 0, buf.value
    kinds = [int(x) for x in buf.value.split()[1:]]          # parent levels 1 .. L-1
    assert kinds[:3] == [0, 0, 0] and kinds[3:] == [2] * (len(kinds) - 3)
    p = tmp_path / "t.txt"
    p.write_text("tune_level 14 3 5 0 0 1.0\ntune_level 14 3 6 1 1024 1.0\n")
    assert L.icm_gb300_tuner_load(str(p).encode()) == 2
    assert L.icm_gb300_check_geometry(n, k, 8, 64, 0, buf, 256) == 0, buf.value
    tuned = [int(x) for x in buf.value.split()[1:]]
    assert tuned[4] == 1                                      # level 5 on coefficients
    assert tuned[:4] == kinds[:4] and tuned[5:] == kinds[5:]


def _kinds(L, n, k, B=8, fm=64, flags=0):
    import ctypes
    buf = ctypes.create_string_buffer(512)
    assert L.icm_gb300_check_geometry(n, k, B, fm, flags, buf, 512) == 0, buf.value
    return [int(x) for x in buf.value.split()[1:]]


def test_vjp_geometry_spectral_band(L):
    """A VJP plan's tree (flags 2): the spectral band over untruncated children
    reaches the root when the root's children are untruncated; otherwise it
    ends at children of degree 8192 at most (its top converts coefficient
    Pbar in one CTA), with coefficient-FFT levels above (host-side, no GPU)."""
    from icm_gb300 import configure
    configure()
    try:
        full = _kinds(L, 1 << 18, 1 << 18, flags=2)
        assert full[-1] == 2 and full.count(2) >= 10      # band up to the root, multi-pass levels included
        trunc = _kinds(L, 40000, 20000, flags=2)          # children of degree 16384 would be untruncated
        degs = [8 << l for l in range(len(trunc))]        # children's degree of parent level l + 1
        top = max(i for i, kd in enumerate(trunc) if kd == 2)
        assert degs[top] == 8192 and all(kd == 1 for kd in trunc[top + 1:])
        fwd = _kinds(L, 40000, 20000, flags=0)            # a forward plan goes one level further
        assert max(i for i, kd in enumerate(fwd) if kd == 2) > top
        assert 2 not in _kinds(L, 1 << 18, 1 << 18, flags=1)
        configure(vjp_spectral_min_degree=-1)             # the VJP on coefficients
        assert 2 not in _kinds(L, 1 << 18, 1 << 18, flags=2)
        configure(vjp_spectral_min_degree=1024)           # the band from children of degree 1024
        band = _kinds(L, 1 << 18, 1 << 18, flags=2)
        first = min(i for i, kd in enumerate(band) if kd == 2)
        assert (8 << first) == 1024
    finally:
        configure()
