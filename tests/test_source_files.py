"""The reference's raw source files (sources_%03d.dat per k1): layout written by
song2_store_sources, read back by song2_load_sources and by a reader that follows
the reference's loop order (type, then k2 <= k1, each a tau*k3 slab)."""
import numpy as np

from song_gb300 import capi
from helpers import problem


def test_store_and_load_round_trip(lib, tmp_path):
    p = problem()
    n = p.tp2_size * p.per_type
    flat = np.random.default_rng(7).standard_normal(n)
    err = capi.errbuf()
    d = str(tmp_path).encode()
    nk = len(p.k)
    for i1 in range(nk):
        assert lib.song2_store_sources(p.spec, capi.dptr(flat), d, i1, err) == 0, err.value
    back = np.zeros(n)
    for i1 in range(nk):
        assert lib.song2_load_sources(p.spec, capi.dptr(back), d, i1, err) == 0, err.value
    assert np.array_equal(back, flat)
    # reference loop order, read independently
    view = flat.reshape(p.tp2_size, p.per_type)
    for i1 in range(nk):
        raw = np.fromfile(tmp_path / f"sources_{i1:03d}.dat", dtype=np.float64)
        pos = 0
        for tp in range(p.tp2_size):
            for i2 in range(i1 + 1):
                ln = len(p.tau) * int(p.k3_size[i1 * nk + i2])
                off = p.pair_offset(i1, i2)
                assert np.array_equal(raw[pos:pos + ln], view[tp, off:off + ln])
                pos += ln
        assert pos == raw.size


def test_missing_or_short_file_is_an_error(lib, tmp_path):
    p = problem()
    err = capi.errbuf()
    buf = np.zeros(p.tp2_size * p.per_type)
    assert lib.song2_load_sources(p.spec, capi.dptr(buf), str(tmp_path).encode(), 0, err) == 1
    (tmp_path / "sources_001.dat").write_bytes(b"\0" * 16)
    assert lib.song2_load_sources(p.spec, capi.dptr(buf), str(tmp_path).encode(), 1, err) == 1
    assert b"Error reading" in err.value
