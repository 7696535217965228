"""Self-describing source files (perturb2_output, perturbations2.c:14688-15340)
in the layout the reference's python/songy.py reads.  The reader here restates
songy's parsing (SongBinary.get_binary_mapping / read_block and the block
numbers of Fixedk1k2File and FixedTauFile) so the files are checked as songy
would open them.  CPU only."""
import ctypes as C
import re

import numpy as np
import pytest

import oracle
from helpers import problem
from song_gb300 import capi


class SongyLike:
    def __init__(self, path, filetype):
        self.path = path
        with open(path, "rb") as f:
            head = f.read(65536).split(b"\0")[0].decode()
        lines = head.split("\n")
        assert filetype in lines[0]
        i = next(j for j, ln in enumerate(lines) if "BLOCK" in ln)
        self.mapping = []
        for ln in lines[i + 1:]:
            if not ln.startswith("#"):
                break
            self.mapping.append(re.split(r"\s{2,}", ln)[1:])

    def read_block(self, n):
        # songy: the type is element 1 of the split map line (without its '#'),
        # the count element 2, the byte offset element 4
        m = self.mapping[n]
        assert int(m[0]) == n
        dtype = "uint8" if m[1][0] == "c" else m[1][0]
        with open(self.path, "rb") as f:
            f.seek(int(m[4]))
            return np.fromfile(f, dtype=dtype, count=int(m[2]))

    def names(self, nblock, sblock):
        n = int(self.read_block(nblock)[0])
        raw = self.read_block(sblock).reshape(n, -1)
        return [bytes(r[r.nonzero()]).decode() for r in raw]


@pytest.fixture(scope="module")
def run(lib):
    p = problem(k_size=3, k3_size=4, sources="TEB", tau_size=12)
    p.set_first_order(oracle.first_order(p, nthreads=4))
    rng = np.random.default_rng(11)
    flat = rng.normal(size=p.tp2_size * p.per_type)
    return p, flat


def test_fixed_k1_k2_file(lib, run, tmp_path):
    p, flat = run
    path = str(tmp_path / "sources_song_k001.dat")
    err = capi.errbuf()
    assert lib.song2_write_sources_k(C.byref(p.spec), C.byref(p.tables), capi.dptr(flat), 2, 1, path.encode(),
                                     err) == 0, err.value
    f = SongyLike(path, "fixed k1 and k2")
    n = len(p.k)
    k3n = int(p.k3_size[2 * n + 1])
    assert f.read_block(2)[0] == p.k[2] and f.read_block(3)[0] == p.k[1]
    assert np.array_equal(f.read_block(5), p.tau)
    a, H = f.read_block(6), f.read_block(7)
    assert np.all(np.diff(a) > 0) and np.all(H > 0)
    off3 = p.pair_offset(2, 1) // len(p.tau)
    k3 = f.read_block(9)
    assert np.array_equal(k3, p.k3[off3: off3 + k3n])
    mu = f.read_block(10)
    assert np.allclose(mu, (k3 ** 2 - p.k[2] ** 2 - p.k[1] ** 2) / (2 * p.k[2] * p.k[1]), rtol=0, atol=1e-14)
    fo_names = f.names(11, 12)
    assert fo_names[0] == "phi" and "delta_cdm" in fo_names
    fo1 = f.read_block(13).reshape(len(p.tau), len(fo_names))
    assert np.all(np.isfinite(fo1))
    names = f.names(15, 16)
    assert names == [f"{k}_{l}_{m}" for k, l, m in p.tp_list()]
    assert f.read_block(17)[0] == len(p.tau) * k3n
    off = p.pair_offset(2, 1)
    for i, nm in enumerate(names):
        got = f.read_block(18 + i).reshape(len(p.tau), k3n)
        want = flat[i * p.per_type + off: i * p.per_type + off + len(p.tau) * k3n].reshape(len(p.tau), k3n)
        assert np.array_equal(got, want), nm


def test_fixed_tau_file(lib, run, tmp_path):
    p, flat = run
    it = 7
    path = str(tmp_path / "sources_song_tau007.dat")
    err = capi.errbuf()
    assert lib.song2_write_sources_tau(C.byref(p.spec), C.byref(p.tables), capi.dptr(flat), it, path.encode(),
                                       err) == 0, err.value
    f = SongyLike(path, "fixed tau")
    assert f.read_block(3)[0] == p.tau[it]
    z, a = f.read_block(2)[0], f.read_block(5)[0]
    assert abs(z - (1 / a - 1)) < 1e-12 * max(1.0, z)
    assert np.array_equal(f.read_block(8), p.k)
    n = len(p.k)
    sizes = f.read_block(9)
    assert list(sizes) == [int(p.k3_size[i1 * n + i2]) for i1 in range(n) for i2 in range(i1 + 1)]
    k3 = np.split(f.read_block(10), sizes[:-1].cumsum())
    assert np.array_equal(np.concatenate(k3), p.k3)
    fo_names = f.names(11, 12)
    assert f.read_block(13).size == n * len(fo_names)
    names = f.names(14, 15)
    assert len(names) == p.tp2_size
    for i in range(p.tp2_size):
        got = np.split(f.read_block(16 + i), sizes[:-1].cumsum())
        for (i1, i2), g in zip([(a_, b_) for a_ in range(n) for b_ in range(a_ + 1)], got):
            k3n = int(p.k3_size[i1 * n + i2])
            off = i * p.per_type + p.pair_offset(i1, i2) + it * k3n
            assert np.array_equal(g, flat[off: off + k3n])


def test_bad_arguments_are_errors(lib, run, tmp_path):
    p, flat = run
    err = capi.errbuf()
    path = str(tmp_path / "x.dat").encode()
    assert lib.song2_write_sources_k(C.byref(p.spec), C.byref(p.tables), capi.dptr(flat), 1, 2, path, err) == 1
    assert lib.song2_write_sources_tau(C.byref(p.spec), C.byref(p.tables), capi.dptr(flat), 99, path, err) == 1
    assert lib.song2_write_sources_k(C.byref(p.spec), C.byref(p.tables), capi.dptr(flat), 1, 0,
                                     str(tmp_path / "no" / "dir.dat").encode(), err) == 1
