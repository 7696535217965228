"""k and k3 grids (perturb2_get_k_lists, perturbations2.c:1973-1984) and the
flat source layout."""
import numpy as np

from helpers import problem


def test_k3_clipping_rule(lib):
    p = problem(k_min=1e-4, k_max=0.05, k_size=8, k3_size=6)
    n = len(p.k)
    off = 0
    for i1 in range(n):
        for i2 in range(i1 + 1):
            k1, k2 = p.k[i1], p.k[i2]
            nk3 = p.k3_size[i1 * n + i2]
            g = p.k3[off: off + nk3]
            off += nk3
            lo = max(abs(k1 - k2) + 1e-10, (k1 + k2) / 100, p.k[0])
            hi = min(k1 + k2 - 1e-10, p.k[-1])
            assert np.isclose(g[0], lo, rtol=1e-14) and np.isclose(g[-1], hi, rtol=1e-14)
            assert np.all(np.diff(g) > 0)
    assert p.n_triplets == 6 * n * (n + 1) // 2


def test_pair_offsets_tile_the_buffer(lib):
    p = problem()
    n = len(p.k)
    seen = []
    for i1 in range(n):
        for i2 in range(i1 + 1):
            seen.append((p.pair_offset(i1, i2), len(p.tau) * p.k3_size[i1 * n + i2]))
    seen.sort()
    pos = 0
    for off, ln in seen:
        assert off == pos
        pos += ln
    assert pos == p.per_type
