"""Uneven batches (per-triplet hierarchy classes): every triplet of an uneven run
gives the sources of a uniform run with its own l_max and modes 0..m_max, and
zeros for the modes it does not evolve."""
import numpy as np
import pytest

import oracle
from helpers import problem

UNEVEN = dict(l_max=7, m=(0, 1, 2), sources="TEB")
CLASSES = dict(seed=20261203, l_base=4, l_cap=7, m_choices=(0, 2))


def tp_index(prob, kind, l, m):
    """Source-type index of (kind, l, m): T, E, B blocks of (l, m) pairs, l-major."""
    s = prob.spec
    ms = [s.m[i] for i in range(s.m_size)]

    def block(lmax):
        return sum(1 for ll in range(lmax + 1) for mm in ms if mm <= ll)

    base = 0
    for kk, lmax, on in (("T", s.l_max_los_t, s.has_source_T), ("E", s.l_max_los_p, s.has_source_E),
                         ("B", s.l_max_los_p, s.has_source_B)):
        if kk == kind:
            return base + sum(1 for ll in range(l) for mm in ms if mm <= ll) + sum(1 for mm in ms if mm < m and mm <= l)
        if on:
            base += block(lmax)
    raise ValueError(kind)


def uneven_problem():
    p = problem(**UNEVEN)
    p.set_uneven(**CLASSES)
    return p


@pytest.fixture(scope="module")
def uneven():
    p = uneven_problem()
    p.set_first_order(oracle.first_order(p, nthreads=8))
    src, st = oracle.evolve(p, nthreads=8)
    return p, src, st


def pair_order(p):
    n = len(p.k)
    out = []
    for i1 in range(n):
        for i2 in range(i1 + 1):
            for i3 in range(int(p.k3_size[i1 * n + i2])):
                out.append((i1, i2, i3))
    return out


def test_classes_cover_the_batch(uneven):
    p, _, st = uneven
    assert len(p.classes) > 1
    assert np.all(st["status"] == 0)
    sizes = p.class_sizes()
    assert sizes.min() < sizes.max()


def test_oracle_uneven_equals_uniform_per_class(uneven):
    p, src, _ = uneven
    a = src.reshape(p.tp2_size, p.per_type)
    order = pair_order(p)
    for cls, (L, mm) in enumerate(p.classes):
        members = [order[i] for i in np.nonzero(p.triplet_class == cls)[0]]
        q = problem(**dict(UNEVEN, l_max=L, m=tuple(range(mm + 1))))
        q.fo_l_max = p.fo_l_max
        q.set_first_order(p.fo)
        work = q.work_order()
        items = [work.index(t) for t in members]
        ref, st = oracle.evolve(q, nthreads=8, items=items)
        assert np.all(st["status"][items] == 0)
        b = ref.reshape(q.tp2_size, q.per_type)
        for (i1, i2, i3) in members:
            ta, tb = p.triplet_view(a, i1, i2, i3), q.triplet_view(b, i1, i2, i3)
            for kind, lmax in (("T", 2), ("E", 2), ("B", 2)):
                for l in range(lmax + 1):
                    for m in range(min(l, 2) + 1):
                        row = ta[tp_index(p, kind, l, m)]
                        if m <= mm:
                            assert np.array_equal(row, tb[tp_index(q, kind, l, m)]), (cls, kind, l, m)
                        else:
                            assert not np.any(row), (cls, kind, l, m)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_gpu_uneven_matches_oracle(lib, uneven, precision):
    """The class-per-item kernel on an uneven batch agrees with the oracle."""
    from helpers import floored_errors, gpu_run
    p, ref, _ = uneven
    src, st, _ = gpu_run(lib, p, precision)
    assert np.all(st["status"] == 0)
    assert np.max(floored_errors(src, ref, p)) < 10 * p.spec.rtol


@pytest.mark.gpu
def test_gpu_uneven_launch_groups_match_single_launch(lib, uneven, monkeypatch):
    """Splitting an uneven batch into launch groups by class size (large plans
    first) computes the same sources as one launch, within the solver tolerance:
    the two groups run different instantiations of the kernel (register budgets
    for one and for two CTAs per SM), compiled separately, whose floating-point
    contractions may differ in the last bits."""
    from helpers import floored_errors, gpu_run
    p, ref, _ = uneven
    one, _, _ = gpu_run(lib, p, 1)
    monkeypatch.setenv("SONG2_CLASS_SPLIT_BYTES", "20000")
    two, st, _ = gpu_run(lib, p, 1)
    assert np.all(st["status"] == 0)
    assert np.max(floored_errors(two, one, p)) < 10 * p.spec.rtol
    assert np.max(floored_errors(two, ref, p)) < 10 * p.spec.rtol


@pytest.mark.gpu
def test_gpu_uneven_with_los_options_and_rsa_matches_oracle(lib):
    """Hierarchy classes with delta-tilde sources, rescaled rotation coefficients and
    the RSA (an m_max = 0 class still needs the rotation coefficients up to m = 2)."""
    from helpers import floored_errors, gpu_run
    p = problem(**UNEVEN, use_delta_tilde_in_los=1, rescale_cmb_sources=1, radiation_streaming_approximation=1)
    p.set_uneven(**CLASSES)
    p.set_first_order(oracle.first_order(p, nthreads=8))
    ref, _ = oracle.evolve(p, nthreads=8)
    tight, _ = oracle.evolve(p, nthreads=8, rtol=p.spec.rtol / 100)
    # the RSA's T monopole source carries the solver's rtol-level error amplified
    bound = max(10 * p.spec.rtol, 3 * np.max(floored_errors(ref, tight, p)))
    src, st, _ = gpu_run(lib, p, 1)
    assert np.all(st["status"] == 0)
    assert np.max(floored_errors(src, ref, p)) < bound
