"""delta-tilde line-of-sight sources and rescaled rotation coefficients (CPU).

The delta-tilde couplings (perturbations2.c:1285-1527) are built by the
reference from coupling_general in song_tools, which is not in the reference
tree; the call site defines them as
    prefactor * i^L * (-1)^m (2l+1) (l1 l2 l; 0 F -F) (l1 l2 l; m1 m2 -m).
Both the product's table (song2_delta_tilde_coupling) and the oracle's are
pinned here against exact 3j symbols (sympy), and the source terms against two
properties: they depend on first-order quantities only (so the difference of a
run with and without them does not depend on the ODE tolerance), and with
rescaled rotation coefficients every m-multipole of the sources is the
unrescaled one divided by sin(theta_k1)^m (perturbations2.c:6025-6064)."""
import ctypes as C

import numpy as np
import pytest

import oracle
from helpers import floored_errors, problem

FIELDS = (0, 1, 2)


def exact_coupling(field, l, m, l1, m1, l2):
    from sympy import Rational
    from sympy.physics.wigner import wigner_3j
    F = 0 if field == 0 else 2
    pre = Rational(1, 2) if field == 0 else 1
    if l2 < F or l < F:
        return 0.0
    L = l - l1 - l2
    if (abs(L) % 2 == 0) != (field != 2):
        return 0.0
    e = abs(L) // 2 if field != 2 else abs(L - 1) // 2
    m2 = m - m1
    v = pre * (-1) ** e * (-1) ** m * (2 * l + 1) * wigner_3j(l1, l2, l, 0, F, -F) * wigner_3j(l1, l2, l, m1, m2, -m)
    return float(v)


def test_couplings_match_exact_3j(lib, olib):
    pytest.importorskip("sympy")
    worst = 0.0
    n_nonzero = 0
    for field in FIELDS:
        for l in range(0, 6):
            for m in range(0, min(l, 4) + 1):
                for l1 in range(0, 4):
                    for m1 in range(-l1, l1 + 1):
                        for l2 in range(0, 4):
                            ref = exact_coupling(field, l, m, l1, m1, l2)
                            a = lib.song2_delta_tilde_coupling(field, l, m, l1, m1, l2)
                            b = olib.song2_oracle_delta_tilde_coupling(field, l, m, l1, m1, l2)
                            worst = max(worst, abs(a - ref), abs(b - ref))
                            n_nonzero += ref != 0.0
    assert n_nonzero > 300
    assert worst < 1e-13, worst


def test_temperature_coupling_is_symmetric(lib):
    """The reference skips the k1<->k2 symmetrisation of delta*delta for T because
    its coupling is symmetric under (l1,m1) <-> (l2,m2) (perturbations2.c:12367-12371)."""
    for l in range(0, 5):
        for m in range(0, l + 1):
            for l1 in range(0, 4):
                for m1 in range(-l1, l1 + 1):
                    for l2 in range(0, 4):
                        m2 = m - m1
                        if abs(m2) > l2:
                            continue
                        a = lib.song2_delta_tilde_coupling(0, l, m, l1, m1, l2)
                        b = lib.song2_delta_tilde_coupling(0, l, m, l2, m2, l1)
                        assert abs(a - b) < 1e-14


def _run(p, rtol=None):
    src, st = oracle.evolve(p, nthreads=8, rtol=rtol)
    assert np.all(st["status"] == 0)
    return src


@pytest.fixture(scope="module")
def dt_problem(lib, olib):
    p = problem(sources="TEB", l_max=5)
    p.set_first_order(oracle.first_order(p, nthreads=8))
    return p


def test_delta_tilde_terms_depend_on_first_order_only(dt_problem):
    p = dt_problem
    spec = p.spec
    diffs = []
    for rtol in (1e-3, 1e-5):
        spec.use_delta_tilde_in_los = 0
        off = _run(p, rtol)
        spec.use_delta_tilde_in_los = 1
        on = _run(p, rtol)
        spec.use_delta_tilde_in_los = 0
        diffs.append(on - off)
    d0, d1 = diffs
    scale = np.abs(d0).max()
    assert scale > 0
    # the terms are added to every T, E, B type of m the couplings reach
    per_tp = np.abs(d0.reshape(p.tp2_size, p.per_type)).max(axis=1)
    kinds = p.tp_list()
    assert all(per_tp[i] > 0 for i, (kind, l, m) in enumerate(kinds) if kind == "T")
    # differences agree to round-off of the sources they were added to
    src_scale = np.abs(_run(p)).max()
    assert np.abs(d0 - d1).max() < 1e-12 * src_scale


def test_delta_tilde_excludes_redshift_term(dt_problem):
    p = dt_problem
    spec = p.spec
    spec.use_delta_tilde_in_los = 1
    spec.has_redshift_in_los = 1
    try:
        with pytest.raises(RuntimeError, match="redshift"):
            oracle.evolve(p, nthreads=8)
    finally:
        spec.use_delta_tilde_in_los = 0
        spec.has_redshift_in_los = 0


def test_rescaled_geometry_self_checks(lib, olib):
    p = problem(k_min=1e-4, k_max=0.3, k_size=6, k3_size=5, l_max=6, m=(0, 1, 2, 3, 4), rescale_cmb_sources=1)
    dev = C.c_double()
    failures = []
    for (i1, i2, i3) in p.work_order():
        f = olib.song2_oracle_geometry_checks(C.byref(p.spec), i1, i2, i3, C.byref(dev))
        if f:
            failures.append((i1, i2, i3, f, dev.value))
    assert not failures, failures[:5]


def test_rescaled_sources_scale_as_sin_theta1(dt_problem):
    p = dt_problem
    plain = _run(p)
    p.spec.rescale_cmb_sources = 1
    try:
        resc = _run(p)
    finally:
        p.spec.rescale_cmb_sources = 0
    ms = np.array([m for (_, _, m) in p.tp_list()])
    expect = plain.reshape(p.tp2_size, p.per_type).copy()
    n = len(p.k)
    for (i1, i2, i3) in p.work_order():
        k1, k2, k = p.triplet_k(i1, i2, i3)
        cosk1k2 = (k * k - k1 * k1 - k2 * k2) / (2 * k1 * k2)
        cosk1k = (k1 + k2 * cosk1k2) / k
        sin1 = np.sqrt(max(0.0, 1 - cosk1k ** 2))
        nk3 = int(p.k3_size[i1 * n + i2])
        off = p.pair_offset(i1, i2)
        cols = slice(off + i3, off + len(p.tau) * nk3, nk3)
        if sin1 < 1e-6:
            continue
        expect[:, cols] /= (sin1 ** ms)[:, None]
    e = floored_errors(resc, expect.ravel(), p)
    assert np.max(e) < 10 * p.spec.rtol, np.max(e)
