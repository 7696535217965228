"""delta-tilde line-of-sight sources and rescaled rotation coefficients (CPU).

The delta-tilde couplings (perturbations2.c:1285-1527) are built by the
reference from coupling_general in song_tools, which is not in the reference
tree; the call site defines them as
    prefactor * i^L * (-1)^m (2l+1) (l1 l2 l; 0 F -F) (l1 l2 l; m1 m2 -m).
Both the product's table (song2_delta_tilde_coupling) and the oracle's are
pinned here against exact 3j symbols (sympy).  The source terms are pinned by
an independent numpy restatement at one sampling time, and by two properties:
they depend on first-order quantities only (so the difference of a run with and
without them does not depend on the ODE tolerance), and with rescaled rotation
coefficients every m-multipole of the sources is the unrescaled one divided by
sin(theta_k1)^m (perturbations2.c:6025-6064)."""
import ctypes as C
import math

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


def _spline(y, dd, x0, dx, x):
    """Natural cubic spline on a uniform grid (rows of y and dd), evaluated at x."""
    u = (x - x0) / dx
    i = min(max(int(np.floor(u)), 0), len(y) - 2)
    b = u - i
    a = 1.0 - b
    return a * y[i] + b * y[i + 1] + ((a ** 3 - a) * dd[i] + (b ** 3 - b) * dd[i + 1]) * dx * dx / 6.0


def test_delta_tilde_terms_against_independent_restatement(dt_problem):
    """The delta-tilde part of the T, E, B sources (the difference of runs with and
    without it), rebuilt in numpy for two triplets at the last sampling time from
    the first-order table, the background table, Legendre rotation coefficients
    (scipy) and exact 3j couplings (sympy), following perturbations2.c:12339-12398,
    12509-12561 and 12658-12710 term by term."""
    pytest.importorskip("sympy")
    from scipy.special import lpmv
    from song_gb300 import capi
    p = dt_problem
    spec = p.spec
    spec.use_delta_tilde_in_los = 0
    off = _run(p)
    spec.use_delta_tilde_in_los = 1
    on = _run(p)
    spec.use_delta_tilde_in_los = 0
    diff = (on - off).reshape(p.tp2_size, p.per_type)
    L1 = p.fo_l_max + 1
    iI, iE, iCG = capi.FO_I, capi.FO_I + L1, capi.FO_I + 3 * L1
    tau = p.tau[-1]
    x = np.log(tau)
    t = p.tables
    kd = np.exp(_spline(p.bg[:, capi.BG_LN_KAPPA_DOT], p.bg_dd[:, capi.BG_LN_KAPPA_DOT], t.bg_lntau0, t.bg_dlntau, x))
    emk = np.exp(-_spline(p.bg[:, capi.BG_KAPPA], p.bg_dd[:, capi.BG_KAPPA], t.bg_lntau0, t.bg_dlntau, x))
    Q = spec.l_max_los_quadratic_t
    assert spec.l_max_los_quadratic_p == Q
    checked = 0
    for (i1, i2, i3) in p.work_order()[:2]:
        k1, k2, k = p.triplet_k(i1, i2, i3)
        c12 = (k * k - k1 * k1 - k2 * k2) / (2 * k1 * k2)
        ck1, ck2 = (k1 + k2 * c12) / k, (k2 + k1 * c12) / k
        f1 = _spline(p.fo[i1], p.fo_dd[i1], p.fo_lntau0, p.fo_dlntau, x)
        f2 = _spline(p.fo[i2], p.fo_dd[i2], p.fo_lntau0, p.fo_dlntau, x)

        def rot(which, l, m):
            if l < 0 or abs(m) > l:
                return 0.0
            am = abs(m)
            cth = ck1 if which == 1 else ck2
            v = np.sqrt(math.factorial(l - am) / math.factorial(l + am)) * lpmv(am, l, cth)
            if which == 2:
                v *= (-1) ** am
            return v * (-1) ** am if m < 0 else v

        def cE(f, l):
            if l < 2:
                return 0.0
            v = -f[iE + l]
            if l == 2:
                v -= np.sqrt(6) * 0.1 * (f[iI + 2] - np.sqrt(6) * f[iE + 2])
            return v

        view = diff
        n = len(p.k)
        nk3 = int(p.k3_size[i1 * n + i2])
        col = p.pair_offset(i1, i2) + (len(p.tau) - 1) * nk3 + i3
        for tp, (kind, l, m) in enumerate(p.tp_list()):
            field = "TEB".index(kind)
            if (kind == "E" and l < 2) or (kind == "B" and (l < 2 or m == 0)):
                continue
            dd = dc = 0.0
            for l1 in range(Q + 1):
                for l2 in range(abs(l1 - l), min(l1 + l, Q) + 1):
                    if ((l1 + l2 + l) % 2 != 0) != (field == 2):
                        continue
                    for m1 in range(-l1, l1 + 1):
                        m2 = m - m1
                        cpl = exact_coupling(field, l, m, l1, m1, l2) if abs(m2) <= l2 else 0.0
                        I1, I2 = rot(1, l1, m1) * f1[iI + l1], rot(2, l1, m1) * f2[iI + l1]
                        if field == 0:
                            c1, c2 = rot(1, l2, m2) * f1[iCG + l2], rot(2, l2, m2) * f2[iCG + l2]
                            dd += cpl * 2 * I1 * rot(2, l2, m2) * f2[iI + l2]
                            dc += cpl * (I1 * c2 + I2 * c1)
                        else:
                            E1, E2 = rot(1, l2, m2) * f1[iE + l2], rot(2, l2, m2) * f2[iE + l2]
                            cI1, cI2 = rot(1, l1, m1) * f1[iCG + l1], rot(2, l1, m1) * f2[iCG + l1]
                            cE1, cE2 = rot(1, l2, m2) * cE(f1, l2), rot(2, l2, m2) * cE(f2, l2)
                            dd += cpl * (I1 * E2 + I2 * E1)
                            dc += cpl * 0.5 * (I1 * cE2 + cI1 * E2 + I2 * cE1 + cI2 * E1)
            expect = (-2 * kd * 0.5 * dd - 2 * kd * dc) * emk
            got = view[tp, col]
            scale = max(abs(expect), 1e-300)
            assert abs(got - expect) <= 1e-9 * scale + 1e-14 * np.abs(view[tp]).max(), (kind, l, m, got, expect)
            checked += expect != 0.0
    assert checked > 10
