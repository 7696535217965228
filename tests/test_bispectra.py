"""Intrinsic bispectrum of the second-order transfer functions (SONG's
bispectra2.c): the k3, k2, k1 and r integrals and the geometrical factors.

CPU: the oracle's 6j symbols against sympy; the reference's own checks that the
full geometrical factor of M3 = 0 reduces to 8/pi^3 (bispectra2.c:2826-2840)
and that odd l1 + l2 + l3 vanish for T and E when M3 > 0 (:660-675);
the configuration list; linearity of the oracle in the second-order transfers;
the quadratic correction.  GPU: the product against the oracle on seeded
synthetic transfers for every option (fields T, E and B, m lists with and
without M3 > 0, linear and cubic interpolation in k1, k2 and in the Bessel
functions).

Tolerance: 1e-8 of the largest |b| of each field combination.  The product
folds the q sums of the k2 and k1 integrals into weights over the k grid before
the dot products (the reference interpolates first, then sums), and it takes
its 3j and 6j symbols from a double-precision table of ln n! (the oracle from
long double), so the two agree to rounding, not bit for bit.
"""
import ctypes as C
import math

import numpy as np
import pytest

import oracle
from helpers import problem
from song_gb300 import capi
from test_los import los_spec

BI_PROBLEM = dict(k_min=1e-3, k_max=0.01, k_size=4, k3_size=6, l_max=4, tau_size=40, sources="TEB")


def first_order_inputs(prob, los, fields, r_size=6, q_size=60, seed=3):
    """r grid around recombination, q grid inside the k range, P(q) and
    seeded synthetic first-order transfers (smooth, oscillating in q)."""
    rng = np.random.default_rng(seed)
    tau0, trec = los.tau0, los.tau_rec
    r = np.linspace(tau0 - 1.4 * trec, tau0 - 0.6 * trec, r_size)
    k = prob.k
    q = np.linspace(k[0] * 1.05, k[-1], q_size)
    pk = 2 * np.pi ** 2 * 2.1e-9 * (q / 0.05) ** (0.966 - 1) / q ** 3
    ls = np.array(los._keep)
    T1 = np.zeros((len(fields), len(ls), q_size))
    for f in range(len(fields)):
        for i, l in enumerate(ls):
            a, ph = rng.normal(), rng.uniform(0, 6.3)
            T1[f, i] = a * np.cos(q * (tau0 - trec) / (1 + 0.01 * l) + ph) * np.exp(-q / 0.02)
    return r, q, pk, T1


def synthetic_transfers(lib, prob, los, seed=5):
    n_tt = lib.song2_transfer_types(C.byref(prob.spec), C.byref(los), None, None, None)
    sz, _, _, kk = oracle.transfer_k_grids(prob, los)
    rng = np.random.default_rng(seed)
    out = np.zeros((n_tt, len(kk)))
    for t in range(n_tt):
        a, w, ph = rng.normal(), rng.uniform(200, 2000), rng.uniform(0, 6.3)
        out[t] = a * np.cos(w * kk + ph)
    return out.ravel(), n_tt, len(kk)


def bispectra_spec(fields, r, q, pk, T1, k1=capi.INTERP_LINEAR, k2=capi.INTERP_LINEAR):
    bs = capi.BispectraSpec()
    bf = np.array(fields, dtype=np.int32)
    bs.bf_size = len(fields)
    bs.bf = capi.iptr(bf)
    bs.r_size, bs.r = len(r), capi.dptr(r)
    bs.q_size, bs.q = len(q), capi.dptr(q)
    bs.pk = capi.dptr(pk)
    T1c = np.ascontiguousarray(T1)
    bs.transfer1 = capi.dptr(T1c)
    bs.k1_interpolation, bs.k2_interpolation = k1, k2
    bs._keep = (bf, r, q, pk, T1c)
    return bs


def n_configs(lib, ls):
    arr = np.ascontiguousarray(ls, dtype=np.int32)
    return lib.song2_bispectra_configs(len(arr), capi.iptr(arr), None, None, None)


# ------------------------------------------------------------------ CPU

def test_oracle_6j_matches_sympy():
    wigner = pytest.importorskip("sympy.physics.wigner")
    lib = oracle.load()
    rng = np.random.default_rng(1)
    n = 0
    while n < 40:
        a, b, d, e = (int(v) for v in rng.integers(0, 9, 4))
        c = int(rng.integers(abs(a - b), a + b + 1))
        f = int(rng.integers(0, 5))
        want = float(wigner.wigner_6j(a, b, c, d, e, f))
        got = lib.song2_oracle_wigner6j(a, b, c, d, e, f)
        assert abs(got - want) < 1e-13, (a, b, c, d, e, f, got, want)
        n += 1


def w3j_row_value(lib, j1, j2, j3, m1, m2, m3):
    """(j1 j2 j3; m1 m2 m3) from the product's Schulten-Gordon row in j1."""
    assert m1 == -m2 - m3
    out = np.zeros(2 * (j2 + j3) + 2)
    lo, hi = C.c_int(), C.c_int()
    if lib.song2_wigner3j_row(j2, j3, m2, m3, C.byref(lo), C.byref(hi), capi.dptr(out), len(out)):
        return 0.0
    return out[j1 - lo.value] if lo.value <= j1 <= hi.value else 0.0


@pytest.mark.parametrize("l1,l2,l3", [(2, 3, 5), (10, 12, 20), (101, 150, 201), (800, 1200, 1500)])
def test_m0_geometry_reduces_to_8_over_pi_cubed(lib, l1, l2, l3):
    """bispectra2.c:2826-2840: for M3 = 0 the full formula (four 3j symbols and
    a 6j) with the (l1 l2 l3; 0 0 0) symbol divided out equals 8/pi^3; here
    with the oracle's 6j in long double and 3j rows by recursion."""
    w6 = oracle.load().song2_oracle_wigner6j
    L1, L3 = l1, l3
    pref = 8 / math.pi ** 3 * (2 * L1 + 1) * (2 * L3 + 1)
    f3 = w3j_row_value(lib, L3, 0, l3, 0, 0, 0)
    f1 = w3j_row_value(lib, L1, l1, 0, 0, 0, 0)
    fl = w3j_row_value(lib, L1, l2, L3, 0, 0, 0)
    f123 = w3j_row_value(lib, l1, l2, l3, 0, 0, 0)
    f6 = w6(L1, L3, l2, l3, l1, 0)
    geometry = f3 * f1 * fl * f6 / f123
    sign = 1 if ((l3 + L3 - l1 - L1) // 2) % 2 == 0 else -1
    assert abs(sign * pref * geometry - 8 / math.pi ** 3) < 1e-9 * 8 / math.pi ** 3


def test_configuration_list(lib):
    ls = np.array([2, 3, 5, 8, 13, 21, 34], dtype=np.int32)
    n = n_configs(lib, ls)
    i1, i2, i3 = (np.zeros(n, dtype=np.int32) for _ in range(3))
    lib.song2_bispectra_configs(len(ls), capi.iptr(ls), capi.iptr(i1), capi.iptr(i2), capi.iptr(i3))
    want = [(a, b, c) for a in range(len(ls)) for b in range(a + 1) for c in range(b + 1)
            if abs(ls[a] - ls[b]) <= ls[c] <= ls[a] + ls[b]]
    assert list(zip(i1, i2, i3)) == want


def test_oracle_bispectrum_is_linear_in_the_transfers(lib):
    prob = problem(**BI_PROBLEM, m=(0, 1, 2))
    los = los_spec(lib, prob, l_max=12, l_logstep=1.5, l_linstep=4)
    fields = [0, 1]
    r, q, pk, T1 = first_order_inputs(prob, los, fields, r_size=4, q_size=30)
    bs = bispectra_spec(fields, r, q, pk, T1)
    t2a, n_tt, nu = synthetic_transfers(lib, prob, los, seed=5)
    t2b, _, _ = synthetic_transfers(lib, prob, los, seed=6)
    n = n_configs(lib, los._keep) * len(fields) ** 3
    ba = oracle.bispectra(prob, los, bs, t2a, n)
    bb = oracle.bispectra(prob, los, bs, t2b, n)
    bab = oracle.bispectra(prob, los, bs, 2.0 * t2a - 0.5 * t2b, n)
    scale = np.max(np.abs(ba)) + np.max(np.abs(bb))
    assert scale > 0
    assert np.max(np.abs(bab - (2.0 * ba - 0.5 * bb))) < 1e-12 * scale


def test_quadratic_correction(lib):
    b = np.array([1.0, -2.0, 3.0])
    bq = np.array([8.0, 16.0, -8.0])
    b1 = b.copy()
    lib.song2_bispectra_add_quadratic(capi.dptr(b1), capi.dptr(bq), 3, 0)
    assert np.array_equal(b1, b - 3 / 8 * bq)
    b2 = b.copy()
    lib.song2_bispectra_add_quadratic(capi.dptr(b2), capi.dptr(bq), 3, 1)
    assert np.array_equal(b2, b + 1 / 8 * bq)


# ------------------------------------------------------------------ GPU

CASES = [
    dict(fields=(0, 1), m=(0, 1, 2)),
    dict(fields=(0,), m=(0,), k1=capi.INTERP_CUBIC, k2=capi.INTERP_CUBIC),
    dict(fields=(0, 1), m=(0, 2), k2=capi.INTERP_CUBIC, bessel=capi.INTERP_CUBIC),
    dict(fields=(0, 1, 2), m=(0, 1, 2)),
]


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=["TE_m012", "T_m0_cubic", "TE_m02_cubic_bessel", "TEB_odd"])
def test_bispectra_match_oracle(lib, case):
    prob = problem(**BI_PROBLEM, m=case["m"])
    kw = {}
    if "bessel" in case:
        kw["bessel_interpolation"] = case["bessel"]
    los = los_spec(lib, prob, l_max=30, l_logstep=1.25, l_linstep=6, **kw)
    fields = list(case["fields"])
    r, q, pk, T1 = first_order_inputs(prob, los, fields)
    bs = bispectra_spec(fields, r, q, pk, T1, case.get("k1", capi.INTERP_LINEAR),
                        case.get("k2", capi.INTERP_LINEAR))
    t2, n_tt, nu = synthetic_transfers(lib, prob, los)
    n = n_configs(lib, los._keep) * len(fields) ** 3
    got = np.zeros(n)
    err = capi.errbuf()
    assert lib.song2_gpu_bispectra(C.byref(prob.spec), C.byref(los), C.byref(bs), capi.dptr(t2), capi.dptr(got),
                                   err) == 0, err.value
    ref = oracle.bispectra(prob, los, bs, t2, n)
    nb = len(fields) ** 3
    g, w = got.reshape(nb, -1), ref.reshape(nb, -1)
    for i in range(nb):
        scale = np.max(np.abs(w[i]))
        if scale == 0:
            assert np.max(np.abs(g[i])) == 0
            continue
        assert np.max(np.abs(g[i] - w[i])) <= 1e-8 * scale, (i, np.max(np.abs(g[i] - w[i])) / scale)
    assert np.any(ref != 0)


@pytest.mark.gpu
def test_bispectra_handle_on_device_transfers(lib):
    """The handle path: transfers already on the device (as song2_los_run
    leaves them), two runs, identical results."""
    import torch
    prob = problem(**BI_PROBLEM, m=(0, 1, 2))
    los = los_spec(lib, prob, l_max=30, l_logstep=1.25, l_linstep=6)
    fields = [0, 1]
    r, q, pk, T1 = first_order_inputs(prob, los, fields)
    bs = bispectra_spec(fields, r, q, pk, T1)
    t2, n_tt, nu = synthetic_transfers(lib, prob, los)
    err = capi.errbuf()
    lh = C.c_void_p()
    assert lib.song2_los_create(C.byref(prob.spec), C.byref(los), C.byref(lh), err) == 0, err.value
    bh = C.c_void_p()
    try:
        assert lib.song2_bispectra_create(lh, C.byref(bs), C.byref(bh), err) == 0, err.value
        n = lib.song2_bispectra_size(bh)
        d_in = torch.tensor(t2, dtype=torch.float64, device="cuda")
        d_out = torch.zeros(n, dtype=torch.float64, device="cuda")
        outs = []
        for _ in range(2):
            assert lib.song2_bispectra_run(bh, C.c_void_p(d_in.data_ptr()), C.c_void_p(d_out.data_ptr()), None,
                                           err) == 0, err.value
            outs.append(d_out.cpu().numpy().copy())
        assert np.array_equal(outs[0], outs[1])
        assert lib.song2_bispectra_last_ms(bh) > 0
        one = np.zeros(n)
        assert lib.song2_gpu_bispectra(C.byref(prob.spec), C.byref(los), C.byref(bs), capi.dptr(t2),
                                       capi.dptr(one), err) == 0
        assert np.array_equal(one, outs[0])
    finally:
        if bh:
            lib.song2_bispectra_destroy(bh)
        lib.song2_los_destroy(lh)


@pytest.mark.gpu
def test_bispectra_argument_errors(lib):
    prob = problem(**BI_PROBLEM, m=(0,))
    los = los_spec(lib, prob, l_max=20, l_logstep=1.25, l_linstep=6)
    r, q, pk, T1 = first_order_inputs(prob, los, [0])
    err = capi.errbuf()
    lh = C.c_void_p()
    assert lib.song2_los_create(C.byref(prob.spec), C.byref(los), C.byref(lh), err) == 0, err.value
    try:
        bh = C.c_void_p()
        q_bad = q.copy()
        q_bad[-1] = prob.k[-1] * 1.5   # beyond the sources' k range
        bs = bispectra_spec([0], r, q_bad, pk, T1)
        assert lib.song2_bispectra_create(lh, C.byref(bs), C.byref(bh), err) == 1
        assert b"beyond" in err.value
        bs = bispectra_spec([0, 0], r, q, pk, np.concatenate([T1, T1]))
        assert lib.song2_bispectra_create(lh, C.byref(bs), C.byref(bh), err) == 1
        assert b"distinct" in err.value
    finally:
        lib.song2_los_destroy(lh)


def unsym_checks(lib, ls, b, nbf):
    """The reference's own checks after its bispectrum loops (bispectra2.c:640-705),
    on the symmetrised output: for an even-parity bispectrum with M3 > 0 in the m
    list every configuration with odd l1 + l2 + l3 vanishes; returns the largest
    such value relative to the largest value."""
    ls = np.ascontiguousarray(ls, dtype=np.int32)
    n = lib.song2_bispectra_configs(len(ls), capi.iptr(ls), None, None, None)
    i1, i2, i3 = (np.zeros(n, dtype=np.int32) for _ in range(3))
    lib.song2_bispectra_configs(len(ls), capi.iptr(ls), capi.iptr(i1), capi.iptr(i2), capi.iptr(i3))
    odd = (ls[i1] + ls[i2] + ls[i3]) % 2 == 1
    bb = b.reshape(nbf ** 3, n)
    return float(np.max(np.abs(bb[:, odd])) / np.max(np.abs(bb))) if odd.any() else 0.0, odd


def test_oracle_parity_check(lib):
    """bispectra2.c:660-675: with m_max > 0, odd l1 + l2 + l3 give exactly zero
    for T and E (the (L1 l2 L3; 0 0 0) symbol vanishes for them)."""
    prob = problem(**BI_PROBLEM, m=(0, 1, 2))
    los = los_spec(lib, prob, l_max=12, l_logstep=1.5, l_linstep=4)
    fields = [0, 1]
    r, q, pk, T1 = first_order_inputs(prob, los, fields, r_size=4, q_size=30)
    bs = bispectra_spec(fields, r, q, pk, T1)
    t2, _, _ = synthetic_transfers(lib, prob, los)
    n = n_configs(lib, los._keep) * 8
    b = oracle.bispectra(prob, los, bs, t2, n)
    worst, odd = unsym_checks(lib, los._keep, b, 2)
    assert odd.any() and worst == 0.0


@pytest.mark.gpu
def test_bispectra_reference_checks_on_gpu(lib):
    """The same parity check on the GPU output (bispectra2.c:660-675): with
    M3 > 0 in the m list, odd l1 + l2 + l3 give exactly zero for T and E."""
    prob = problem(**BI_PROBLEM, m=(0, 1, 2))
    los = los_spec(lib, prob, l_max=30, l_logstep=1.25, l_linstep=6)
    fields = [0, 1]
    r, q, pk, T1 = first_order_inputs(prob, los, fields)
    bs = bispectra_spec(fields, r, q, pk, T1)
    t2, n_tt, nu = synthetic_transfers(lib, prob, los)
    n = n_configs(lib, los._keep) * 8
    got = np.zeros(n)
    err = capi.errbuf()
    assert lib.song2_gpu_bispectra(C.byref(prob.spec), C.byref(los), C.byref(bs), capi.dptr(t2), capi.dptr(got),
                                   err) == 0, err.value
    worst, odd = unsym_checks(lib, los._keep, got, 2)
    assert odd.any() and worst == 0.0
