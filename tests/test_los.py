"""Line-of-sight integration (SONG's transfer2.c / bessel2.c): the second-order
transfer functions of the sources.

CPU: the oracle's spherical Bessel functions against scipy and its 3j symbols
against sympy (the pins of the restatement: the reference's CLASS routines are
absent); the product's host side (3j recursion, l list, transfer k grids, type
layout) against the oracle, bit for bit where the work is integer or grid
arithmetic.  GPU: the device tables (j_l1, J_Llm and their x_min) and the
transfer functions against the oracle on seeded synthetic sources, for every
sampling and interpolation option of the reference, and on sources from the
evolver through the device pointer of a context.

Tolerances: j_l1 1e-12 of the row's largest value (the two sides use
different Bessel recurrences); J_Llm 1e-10 of the row's largest value (the
oracle's Racah 3j symbols from log-factorials carry about 1e-12 relative error
at l ~ 300); transfers 1e-9 of the largest |T| of the transfer type over all k
(different summation order of the same FP64 terms).
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from helpers import problem
from song_gb300 import capi

LOS_PROBLEM = dict(k_min=1e-3, k_max=0.01, k_size=4, k3_size=6, l_max=4, m=(0, 1, 2), tau_size=40,
                   sources="TEB")


def los_spec(lib, prob, l_max=60, l_logstep=1.25, l_linstep=10, **kw):
    los = capi.LosSpec()
    lib.song2_los_defaults(C.byref(los), C.byref(prob.spec), C.byref(prob.tables))
    n = lib.song2_l_list(l_max, l_logstep, l_linstep, None)
    ls = np.zeros(n, dtype=np.int32)
    lib.song2_l_list(l_max, l_logstep, l_linstep, capi.iptr(ls))
    los.l_size = n
    los.l = capi.iptr(ls)
    for key, val in kw.items():
        setattr(los, key, val)
    los._keep = ls
    return los


def synthetic_sources(prob, seed=7):
    """Seeded sources, smooth in k3 and tau, in the flat layout."""
    rng = np.random.default_rng(seed)
    src = np.zeros(prob.tp2_size * prob.per_type)
    n = len(prob.k)
    tau = prob.tau
    for tp in range(prob.tp2_size):
        for i1 in range(n):
            for i2 in range(i1 + 1):
                k3n = int(prob.k3_size[i1 * n + i2])
                off = prob.pair_offset(i1, i2)
                a, w, ph, wk = rng.normal(), rng.uniform(0.002, 0.02), rng.uniform(0, 6.3), rng.uniform(50, 400)
                kk = np.linspace(0, 1, k3n)
                blk = a * np.cos(w * tau[:, None] + wk * kk[None, :] * 0.01 + ph) * np.exp(-tau[:, None] / 8000.0)
                src[tp * prob.per_type + off: tp * prob.per_type + off + blk.size] = blk.ravel()
    return src


def tt_layout(lib, prob, los):
    n = lib.song2_transfer_types(C.byref(prob.spec), C.byref(los), None, None, None)
    t, l, m = (np.zeros(n, dtype=np.int32) for _ in range(3))
    lib.song2_transfer_types(C.byref(prob.spec), C.byref(los), capi.iptr(t), capi.iptr(l), capi.iptr(m))
    return t, l, m


def rel_err_per_type(gpu, ref, n_tt):
    g = gpu.reshape(n_tt, -1)
    r = ref.reshape(n_tt, -1)
    scale = np.max(np.abs(r), axis=1)
    diff = np.max(np.abs(g - r), axis=1)
    ok = scale > 0
    worst = np.max(diff[ok] / scale[ok]) if ok.any() else 0.0
    # rows whose reference is exactly zero must be zero on the GPU too
    zero_rows_bad = np.max(np.abs(g[~ok])) if (~ok).any() else 0.0
    return worst, zero_rows_bad


# ---------------------------------------------------------------- CPU pins

def test_oracle_bessel_matches_scipy():
    sp = pytest.importorskip("scipy.special")
    lmax = 700
    for x in (1e-6, 0.01, 0.2, 1.0, np.pi, 7.5, 50.0, 333.3, 650.0, 1200.0):
        ref = sp.spherical_jn(np.arange(lmax + 1), x)
        got = oracle.bessel_all(x, lmax)
        env = max(1.0 / max(x, 1.0), 1e-300)
        assert np.max(np.abs(got - ref)) <= 1e-13 * max(env, np.max(np.abs(ref))), x


def test_product_host_bessel_matches_scipy(lib):
    sp = pytest.importorskip("scipy.special")
    f = lib.s2los_bessel_all
    f.restype = None
    f.argtypes = [C.c_double, C.c_int, C.POINTER(C.c_double)]
    lmax = 700
    for x in (1e-6, 0.01, 0.2, 1.0, np.pi, 7.5, 50.0, 333.3, 650.0, 1200.0):
        out = np.zeros(lmax + 1)
        f(x, lmax, capi.dptr(out))
        ref = sp.spherical_jn(np.arange(lmax + 1), x)
        assert np.max(np.abs(out - ref)) <= 1e-13 * max(np.max(np.abs(ref)), 1e-300), x


def test_wigner3j_row_matches_sympy_and_oracle(lib):
    wig = pytest.importorskip("sympy.physics.wigner")
    out = np.zeros(64)
    lo, hi = C.c_int(), C.c_int()
    cases = [(2, 2, 0, 0), (2, 5, 2, -2), (4, 7, -2, 2), (3, 3, 1, -1), (4, 12, 0, 0), (0, 6, 0, 0), (4, 9, -4, 4),
             (2, 2, 2, -2), (5, 5, 2, -2)]
    for l2, l3, m2, m3 in cases:
        assert lib.song2_wigner3j_row(l2, l3, m2, m3, C.byref(lo), C.byref(hi), capi.dptr(out), 64) == 0
        for l1 in range(lo.value, hi.value + 1):
            ref = float(wig.wigner_3j(l1, l2, l3, -m2 - m3, m2, m3))
            assert abs(out[l1 - lo.value] - ref) <= 1e-14 * max(1.0, abs(ref)), (l1, l2, l3, m2, m3)
    olib = oracle.load()
    for l3 in (150, 999, 2000):
        for (l2, m2, m3) in ((4, 2, -2), (4, -4, 4), (2, 0, 0), (3, 2, -2)):
            assert lib.song2_wigner3j_row(l2, l3, m2, m3, C.byref(lo), C.byref(hi), capi.dptr(out), 64) == 0
            for l1 in range(lo.value, hi.value + 1):
                ref = olib.song2_oracle_wigner3j(l1, l2, l3, -m2 - m3, m2, m3)
                assert abs(out[l1 - lo.value] - ref) <= 1e-10 * max(1e-3, abs(ref)), (l1, l2, l3)


def test_l_list_matches_oracle(lib):
    for args in ((2000, 1.25, 36), (60, 1.25, 10), (500, 1.12, 40), (3, 1.5, 2), (100, 2.0, 1)):
        n = lib.song2_l_list(*args, None)
        mine = np.zeros(n, dtype=np.int32)
        lib.song2_l_list(*args, capi.iptr(mine))
        ref = oracle.l_list(*args)
        assert np.array_equal(mine, ref), args
        assert mine[0] == 2 and mine[-1] == args[0] and np.all(np.diff(mine) > 0)


@pytest.mark.parametrize("opts", [
    dict(),
    dict(k3_sampling=capi.K3_SAMPLING_BESSEL),
    dict(k3_extrapolation=capi.K3_EXTRAP_FLAT, extra_k3_oscillations_left=3, extra_k3_oscillations_right=5),
    dict(k3_extrapolation=capi.K3_EXTRAP_FLAT, extra_k3_oscillations_left=-1, extra_k3_oscillations_right=-1),
])
def test_transfer_k_grids_match_oracle(lib, opts):
    prob = problem(**LOS_PROBLEM)
    los = los_spec(lib, prob, **opts)
    n_pairs = len(prob.k) * (len(prob.k) + 1) // 2
    sz, ps, pn = (np.zeros(n_pairs, dtype=np.int32) for _ in range(3))
    err = capi.errbuf()
    n = lib.song2_transfer_k_grids(C.byref(prob.spec), C.byref(los), capi.iptr(sz), capi.iptr(ps), capi.iptr(pn),
                                   None, err)
    assert n > 0, err.value
    kk = np.zeros(n)
    lib.song2_transfer_k_grids(C.byref(prob.spec), C.byref(los), None, None, None, capi.dptr(kk), err)
    rsz, rps, rpn, rkk = oracle.transfer_k_grids(prob, los)
    assert np.array_equal(sz, rsz) and np.array_equal(ps, rps) and np.array_equal(pn, rpn)
    assert np.array_equal(kk, rkk)
    # every pair's grid ascends and holds the sources' k3 values it passed
    off = 0
    for p in range(n_pairs):
        g = kk[off: off + sz[p]]
        assert np.all(np.diff(g) > 0)
        off += sz[p]


def test_transfer_types_layout(lib):
    prob = problem(**LOS_PROBLEM)
    los = los_spec(lib, prob)
    t, l, m = tt_layout(lib, prob, los)
    ls = los._keep
    per = sum(1 for lv in ls for mm in (0, 1, 2) if mm <= lv)
    assert len(t) == 3 * per
    assert list(t[:per]) == [0] * per and list(t[per:2 * per]) == [1] * per
    # l major, m minor inside each type
    assert list(l[:3]) == [2, 2, 2] and list(m[:3]) == [0, 1, 2]


def test_recombination_time_is_the_visibility_peak(lib):
    prob = problem(**LOS_PROBLEM)
    tr = lib.song2_recombination_time(C.byref(prob.tables))
    assert 200.0 < tr < 400.0
    assert abs(tr - prob.tau_rec()) <= 2 * prob.tables.bg_dlntau * tr


def test_oracle_transfer_is_linear_in_the_sources(lib):
    """A property of the oracle itself: T(a S1 + S2) = a T(S1) + T(S2)."""
    prob = problem(**LOS_PROBLEM)
    los = los_spec(lib, prob, l_max=20, l_linstep=5)
    n_tt = lib.song2_transfer_types(C.byref(prob.spec), C.byref(los), None, None, None)
    err = capi.errbuf()
    nu = lib.song2_transfer_k_grids(C.byref(prob.spec), C.byref(los), None, None, None, None, err)
    s1, s2 = synthetic_sources(prob, 1), synthetic_sources(prob, 2)
    t1 = oracle.transfer(prob, los, s1, n_tt * nu)
    t2 = oracle.transfer(prob, los, s2, n_tt * nu)
    t12 = oracle.transfer(prob, los, 2.5 * s1 + s2, n_tt * nu)
    assert np.max(np.abs(t12 - (2.5 * t1 + t2))) <= 1e-12 * np.max(np.abs(t12))
    assert np.max(np.abs(t1)) > 0


# ---------------------------------------------------------------- GPU parity

def los_create(lib, prob, los):
    h = C.c_void_p()
    err = capi.errbuf()
    assert lib.song2_los_create(C.byref(prob.spec), C.byref(los), C.byref(h), err) == 0, err.value
    return h


def gpu_transfer(lib, h, src):
    import torch
    n_out = lib.song2_los_transfer_size(h)
    d_src = torch.from_numpy(src).cuda()
    d_out = torch.zeros(n_out, dtype=torch.float64, device="cuda")
    err = capi.errbuf()
    assert lib.song2_los_run(h, C.c_void_p(d_src.data_ptr()), C.c_void_p(d_out.data_ptr()), None, err) == 0, \
        err.value
    torch.cuda.synchronize()
    return d_out.cpu().numpy()


@pytest.mark.gpu
@pytest.mark.parametrize("lmax,kmax", [(60, 0.01), (300, 0.03)])
def test_device_tables_match_oracle(lib, lmax, kmax):
    prob = problem(**dict(LOS_PROBLEM, k_max=kmax))
    los = los_spec(lib, prob, l_max=lmax, l_linstep=max(10, lmax // 12))
    h = los_create(lib, prob, los)
    try:
        xs, nl1, Ls, ms, nr = (C.c_int() for _ in range(5))
        lib.song2_los_table_sizes(h, C.byref(xs), C.byref(nl1), C.byref(Ls), C.byref(ms), C.byref(nr))
        l1 = np.zeros(nl1.value, dtype=np.int32)
        jt = np.zeros((nl1.value, xs.value))
        J = np.zeros((nr.value, xs.value))
        xm = np.zeros(nr.value, dtype=np.int32)
        err = capi.errbuf()
        assert lib.song2_los_tables(h, capi.iptr(l1), capi.dptr(jt), capi.dptr(J), capi.iptr(xm), err) == 0
    finally:
        lib.song2_los_destroy(h)
    rl1, rjt, rJ, rxm = oracle.los_tables(prob, los)
    assert np.array_equal(l1, rl1)
    # j_l1: device recurrence vs the oracle's long-double one
    scale = np.maximum(np.max(np.abs(rjt), axis=1, keepdims=True), 1e-300)
    assert np.max(np.abs(jt - rjt) / scale) <= 1e-12
    # J rows from their x_min on (below it both sides ignore the values)
    assert np.array_equal(xm, rxm), np.nonzero(xm != rxm)
    for r in range(nr.value):
        a, b = J[r, xm[r]:], rJ[r, xm[r]:]
        s = np.max(np.abs(b))
        if s > 0:
            assert np.max(np.abs(a - b)) <= 1e-10 * s, r


LOS_CASES = [
    dict(),
    dict(tau_sampling=capi.TAU_SAMPLING_CUSTOM, tau_linstep=0.05),
    dict(tau_sampling=capi.TAU_SAMPLING_BESSEL),
    dict(tau_sampling=capi.TAU_SAMPLING_CUSTOM, tau_linstep=0.05, time_interpolation=capi.INTERP_CUBIC,
         k3_interpolation=capi.INTERP_CUBIC),
    dict(bessel_interpolation=capi.INTERP_CUBIC, k3_sampling=capi.K3_SAMPLING_BESSEL),
    dict(k3_extrapolation=capi.K3_EXTRAP_FLAT, extra_k3_oscillations_left=3, extra_k3_oscillations_right=5),
]


@pytest.mark.gpu
@pytest.mark.parametrize("opts", LOS_CASES)
def test_transfers_match_oracle(lib, opts):
    prob = problem(**LOS_PROBLEM)
    los = los_spec(lib, prob, **opts)
    src = synthetic_sources(prob)
    h = los_create(lib, prob, los)
    try:
        got = gpu_transfer(lib, h, src)
    finally:
        lib.song2_los_destroy(h)
    n_tt = lib.song2_transfer_types(C.byref(prob.spec), C.byref(los), None, None, None)
    ref = oracle.transfer(prob, los, src, got.size)
    worst, zero_bad = rel_err_per_type(got, ref, n_tt)
    assert worst <= 1e-9, worst
    assert zero_bad == 0.0
    assert np.max(np.abs(ref)) > 0


@pytest.mark.gpu
def test_transfers_of_evolver_sources_on_the_device(lib):
    """The evolver's device buffer feeds the line of sight directly; the one-shot
    host entry gives the same transfers."""
    from helpers import gpu_run  # noqa: F401
    prob = problem(k_min=1e-3, k_max=0.01, k_size=3, k3_size=4, l_max=6, m=(0, 1, 2), tau_size=30, sources="TEB")
    prob.set_first_order(oracle.first_order(prob, nthreads=4))
    los = los_spec(lib, prob, l_max=40, l_linstep=8)
    c = C.c_void_p()
    err = capi.errbuf()
    assert lib.song2_ctx_create(C.byref(prob.spec), C.byref(prob.tables), capi.SONG2_PREC_MIXED, C.byref(c), err) == 0
    h = los_create(lib, prob, los)
    try:
        assert lib.song2_ctx_run(c, None, err) == 0, err.value
        src = np.zeros(prob.tp2_size * prob.per_type)
        st = (capi.TripletStats * prob.n_triplets)()
        assert lib.song2_ctx_download(c, capi.dptr(src), st, err) == 0
        import torch
        n_out = lib.song2_los_transfer_size(h)
        d_out = torch.zeros(n_out, dtype=torch.float64, device="cuda")
        dsrc = lib.song2_ctx_device_sources(c)
        assert lib.song2_los_run(h, C.c_void_p(dsrc), C.c_void_p(d_out.data_ptr()), None, err) == 0, err.value
        torch.cuda.synchronize()
        got = d_out.cpu().numpy()
    finally:
        lib.song2_los_destroy(h)
        lib.song2_ctx_destroy(c)
    one = np.zeros(got.size)
    assert lib.song2_gpu_transfer(C.byref(prob.spec), C.byref(los), capi.dptr(src), capi.dptr(one), err) == 0
    assert np.array_equal(one, got)
    n_tt = lib.song2_transfer_types(C.byref(prob.spec), C.byref(los), None, None, None)
    ref = oracle.transfer(prob, los, src, got.size)
    worst, zero_bad = rel_err_per_type(got, ref, n_tt)
    assert worst <= 1e-9 and zero_bad == 0.0
