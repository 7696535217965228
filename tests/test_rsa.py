"""Radiation-streaming approximation (CPU): the free-streaming time, the switch
gating, and the approximation against the fully evolved hierarchies.

After photon decoupling the RSA replaces the photon and neutrino hierarchies by
the algebraic monopole and dipole of perturb2_rsa_variables
(perturbations2.c:9773-10164); on subhorizon scales it is a good approximation
of the evolved solution, which the oracle (with and without the RSA) shows."""
import ctypes as C

import numpy as np
import pytest

import oracle
from helpers import floored_errors, problem
from song_gb300 import capi


@pytest.fixture(scope="module")
def rsa_problem(lib, olib):
    p = problem(sources="TEB", l_max=5)
    p.set_first_order(oracle.first_order(p, nthreads=8))
    return p


def test_free_streaming_time(lib, rsa_problem):
    """tau_c/tau = 1/(kappa' tau) crosses the trigger once, after recombination."""
    p = rsa_problem
    x = p.tables.bg_lntau0 + p.tables.bg_dlntau * np.arange(p.tables.bg_size)
    g = -p.bg[:, capi.BG_LN_KAPPA_DOT] - x - np.log(capi.RSA_TRIGGER_TAU_C_OVER_TAU)
    # one sign change (the bisection's bracket), though not strictly monotonic at
    # the hydrogen-recombination onset, far below the trigger
    assert np.count_nonzero(np.diff(np.sign(g)) != 0) == 1
    j = int(np.argmax(g > 0))
    x0 = x[j - 1] - g[j - 1] * (x[j] - x[j - 1]) / (g[j] - g[j - 1])
    tfs = p.tables.tau_free_streaming
    assert abs(np.log(tfs) - x0) < 1e-3
    assert p.tau_rec() < tfs < p.tau0


def _run(p, **kw):
    spec = capi.Spec.from_buffer_copy(p.spec)
    for k, v in kw.items():
        setattr(spec, k, v)
    saved = p.spec
    p.spec = spec
    try:
        src, st = oracle.evolve(p, nthreads=8)
    finally:
        p.spec = saved
    assert np.all(st["status"] == 0)
    return src, st


def test_rsa_close_to_full_hierarchies(rsa_problem):
    p = rsa_problem
    full, st_full = _run(p)
    rsa, st_rsa = _run(p, radiation_streaming_approximation=capi.SONG2_RSA_MD)
    assert not np.array_equal(full, rsa)
    # T, E, B sources within a few per cent of their maximum (the RSA neglects O(1/(k tau)))
    assert np.max(floored_errors(rsa, full, p)) < 5e-2


def test_rsa_switch_gating(rsa_problem):
    """A trigger no triplet reaches leaves the run bit for bit unchanged."""
    p = rsa_problem
    full, _ = _run(p)
    same, _ = _run(p, radiation_streaming_approximation=capi.SONG2_RSA_MD,
                   radiation_streaming_trigger_tau_over_tau_k=1e12)
    assert np.array_equal(full, same)


def test_reio_terms_are_small_without_reionisation(rsa_problem):
    """rsa2_MD_with_reio adds collision terms of order tau_c (perturbations2.c:9929-9953,
    10064-10084); the synthetic cosmology has no reionisation, so once photons
    free-stream they change the sources by far less than the integration error."""
    p = rsa_problem
    md, _ = _run(p, radiation_streaming_approximation=capi.SONG2_RSA_MD)
    reio, _ = _run(p, radiation_streaming_approximation=capi.SONG2_RSA_MD_WITH_REIO)
    assert 0 < np.max(floored_errors(reio, md, p)) < 1e-6


def test_rsa_options_are_checked(rsa_problem):
    p = rsa_problem
    with pytest.raises(RuntimeError, match="none, MD or MD_with_reio"):
        _run(p, radiation_streaming_approximation=3)
    t = p.tables
    old = t.tau_free_streaming
    t.tau_free_streaming = 0.0
    try:
        with pytest.raises(RuntimeError, match="tau_free_streaming"):
            _run(p, radiation_streaming_approximation=capi.SONG2_RSA_MD)
    finally:
        t.tau_free_streaming = old


def test_rsa_vector_drops_massless_hierarchies(olib, rsa_problem):
    """In RSA the evolved vector holds matter and metric only (perturbations2.c:6778-6796)."""
    p = rsa_problem
    spec = capi.Spec.from_buffer_copy(p.spec)
    spec.radiation_streaming_approximation = capi.SONG2_RSA_MD
    y = np.zeros(4096)
    dy = np.zeros(4096)
    n_full = olib.song2_oracle_rhs(C.byref(spec), C.byref(p.tables), 2, 1, 0, 0, 1000.0, capi.dptr(y), capi.dptr(dy),
                                   capi.errbuf())
    n_rsa = olib.song2_oracle_rhs(C.byref(spec), C.byref(p.tables), 2, 1, 0, 2, 1000.0, capi.dptr(y), capi.dptr(dy),
                                  capi.errbuf())
    # baryons and CDM: (0,0,0) and (1,1,m) for m <= 1 in the list; metric phi, phi', omega, gamma, gamma'
    assert n_rsa == 2 * 3 + 5
    assert n_full > n_rsa


def test_free_streaming_time_edges(lib, rsa_problem):
    """A trigger never reached gives tau0; one met from the first node gives the
    start of the table."""
    t = rsa_problem.tables
    assert lib.song2_free_streaming_time(C.byref(t), 1e30) == t.tau0
    assert abs(lib.song2_free_streaming_time(C.byref(t), 1e-30) - np.exp(t.bg_lntau0)) < 1e-12 * np.exp(t.bg_lntau0)


def test_rsa_dipole_enters_the_baryon_equation(olib, rsa_problem):
    """With the quadratic sources off, the RSA photon dipole is I_10 = 4*3/k (phi' + psi')
    with psi' = phi' (perturbations2.c:10033-10090); the baryon dipole equation in
    the RSA vector must then equal the full-vector one evaluated with that I_10
    (perturbations2.c:8802-8804: C_1m from the RSA dipole)."""
    p = rsa_problem
    spec = capi.Spec.from_buffer_copy(p.spec)
    spec.radiation_streaming_approximation = capi.SONG2_RSA_MD
    spec.has_quadratic_sources = 0
    i1, i2, i3 = 2, 1, 0
    k = p.triplet_k(i1, i2, i3)[2]
    err = capi.errbuf()
    y = np.zeros(4096)
    dy = np.zeros(4096)
    n_rsa = olib.song2_oracle_rhs(C.byref(spec), C.byref(p.tables), i1, i2, i3, 2, 3000.0, capi.dptr(y), capi.dptr(dy), err)
    n_full = olib.song2_oracle_rhs(C.byref(spec), C.byref(p.tables), i1, i2, i3, 0, 3000.0, capi.dptr(y), capi.dptr(dy), err)
    assert n_rsa == 11 and n_full > n_rsa
    rng = np.random.default_rng(7)
    tail = rng.normal(size=11)          # b000 b110 b111 c000 c110 c111 phi phi' omega gamma gamma'
    y_rsa = np.zeros(4096)
    y_rsa[:11] = tail
    y_full = np.zeros(4096)
    y_full[n_full - 11:n_full] = tail
    y_full[1] = 24 * tail[7] / k        # I(1,0): lm(1,0) = 1 in the photon block at the start of the vector
    d_rsa = np.zeros(4096)
    d_full = np.zeros(4096)
    olib.song2_oracle_rhs(C.byref(spec), C.byref(p.tables), i1, i2, i3, 2, 3000.0, capi.dptr(y_rsa), capi.dptr(d_rsa), err)
    olib.song2_oracle_rhs(C.byref(spec), C.byref(p.tables), i1, i2, i3, 0, 3000.0, capi.dptr(y_full), capi.dptr(d_full), err)
    for j in (1, 2):                    # b110, b111 (I(1,1) = 0 in both)
        assert abs(d_rsa[j] - d_full[n_full - 11 + j]) <= 1e-12 * max(abs(d_rsa[j]), 1e-30), j
