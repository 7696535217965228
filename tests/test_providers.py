"""The table providers: the adapter that fills song2_tables from the caller's own
first-order and background modules (CLASS's perturb_song_sources_at_tau_and_k,
background_at_tau and thermodynamics_at_z in the reference,
perturbations2.c:9133-9163, 10727-10762).

The project's own tables stand in for CLASS: a callback serves them in a
different (reversed) column order, as a provider with its own index_qs_* layout
would, and the filled tables must reproduce them exactly, with the same spline
coefficients.  CPU only."""
import ctypes as C

import numpy as np

import oracle
from song_gb300 import capi
from helpers import problem


def test_first_order_provider_reproduces_the_table(lib):
    p = problem()
    p.set_first_order(oracle.first_order(p, nthreads=4))
    nk, nt, nq = p.fo.shape
    perm = np.arange(nq)[::-1].copy()          # provider order: reversed
    extra = 3                                  # the provider also carries quantities the run does not use
    n_provided = nq + extra

    def serve(user, index_k, k, tau, out):
        assert abs(k - p.k[index_k]) <= 1e-15 * k
        j = int(round((np.log(tau) - p.fo_lntau0) / p.fo_dlntau))
        row = np.full(n_provided, 7.0)
        row[perm] = p.fo[index_k, j]
        for q in range(n_provided):
            out[q] = row[q]
        return 0

    cb = capi.FO_PROVIDER(serve)
    qs_map = np.ascontiguousarray(perm, dtype=np.int32)      # song2 quantity q sits at perm[q]
    fo = np.zeros_like(p.fo)
    dd = np.zeros_like(p.fo)
    tab = capi.Tables.from_buffer_copy(p.tables)
    err = capi.errbuf()
    rc = lib.song2_first_order_from_provider(C.byref(p.spec), p.fo_l_max, nt, p.fo_lntau0, p.fo_dlntau,
                                             C.cast(cb, C.c_void_p), None, n_provided, capi.iptr(qs_map),
                                             capi.dptr(fo), capi.dptr(dd), C.byref(tab), err)
    assert rc == 0, err.value
    assert np.array_equal(fo, p.fo)
    assert np.allclose(dd, p.fo_dd, rtol=0, atol=1e-12 * np.max(np.abs(p.fo_dd)))
    assert tab.fo_size == nq and tab.fo_tau_size == nt and tab.fo_k_size == nk
    # an unused quantity maps to -1 and is stored as zero
    qs_map[0] = -1
    rc = lib.song2_first_order_from_provider(C.byref(p.spec), p.fo_l_max, nt, p.fo_lntau0, p.fo_dlntau,
                                             C.cast(cb, C.c_void_p), None, n_provided, capi.iptr(qs_map),
                                             capi.dptr(fo), capi.dptr(dd), C.byref(tab), err)
    assert rc == 0 and np.all(fo[:, :, 0] == 0.0)
    # a map beyond the provided quantities is an error
    qs_map[1] = n_provided
    assert lib.song2_first_order_from_provider(C.byref(p.spec), p.fo_l_max, nt, p.fo_lntau0, p.fo_dlntau,
                                               C.cast(cb, C.c_void_p), None, n_provided, capi.iptr(qs_map),
                                               capi.dptr(fo), capi.dptr(dd), C.byref(tab), err) == 1


def test_background_provider_reproduces_the_table(lib):
    p = problem()
    t = p.tables
    n = t.bg_size

    def serve(user, tau, cols):
        j = int(round((np.log(tau) - t.bg_lntau0) / t.bg_dlntau))
        for q in range(capi.BG_SIZE):
            cols[q] = p.bg[j, q]
        return 0

    cb = capi.BG_PROVIDER(serve)
    bg = np.zeros_like(p.bg)
    dd = np.zeros_like(p.bg)
    tab = capi.Tables()
    err = capi.errbuf()
    rc = lib.song2_background_from_provider(n, t.bg_lntau0, t.bg_dlntau, C.cast(cb, C.c_void_p), None,
                                            capi.dptr(bg), capi.dptr(dd), C.byref(tab), err)
    assert rc == 0, err.value
    assert np.array_equal(bg, p.bg)
    assert np.allclose(dd, p.bg_dd, rtol=0, atol=1e-12 * np.max(np.abs(p.bg_dd)))
    assert tab.bg_size == n

    def fail(user, tau, cols):
        return 1

    cbf = capi.BG_PROVIDER(fail)
    assert lib.song2_background_from_provider(n, t.bg_lntau0, t.bg_dlntau, C.cast(cbf, C.c_void_p), None,
                                              capi.dptr(bg), capi.dptr(dd), C.byref(tab), err) == 1
    assert b"background provider failed" in err.value
