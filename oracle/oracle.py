"""ctypes bindings of the CPU oracle (oracle/song2_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the product package.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libsong2_oracle.so")

_lib = None


def build():
    subprocess.check_call(["make", "-s", "-C", HERE])


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        from song_gb300 import capi
        lib = C.CDLL(LIB)
        lib.song2_oracle_evolve.restype = C.c_int
        lib.song2_oracle_evolve.argtypes = [C.POINTER(capi.Spec), C.POINTER(capi.Tables), C.POINTER(C.c_double),
                                            C.POINTER(capi.TripletStats), C.c_int, C.c_char_p]
        lib.song2_oracle_evolve_range.restype = C.c_int
        lib.song2_oracle_evolve_range.argtypes = [C.POINTER(capi.Spec), C.POINTER(capi.Tables),
                                                  C.POINTER(C.c_double), C.POINTER(capi.TripletStats),
                                                  C.c_int64, C.c_int64, C.c_int, C.c_char_p]
        lib.song2_oracle_evolve_list.restype = C.c_int
        lib.song2_oracle_evolve_list.argtypes = [C.POINTER(capi.Spec), C.POINTER(capi.Tables),
                                                 C.POINTER(C.c_double), C.POINTER(capi.TripletStats),
                                                 C.POINTER(C.c_int64), C.c_int64, C.c_int, C.c_char_p]
        lib.song2_oracle_first_order.restype = C.c_int
        lib.song2_oracle_first_order.argtypes = [C.POINTER(capi.Spec), C.POINTER(capi.Tables), C.c_int, C.c_int,
                                                 C.c_double, C.c_double, C.POINTER(C.c_double), C.c_int,
                                                 C.c_char_p]
        lib.song2_oracle_coupling.restype = C.c_double
        lib.song2_oracle_coupling.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int]
        lib.song2_oracle_delta_tilde_coupling.restype = C.c_double
        lib.song2_oracle_delta_tilde_coupling.argtypes = [C.c_int] * 6
        lib.song2_oracle_rhs.restype = C.c_int
        lib.song2_oracle_rhs.argtypes = [C.POINTER(capi.Spec), C.POINTER(capi.Tables), C.c_int, C.c_int, C.c_int,
                                         C.c_int, C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                         C.c_char_p]
        lib.song2_oracle_geometry_checks.restype = C.c_int
        lib.song2_oracle_geometry_checks.argtypes = [C.POINTER(capi.Spec), C.c_int, C.c_int, C.c_int,
                                                     C.POINTER(C.c_double)]
        # line-of-sight restatement (song2_los_oracle.c)
        LS = C.POINTER(capi.LosSpec)
        lib.song2_oracle_wigner3j.restype = C.c_double
        lib.song2_oracle_wigner3j.argtypes = [C.c_int] * 6
        lib.song2_oracle_bessel_all.restype = None
        lib.song2_oracle_bessel_all.argtypes = [C.c_double, C.c_int, C.POINTER(C.c_double)]
        lib.song2_oracle_l_list.restype = C.c_int
        lib.song2_oracle_l_list.argtypes = [C.c_int, C.c_double, C.c_int, C.POINTER(C.c_int)]
        lib.song2_oracle_transfer_k_grids.restype = C.c_int64
        lib.song2_oracle_transfer_k_grids.argtypes = [C.POINTER(capi.Spec), LS, C.POINTER(C.c_int),
                                                      C.POINTER(C.c_int), C.POINTER(C.c_int),
                                                      C.POINTER(C.c_double), C.c_char_p]
        lib.song2_oracle_los_table_sizes.restype = C.c_int
        lib.song2_oracle_los_table_sizes.argtypes = [C.POINTER(capi.Spec), LS, C.POINTER(C.c_int),
                                                     C.POINTER(C.c_int), C.POINTER(C.c_int)]
        lib.song2_oracle_los_tables.restype = C.c_int
        lib.song2_oracle_los_tables.argtypes = [C.POINTER(capi.Spec), LS, C.POINTER(C.c_int), C.POINTER(C.c_double),
                                                C.POINTER(C.c_double), C.POINTER(C.c_int), C.c_char_p]
        lib.song2_oracle_transfer_pairs.restype = C.c_int
        lib.song2_oracle_transfer_pairs.argtypes = [C.POINTER(capi.Spec), LS, C.POINTER(C.c_double),
                                                    C.POINTER(C.c_double), C.c_int, C.c_int, C.c_int, C.c_char_p]
        lib.song2_oracle_wigner6j.restype = C.c_double
        lib.song2_oracle_wigner6j.argtypes = [C.c_int] * 6
        lib.song2_oracle_bispectra.restype = C.c_int
        lib.song2_oracle_bispectra.argtypes = [C.POINTER(capi.Spec), LS, C.POINTER(capi.BispectraSpec),
                                               C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_char_p]
        lib.song2_oracle_transfer.restype = C.c_int
        lib.song2_oracle_transfer.argtypes = [C.POINTER(capi.Spec), LS, C.POINTER(C.c_double),
                                              C.POINTER(C.c_double), C.c_int, C.c_char_p]
        _lib = lib
    return _lib


def bessel_all(x, lmax):
    """j_l(x) for l = 0..lmax (the oracle's long-double recurrence)."""
    out = np.zeros(lmax + 1)
    load().song2_oracle_bessel_all(float(x), int(lmax), out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


def l_list(l_max, l_logstep, l_linstep):
    out = np.zeros(l_max + 8, dtype=np.int32)
    n = load().song2_oracle_l_list(l_max, l_logstep, l_linstep, out.ctypes.data_as(C.POINTER(C.c_int)))
    return out[:n].copy()


def transfer_k_grids(prob, los):
    """(sizes, physical_start, physical_size, k values) of the transfer k grids."""
    from song_gb300 import capi
    lib = load()
    n_pairs = len(prob.k) * (len(prob.k) + 1) // 2
    sz, ps, pn = (np.zeros(n_pairs, dtype=np.int32) for _ in range(3))
    err = capi.errbuf()
    n = lib.song2_oracle_transfer_k_grids(C.byref(prob.spec), C.byref(los), capi.iptr(sz), capi.iptr(ps),
                                          capi.iptr(pn), None, err)
    if n < 0:
        raise RuntimeError(err.value.decode())
    kk = np.zeros(n)
    lib.song2_oracle_transfer_k_grids(C.byref(prob.spec), C.byref(los), None, None, None, capi.dptr(kk), err)
    return sz, ps, pn, kk


def los_tables(prob, los):
    """(l1 list, j_l1 [n_l1][x], J [rows][x], J x_min [rows]) in the product's full-row layout."""
    from song_gb300 import capi
    lib = load()
    xs, nl1, nr = C.c_int(), C.c_int(), C.c_int()
    if lib.song2_oracle_los_table_sizes(C.byref(prob.spec), C.byref(los), C.byref(xs), C.byref(nl1), C.byref(nr)):
        raise RuntimeError("oracle line-of-sight tables failed")
    l1 = np.zeros(nl1.value, dtype=np.int32)
    jt = np.zeros((nl1.value, xs.value))
    J = np.zeros((nr.value, xs.value))
    xm = np.zeros(nr.value, dtype=np.int32)
    err = capi.errbuf()
    if lib.song2_oracle_los_tables(C.byref(prob.spec), C.byref(los), capi.iptr(l1), capi.dptr(jt), capi.dptr(J),
                                   capi.iptr(xm), err):
        raise RuntimeError(err.value.decode())
    return l1, jt, J, xm


def transfer(prob, los, sources, n_out, nthreads=0, pairs=None):
    """Flat transfer functions [tt][units] of flat sources (of the pairs
    pairs = (lo, hi) only, the rest left zero, when given)."""
    from song_gb300 import capi
    out = np.zeros(n_out)
    err = capi.errbuf()
    src = np.ascontiguousarray(sources, dtype=np.float64)
    lo, hi = pairs if pairs is not None else (0, 1 << 30)
    if load().song2_oracle_transfer_pairs(C.byref(prob.spec), C.byref(los), capi.dptr(src), capi.dptr(out), lo, hi,
                                          nthreads or (os.cpu_count() or 1), err):
        raise RuntimeError(err.value.decode())
    return out


def bispectra(prob, los, bs, transfer2, n_out):
    """Symmetrised intrinsic bispectra [X][Y][Z][conf] of flat second-order transfers."""
    from song_gb300 import capi
    out = np.zeros(n_out)
    err = capi.errbuf()
    t2 = np.ascontiguousarray(transfer2, dtype=np.float64)
    if load().song2_oracle_bispectra(C.byref(prob.spec), C.byref(los), C.byref(bs), capi.dptr(t2), capi.dptr(out),
                                     err):
        raise RuntimeError(err.value.decode())
    return out


def first_order(prob, nthreads=0):
    """First-order table fo[k][tau][q] from the oracle's first-order mode."""
    from song_gb300 import capi
    lib = load()
    fo = np.zeros(prob.fo_shape())
    err = capi.errbuf()
    rc = lib.song2_oracle_first_order(C.byref(prob.spec), C.byref(prob.tables), prob.fo_l_max, prob.fo_tau_size,
                                      prob.fo_lntau0, prob.fo_dlntau, capi.dptr(fo), nthreads, err)
    if rc:
        raise RuntimeError(err.value.decode())
    return fo


def evolve(prob, nthreads=0, first=None, count=None, rtol=None, items=None):
    """Flat sources [tp2][per_type] and per-triplet stats (work order)."""
    from song_gb300 import capi
    lib = load()
    spec = capi.Spec.from_buffer_copy(prob.spec)
    if rtol is not None:
        spec.rtol = rtol
    src = np.zeros(prob.tp2_size * prob.per_type)
    n = prob.n_triplets
    stats = (capi.TripletStats * n)()
    err = capi.errbuf()
    if items is not None:
        items = np.ascontiguousarray(items, dtype=np.int64)
        rc = lib.song2_oracle_evolve_list(C.byref(spec), C.byref(prob.tables), capi.dptr(src), stats,
                                          items.ctypes.data_as(C.POINTER(C.c_int64)), len(items), nthreads, err)
    elif first is None:
        rc = lib.song2_oracle_evolve(C.byref(spec), C.byref(prob.tables), capi.dptr(src), stats, nthreads, err)
    else:
        rc = lib.song2_oracle_evolve_range(C.byref(spec), C.byref(prob.tables), capi.dptr(src), stats, first,
                                           count, nthreads, err)
    st = np.frombuffer(stats, dtype=capi.STATS_DTYPE).copy()
    if rc:
        raise RuntimeError(err.value.decode() + f" statuses={np.unique(st['status'])}")
    return src, st
