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
        _lib = lib
    return _lib


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
