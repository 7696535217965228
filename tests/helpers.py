"""Shared helpers of the test suite: problem set-up and GPU runs through the C ABI."""
import ctypes as C

import numpy as np

from song_gb300 import capi
from song_gb300.problem import Problem, source_errors  # noqa: F401

TINY = dict(k_min=1e-3, k_max=0.02, k_size=3, k3_size=2, l_max=4, m=(0, 1, 2), rtol=1e-4, tau_size=10,
            max_steps=60000)


def problem(**kw):
    args = dict(TINY)
    args.update(kw)
    return Problem(**args)


def gpu_run(lib, prob, precision):
    """Flat sources, stats (reference work order) and kernel ms of one GPU run."""
    c = C.c_void_p()
    err = capi.errbuf()
    assert lib.song2_ctx_create(C.byref(prob.spec), C.byref(prob.tables), precision, C.byref(c), err) == 0, err.value
    try:
        assert lib.song2_ctx_run(c, None, err) == 0, err.value
        src = np.zeros(prob.tp2_size * prob.per_type)
        st = (capi.TripletStats * prob.n_triplets)()
        assert lib.song2_ctx_download(c, capi.dptr(src), st, err) == 0, err.value
        ms = lib.song2_ctx_last_kernel_ms(c)
    finally:
        lib.song2_ctx_destroy(c)
    return src, np.frombuffer(st, dtype=capi.STATS_DTYPE).copy(), ms


def nested_slabs(prob):
    """Host slabs in the reference layout sources[tp][k1][k2<=k1][tau*k3_size+k3]
    (ppt2->sources) as a double**** for the drop-in entry, and a function that
    gathers them into a flat buffer."""
    n = len(prob.k)
    keep, bufs = [], []
    tp_level = (C.POINTER(C.POINTER(C.POINTER(C.c_double))) * prob.tp2_size)()
    for tp in range(prob.tp2_size):
        k1_level = (C.POINTER(C.POINTER(C.c_double)) * n)()
        for i1 in range(n):
            k2_level = (C.POINTER(C.c_double) * (i1 + 1))()
            for i2 in range(i1 + 1):
                buf = np.zeros(len(prob.tau) * int(prob.k3_size[i1 * n + i2]))
                bufs.append((tp, i1, i2, buf))
                k2_level[i2] = capi.dptr(buf)
            keep.append(k2_level)
            k1_level[i1] = k2_level
        keep.append(k1_level)
        tp_level[tp] = k1_level

    def gather():
        flat = np.zeros(prob.tp2_size * prob.per_type)
        nested = prob.to_nested(flat)
        for tp, i1, i2, buf in bufs:
            nested[tp][i1][i2][:] = buf
        return flat
    gather.keep = (keep, bufs, tp_level)
    return C.cast(tp_level, C.c_void_p), gather


def floored_errors(test, ref, prob, floor=1e-10):
    """max_tau |S - S_ref| / max_tau |S_ref| per (triplet, source type); the denominator is
    floored at `floor` times the largest source of the triplet, because odd-m sources vanish
    by symmetry when k1 = k2 (perturbations2.c:11036-11041) and are pure round-off there."""
    a = test.reshape(prob.tp2_size, prob.per_type)
    b = ref.reshape(prob.tp2_size, prob.per_type)
    out = []
    for (i1, i2, i3) in prob.work_order():
        ta = prob.triplet_view(a, i1, i2, i3)
        tb = prob.triplet_view(b, i1, i2, i3)
        den = np.max(np.abs(tb), axis=1)
        den = np.maximum(den, floor * max(den.max(), 1e-300))
        out.append(np.max(np.abs(ta - tb), axis=1) / den)
    return np.array(out)


def fo_errors(test, ref):
    """First-order table error per (k, quantity), normalised by max_tau |ref| (floored)."""
    den = np.abs(ref).max(axis=1)
    scale = np.abs(ref).max(axis=(1, 2), keepdims=False)[:, None]
    den = np.maximum(den, 1e-9 * scale)
    return np.abs(test - ref).max(axis=1) / den
