"""GPU evolver (through the C ABI) against the CPU oracle on identical inputs.

Tolerances: both sides run the same NDF algorithm at the same rtol, so they
agree to round-off until a step-size decision flips; the bound below is the
rtol contract of the run (errors are max_tau|S - S_ref| / max_tau|S_ref| per
source type and triplet, floored at 1e-10 of the triplet's largest source,
see helpers.floored_errors).  The FP32 iteration matrix of the mixed form only
changes the Newton iterates, so the same bound applies."""
import ctypes as C
import os

import numpy as np
import pytest

import oracle
from song_gb300 import capi
from helpers import floored_errors, fo_errors, gpu_run, nested_slabs, problem

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def tiny(lib):
    p = problem()
    p.set_first_order(oracle.first_order(p, nthreads=8))
    ref, st = oracle.evolve(p, nthreads=8)
    return p, ref, st


def test_first_order_mode_matches_oracle(lib, olib):
    p = problem(k_size=4, rtol=1e-5)
    ref = oracle.first_order(p, nthreads=8)
    got = p.first_order_gpu()
    assert np.all(np.isfinite(got))
    assert np.max(fo_errors(got, ref)) < 1e-4


@pytest.mark.parametrize("precision", [capi.SONG2_PREC_FP64, capi.SONG2_PREC_MIXED])
def test_second_order_matches_oracle(lib, tiny, precision):
    p, ref, st_ref = tiny
    src, st, _ = gpu_run(lib, p, precision)
    assert np.all(st["status"] == capi.SONG2_OK)
    assert np.all(st["sources_calls"] == len(p.tau))
    e = floored_errors(src, ref, p)
    assert np.max(e) < 10 * p.spec.rtol, np.max(e)
    # the same algorithm takes the same steps up to a few flipped decisions
    assert np.all(np.abs(st["n_steps"] - st_ref["n_steps"]) <= 0.05 * st_ref["n_steps"] + 5)


def test_against_tight_oracle(lib, tiny):
    """Every source of an rtol=1e-5 GPU run lies within 1e-4 (relative to its
    maximum over time) of the FP64 oracle at rtol=1e-8."""
    p, _, _ = tiny
    tight, _ = oracle.evolve(p, nthreads=8, rtol=1e-8)
    spec = p.spec
    old = spec.rtol
    spec.rtol = 1e-5
    try:
        for precision in (capi.SONG2_PREC_FP64, capi.SONG2_PREC_MIXED):
            src, st, _ = gpu_run(lib, p, precision)
            assert np.max(floored_errors(src, tight, p)) < 1e-4
    finally:
        spec.rtol = old


@pytest.mark.parametrize("kw", [
    dict(m=(0,), has_polarization2=0, sources="T"),
    dict(tight_coupling=0, sources="TEBD", l_max=5),
    dict(l_max=4, m=(0, 2)),
    dict(m=(0, 1, 2, 3, 4), l_max=6, sources="TEB"),
    dict(k_size=2, k3_size=1),
    dict(los="all", sources="TEB"),
    dict(l_max=20, k_size=2, k3_size=2),
])
def test_edge_cases(lib, olib, kw):
    p = problem(**kw)
    p.set_first_order(oracle.first_order(p, nthreads=8))
    ref, _ = oracle.evolve(p, nthreads=8)
    for precision in (capi.SONG2_PREC_FP64, capi.SONG2_PREC_MIXED):
        src, st, _ = gpu_run(lib, p, precision)
        assert np.all(st["status"] == capi.SONG2_OK)
        assert np.max(floored_errors(src, ref, p)) < 10 * p.spec.rtol


def test_closure_limit_is_rejected(lib):
    """l_max_pol = 3 with m = 2 makes the reference's polarisation closure imaginary:
    the C ABI refuses the spec with a message instead of producing NaNs."""
    p = problem(l_max=3, m=(0, 2))
    p.set_first_order(np.zeros(p.fo_shape()))
    c = C.c_void_p()
    err = capi.errbuf()
    assert lib.song2_ctx_create(C.byref(p.spec), C.byref(p.tables), capi.SONG2_PREC_FP64, C.byref(c), err) == 1
    assert b"closure" in err.value


@pytest.mark.parametrize("launch", [(1, 2, 32, 0), (1, 8, 32, 0), (1, 4, 32, 1), (0, 1, 128, 1), (0, 1, 256, 0),
                                    (2, 32, 1, 0), (2, 64, 2, 0), (2, 32, 4, 0), (2, 16, 8, 0), (2, 4, 32, 0)])
def test_launch_configurations_agree(lib, tiny, launch):
    """Every launch configuration the autotuner may pick computes the same numbers
    within the solver tolerance, against the default configuration and against the
    oracle.  The team layouts are separate kernels compiled in separate translation
    units, so their floating-point contractions (fused or separate multiply-adds)
    may differ in the last bits; a CTA team gives the same result in every run."""
    p, ref, _ = tiny
    base, _, _ = gpu_run(lib, p, capi.SONG2_PREC_MIXED)
    L = capi.Launch(*launch)
    c = C.c_void_p()
    err = capi.errbuf()
    assert lib.song2_ctx_create_ex(C.byref(p.spec), C.byref(p.tables), capi.SONG2_PREC_MIXED, C.byref(L), 0, 1,
                                   C.byref(c), err) == 0, err.value
    assert lib.song2_ctx_run(c, None, err) == 0, err.value
    src = np.zeros_like(base)
    st = (capi.TripletStats * p.n_triplets)()
    lib.song2_ctx_download(c, capi.dptr(src), st, err)
    lib.song2_ctx_destroy(c)
    assert np.all(np.frombuffer(st, dtype=capi.STATS_DTYPE)["status"] == capi.SONG2_OK)
    assert np.max(floored_errors(src, base, p)) < 10 * p.spec.rtol
    assert np.max(floored_errors(src, ref, p)) < 10 * p.spec.rtol
    if launch[0] == 0:
        again, _, _ = gpu_run(lib, p, capi.SONG2_PREC_MIXED)
        assert np.array_equal(again, base)


def test_autotune_picks_a_layout_that_runs(lib, tiny):
    """song2_autotune times its candidate launch configurations on a sample of the
    problem and returns the fastest; a context created with it evolves the triplets
    as the default does."""
    p, ref, _ = tiny
    for precision in (capi.SONG2_PREC_FP64, capi.SONG2_PREC_MIXED):
        best = capi.Launch()
        ms = C.c_double()
        err = capi.errbuf()
        assert lib.song2_autotune(C.byref(p.spec), C.byref(p.tables), precision, 8, C.byref(best), C.byref(ms),
                                  err) == 0, err.value
        assert best.warp_team in (0, 1, 2) and ms.value > 0
        c = C.c_void_p()
        assert lib.song2_ctx_create_ex(C.byref(p.spec), C.byref(p.tables), precision, C.byref(best), 0, 1,
                                       C.byref(c), err) == 0, err.value
        assert lib.song2_ctx_run(c, None, err) == 0, err.value
        src = np.zeros_like(ref)
        st = (capi.TripletStats * p.n_triplets)()
        lib.song2_ctx_download(c, capi.dptr(src), st, err)
        lib.song2_ctx_destroy(c)
        assert np.all(np.frombuffer(st, dtype=capi.STATS_DTYPE)["status"] == capi.SONG2_OK)
        assert np.max(floored_errors(src, ref, p)) < 10 * p.spec.rtol


def test_give_up_path_returns_status(lib, tiny):
    """A triplet that breaches its step limit retires with SONG2_E_MAXSTEPS; the
    kernel neither traps nor hangs."""
    p, _, _ = tiny
    spec = capi.Spec.from_buffer_copy(p.spec)
    spec.max_steps = 3
    c = C.c_void_p()
    err = capi.errbuf()
    assert lib.song2_ctx_create(C.byref(spec), C.byref(p.tables), capi.SONG2_PREC_MIXED, C.byref(c), err) == 0
    assert lib.song2_ctx_run(c, None, err) == 0, err.value
    st = (capi.TripletStats * p.n_triplets)()
    lib.song2_ctx_download(c, None, st, err)
    lib.song2_ctx_destroy(c)
    status = np.frombuffer(st, dtype=capi.STATS_DTYPE)["status"]
    assert np.all(status == capi.SONG2_E_MAXSTEPS)


def test_drop_in_entry_fills_nested_slabs(lib, tiny):
    """song2_gpu_evolve writes ppt2->sources[tp][k1][k2][tau*k3_size+k3]."""
    p, ref, _ = tiny
    n = len(p.k)
    keep = []
    tp_level = (C.POINTER(C.POINTER(C.POINTER(C.c_double))) * p.tp2_size)()
    for tp in range(p.tp2_size):
        k1_level = (C.POINTER(C.POINTER(C.c_double)) * n)()
        for i1 in range(n):
            k2_level = (C.POINTER(C.c_double) * (i1 + 1))()
            for i2 in range(i1 + 1):
                buf = np.zeros(len(p.tau) * int(p.k3_size[i1 * n + i2]))
                keep.append((tp, i1, i2, buf))
                k2_level[i2] = capi.dptr(buf)
            keep.append(k2_level)
            k1_level[i1] = k2_level
        keep.append(k1_level)
        tp_level[tp] = k1_level
    st = (capi.TripletStats * p.n_triplets)()
    err = capi.errbuf()
    assert lib.song2_gpu_evolve(C.byref(p.spec), C.byref(p.tables), capi.SONG2_PREC_FP64,
                                C.cast(tp_level, C.c_void_p), st, err) == 0, err.value
    flat = np.zeros_like(ref)
    nested = p.to_nested(flat)
    for item in keep:
        if isinstance(item, tuple):
            tp, i1, i2, buf = item
            nested[tp][i1][i2][:] = buf
    assert np.max(floored_errors(flat, ref, p)) < 10 * p.spec.rtol


def test_drop_in_reruns_failed_triplets(lib, tiny):
    """The drop-in's exit strategy (what_if_ndf15_fails, perturbations2.c:12877-12957):
    with a step budget below what the larger triplets need, their first pass
    retires with SONG2_E_MAXSTEPS and song2_gpu_evolve evolves them again in plain
    FP64 with eight times the budget; the result matches the oracle and the stats
    mark exactly the re-run triplets."""
    p, ref, st_ref = tiny
    attempts = st_ref["n_steps"] + st_ref["n_rejected"]
    budget = int(np.median(attempts))
    assert 8 * budget > 2 * attempts.max()        # the re-run has room
    spec = capi.Spec.from_buffer_copy(p.spec)
    spec.max_steps = budget
    slabs, gather = nested_slabs(p)
    st = (capi.TripletStats * p.n_triplets)()
    err = capi.errbuf()
    assert lib.song2_gpu_evolve(C.byref(spec), C.byref(p.tables), capi.SONG2_PREC_MIXED, slabs, st, err) == 0, \
        err.value
    stats = np.frombuffer(st, dtype=capi.STATS_DTYPE)
    assert np.all(stats["status"] == capi.SONG2_OK)
    retried = stats["retried"] == 1
    assert retried.any() and not retried.all()
    assert np.all(retried[attempts > 1.2 * budget])
    assert np.max(floored_errors(gather(), ref, p)) < 10 * p.spec.rtol
    # a budget the re-run cannot meet either: the call fails and names the triplet
    spec.max_steps = 3
    assert lib.song2_gpu_evolve(C.byref(spec), C.byref(p.tables), capi.SONG2_PREC_MIXED, slabs, st, err) == 1
    assert b"also on its plain-FP64 re-run" in err.value


def test_shards_sum_to_full_run(lib, tiny):
    p, ref, _ = tiny
    total = np.zeros_like(ref)
    for r in range(3):
        c = C.c_void_p()
        err = capi.errbuf()
        assert lib.song2_ctx_create_shard(C.byref(p.spec), C.byref(p.tables), capi.SONG2_PREC_MIXED, r, 3,
                                          C.byref(c), err) == 0, err.value
        assert lib.song2_ctx_run(c, None, err) == 0
        part = np.zeros_like(ref)
        lib.song2_ctx_download(c, capi.dptr(part), None, err)
        lib.song2_ctx_destroy(c)
        total += part
    full, _, _ = gpu_run(lib, p, capi.SONG2_PREC_MIXED)
    assert np.array_equal(total, full)


def test_gpu_matches_golden_fixture(lib):
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden"))
    from make_golden import CASES, GPU_TOL_RTOL
    for name, kw in CASES.items():
        g = np.load(os.path.join(HERE, "golden", name + ".npz"))
        p = problem(**kw)
        p.set_first_order(g["fo"])
        for precision in (capi.SONG2_PREC_FP64, capi.SONG2_PREC_MIXED):
            src, st, _ = gpu_run(lib, p, precision)
            tol = GPU_TOL_RTOL.get(name, 10) * p.spec.rtol
            assert np.max(floored_errors(src, g["sources"], p)) < tol, name


def test_large_blocks_in_global_scratch(lib, olib):
    """l_max = 20 (m blocks of 67-81 rows) with the iteration-matrix factors and the
    structured Jacobian in global scratch instead of shared memory: both forms agree
    with the oracle."""
    p = problem(l_max=20, k_size=2, k3_size=2)
    p.set_first_order(oracle.first_order(p, nthreads=8))
    ref, _ = oracle.evolve(p, nthreads=8)
    for precision in (capi.SONG2_PREC_FP64, capi.SONG2_PREC_MIXED):
        L = capi.Launch(0, 1, 256, 0)
        c = C.c_void_p()
        err = capi.errbuf()
        assert lib.song2_ctx_create_ex(C.byref(p.spec), C.byref(p.tables), precision, C.byref(L), 0, 1, C.byref(c),
                                       err) == 0, err.value
        assert lib.song2_ctx_run(c, None, err) == 0, err.value
        src = np.zeros(p.tp2_size * p.per_type)
        st = (capi.TripletStats * p.n_triplets)()
        lib.song2_ctx_download(c, capi.dptr(src), st, err)
        lib.song2_ctx_destroy(c)
        assert np.all(np.frombuffer(st, dtype=capi.STATS_DTYPE)["status"] == capi.SONG2_OK)
        assert np.max(floored_errors(src, ref, p)) < 10 * p.spec.rtol


def test_graph_replay_matches_direct_run(lib, tiny):
    """song2_ctx_run_graph (captured once, replayed) computes what song2_ctx_run does."""
    p, _, _ = tiny
    c = C.c_void_p()
    err = capi.errbuf()
    assert lib.song2_ctx_create(C.byref(p.spec), C.byref(p.tables), capi.SONG2_PREC_MIXED, C.byref(c), err) == 0
    try:
        out = []
        for run in (lib.song2_ctx_run, lib.song2_ctx_run_graph, lib.song2_ctx_run_graph):
            assert run(c, None, err) == 0, err.value
            src = np.zeros(p.tp2_size * p.per_type)
            lib.song2_ctx_download(c, capi.dptr(src), None, err)
            out.append(src)
    finally:
        lib.song2_ctx_destroy(c)
    assert np.array_equal(out[0], out[1]) and np.array_equal(out[0], out[2])


@pytest.mark.parametrize("kw", [
    dict(sources="TEB", l_max=5, use_delta_tilde_in_los=1, rescale_cmb_sources=1),
    dict(sources="TEB", l_max=6, l_max_los_t=4, l_max_los_p=4, use_delta_tilde_in_los=1,
         l_max_los_quadratic_t=3, l_max_los_quadratic_p=4),
    dict(m=(0,), sources="TE", use_delta_tilde_in_los=1),
    dict(m=(0, 1, 2, 3, 4), l_max=6, sources="TEB", rescale_cmb_sources=1),
])
def test_delta_tilde_and_rescaling_match_oracle(lib, olib, kw):
    """delta-tilde LOS sources (couplings up to |m1|, |m2| = the quadratic cut, past
    the modes the hierarchy evolves) and rescaled rotation coefficients agree with
    the oracle in both precisions."""
    _check_options_against_oracle(lib, kw)


@pytest.mark.parametrize("kw", [
    dict(sources="TEB", l_max=5, radiation_streaming_approximation=1),
    dict(sources="TEB", l_max=5, radiation_streaming_approximation=1, use_delta_tilde_in_los=1, rescale_cmb_sources=1),
    dict(m=(0,), sources="T", has_polarization2=0, radiation_streaming_approximation=1),
    dict(tight_coupling=0, sources="TEBD", l_max=5, radiation_streaming_approximation=1),
    # MD_with_reio with an early switch (free streaming from 300 Mpc, k tau > 10)
    dict(sources="TEB", l_max=5, radiation_streaming_approximation=2, radiation_streaming_trigger_tau_over_tau_k=10,
         rtol=1e-6, tau_free_streaming=300.0),
])
def test_rsa_matches_oracle(lib, olib, kw):
    """The radiation-streaming interval (massless hierarchies frozen, RSA monopoles
    and dipoles) agrees with the oracle's reduced vector in both precisions and in
    the warp and lane-team kernels."""
    _check_options_against_oracle(lib, kw)


def _check_options_against_oracle(lib, kw):
    """GPU runs against the oracle at the same rtol, within 10 rtol or three times
    the oracle's own error (its distance to an rtol/100 run), whichever is larger:
    with the RSA the T monopole source is a difference of large terms, and both
    sides carry that rtol-level error."""
    kw = dict(kw)
    tau_fs = kw.pop("tau_free_streaming", None)
    p = problem(**kw)
    if tau_fs is not None:
        p.tables.tau_free_streaming = tau_fs
    p.set_first_order(oracle.first_order(p, nthreads=8))
    ref, _ = oracle.evolve(p, nthreads=8)
    tight, _ = oracle.evolve(p, nthreads=8, rtol=p.spec.rtol / 100)
    bound = max(10 * p.spec.rtol, 3 * np.max(floored_errors(ref, tight, p)))
    for precision in (capi.SONG2_PREC_FP64, capi.SONG2_PREC_MIXED):
        src, st, _ = gpu_run(lib, p, precision)
        assert np.all(st["status"] == capi.SONG2_OK)
        assert np.max(floored_errors(src, ref, p)) < bound
    # the warp-per-triplet and lane-team kernels carry the same source terms
    for launch in ((1, 4, 32, 0), (2, 16, 8, 0)) if p.spec.l_max_g <= 5 else ():
        L = capi.Launch(*launch)
        c = C.c_void_p()
        err = capi.errbuf()
        assert lib.song2_ctx_create_ex(C.byref(p.spec), C.byref(p.tables), capi.SONG2_PREC_MIXED, C.byref(L), 0, 1,
                                       C.byref(c), err) == 0, err.value
        assert lib.song2_ctx_run(c, None, err) == 0, err.value
        src = np.zeros(p.tp2_size * p.per_type)
        st = (capi.TripletStats * p.n_triplets)()
        lib.song2_ctx_download(c, capi.dptr(src), st, err)
        lib.song2_ctx_destroy(c)
        assert np.all(np.frombuffer(st, dtype=capi.STATS_DTYPE)["status"] == capi.SONG2_OK)
        assert np.max(floored_errors(src, ref, p)) < bound


def test_delta_tilde_excludes_redshift_term(lib):
    """input2.c:742-744: use_delta_tilde_in_los with has_redshift_in_los is refused."""
    p = problem(use_delta_tilde_in_los=1, has_redshift_in_los=1)
    p.set_first_order(np.zeros(p.fo_shape()))
    c = C.c_void_p()
    err = capi.errbuf()
    assert lib.song2_ctx_create(C.byref(p.spec), C.byref(p.tables), capi.SONG2_PREC_FP64, C.byref(c), err) == 1
    assert b"redshift" in err.value
