"""Physics limits that pin the CPU restatement (the reference ships no golden
vectors and cannot be built here, so these are the checks it documents):

- first-order mode (quadratic_sources = no with has_ad_first_order initial
  conditions, perturbations2.h:270-287) starts from the adiabatic superhorizon
  solution of Ma & Bertschinger (1995) eq. 98;
- with no quadratic sources the m=0 second-order solution depends on k3 only,
  not on k1 and k2 (the same debug mode);
- the second-order result is converged: rtol 1e-6 and 1e-8 runs agree well
  within 1e-4 (the tolerance contract of the benchmark);
- today's second-order CDM density on subhorizon scales is the Newtonian
  2 F2(k1,k2) delta_1 delta_2 (the comparison of test/print_kernel.c:205-216);
- the sources obey S(k2,k1,k3) = (-1)^m S(k1,k2,k3) (perturbations2.h:382-388),
  so odd-m sources vanish when k1 = k2, and B has no m = 0 part.
"""
import numpy as np

import oracle
from song_gb300 import capi
from helpers import floored_errors, problem


def test_first_order_superhorizon_initial_state(lib, olib):
    p = problem()
    fo = oracle.first_order(p, nthreads=4)
    rho_g = np.exp(p.bg[0, capi.BG_LN_RHO_G]); rho_ur = np.exp(p.bg[0, capi.BG_LN_RHO_UR])
    fnu = rho_ur / (rho_g + rho_ur)
    psi = -10.0 / (15.0 + 4.0 * fnu)          # zeta = 1
    first = fo[:, 0, :]
    assert np.allclose(first[:, capi.FO_PSI], psi, rtol=2e-3)
    assert np.allclose(first[:, capi.FO_PHI], (1 + 0.4 * fnu) * psi, rtol=2e-3)
    assert np.allclose(first[:, capi.FO_DELTA_G], -2 * first[:, capi.FO_PSI], rtol=2e-3)
    assert np.allclose(first[:, capi.FO_DELTA_CDM], 0.75 * first[:, capi.FO_DELTA_G], rtol=2e-3)
    assert np.allclose(first[:, capi.FO_DELTA_B], 0.75 * first[:, capi.FO_DELTA_G], rtol=2e-3)
    # matter domination today: delta_cdm grows, phi decays towards the Lambda era
    assert np.all(np.abs(fo[:, -1, capi.FO_DELTA_CDM]) > 10 * np.abs(fo[:, 0, capi.FO_DELTA_CDM]))


def test_first_order_mode_independent_of_k1_k2(lib, olib):
    # second-order code with no quadratic sources: the solution at fixed k3 must not
    # depend on (k1, k2) beyond the tight-coupling switch and start time, which use max(k1,k2,k3)
    p = problem(k_min=0.010, k_max=0.016, k_size=3, k3_size=2, l_max=6, m=(0,), has_quadratic_sources=0,
                ic=capi.SONG2_IC_AD_FIRST_ORDER, primordial_local_fnl_phi=5.0 / 6.0, los="none",
                has_pure_scattering_in_los=1, has_sw=1, has_isw=1, rtol=1e-6, tight_coupling=0, sources="T")
    # overwrite every k3 grid with the same two wavenumbers (triangle-compatible for all pairs)
    p.k3[:] = np.tile([0.011, 0.014], p.k3.size // 2)
    p.set_first_order(np.zeros(p.fo_shape()))
    src, st = oracle.evolve(p, nthreads=4)
    a = src.reshape(p.tp2_size, p.per_type)
    rows = {}
    for (i1, i2, i3) in p.work_order():
        rows.setdefault(i3, []).append(p.triplet_view(a, i1, i2, i3)[0])
    for i3, lst in rows.items():
        ref = lst[0]
        for other in lst[1:]:
            assert np.max(np.abs(other - ref)) / np.max(np.abs(ref)) < 2e-3


def test_convergence_in_rtol(lib, olib):
    p = problem(rtol=1e-6)
    p.set_first_order(oracle.first_order(p, nthreads=4))
    a, _ = oracle.evolve(p, nthreads=4, rtol=1e-6)
    b, _ = oracle.evolve(p, nthreads=4, rtol=1e-8)
    e = floored_errors(a, b, p)
    assert np.max(e) < 1e-4


def test_late_cdm_density_follows_the_f2_kernel(lib, olib):
    """delta_cdm^(2)(tau0) = 2 F2 delta_1 delta_2 with
    F2 = 5/7 + (k1.k2)/2 (1/k1^2 + 1/k2^2) + 2/7 (k1.k2)^2/(k1^2 k2^2); the stored
    source is delta^(2)/2 (perturbations2.c:12778).  Lambda, baryons and the
    relativistic terms keep the ratio within a few per cent at 0.02 <= k <= 0.1."""
    p = problem(k_min=0.02, k_max=0.1, k_size=3, k3_size=3, l_max=6, m=(0,), sources="TD", tau_size=10)
    p.set_first_order(oracle.first_order(p, nthreads=8))
    src, st = oracle.evolve(p, nthreads=8)
    assert np.all(st["status"] == 0)
    tp_d = [i for i, (kind, _, _) in enumerate(p.tp_list()) if kind == "D"][0]
    assert abs(p.tau[-1] / p.fo_tau_grid()[-1] - 1) < 1e-12
    ratios = []
    for (i1, i2, i3) in p.work_order():
        k1, k2, k = p.triplet_k(i1, i2, i3)
        s_d = p.triplet_view(src, i1, i2, i3)[tp_d][-1]
        d1, d2 = p.fo[i1, -1, capi.FO_DELTA_CDM], p.fo[i2, -1, capi.FO_DELTA_CDM]
        kk = (k * k - k1 * k1 - k2 * k2) / 2
        f2 = 5 / 7 + 0.5 * kk * (1 / k1 ** 2 + 1 / k2 ** 2) + 2 / 7 * kk * kk / (k1 ** 2 * k2 ** 2)
        ratios.append(s_d / (f2 * d1 * d2))
    ratios = np.array(ratios)
    assert np.all(np.abs(ratios - 1) < 0.03), ratios


def test_source_symmetries(lib, olib):
    p = problem(sources="TEB", l_max=5)
    p.set_first_order(oracle.first_order(p, nthreads=8))
    src, st = oracle.evolve(p, nthreads=8)
    assert np.all(st["status"] == 0)
    kinds = p.tp_list()
    odd = [i for i, (kind, _, m) in enumerate(kinds) if m % 2 == 1]
    even = [i for i, (kind, _, m) in enumerate(kinds) if m % 2 == 0 and kind != "B"]
    b0 = [i for i, (kind, _, m) in enumerate(kinds) if kind == "B" and m == 0]
    assert odd and even and b0
    n_diag = 0
    for (i1, i2, i3) in p.work_order():
        v = p.triplet_view(src, i1, i2, i3)
        assert not np.any(v[b0])
        if i1 == i2:
            n_diag += 1
            assert np.abs(v[odd]).max() <= 1e-9 * np.abs(v[even]).max()
    assert n_diag > 0
