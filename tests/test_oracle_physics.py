"""Physics limits that pin the CPU restatement (the reference ships no golden
vectors and cannot be built here, so these are the checks it documents):

- first-order mode (quadratic_sources = no with has_ad_first_order initial
  conditions, perturbations2.h:270-287) starts from the adiabatic superhorizon
  solution of Ma & Bertschinger (1995) eq. 98;
- with no quadratic sources the m=0 second-order solution depends on k3 only,
  not on k1 and k2 (the same debug mode);
- the second-order result is converged: rtol 1e-6 and 1e-8 runs agree well
  within 1e-4 (the tolerance contract of the benchmark).
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
