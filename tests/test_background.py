"""Background and recombination stand-in for CLASS (song2_host.c)."""
import numpy as np

from song_gb300 import capi
from helpers import problem


def test_background_sanity(lib):
    p = problem()
    t = p.tables
    x = t.bg_lntau0 + t.bg_dlntau * np.arange(t.bg_size)
    tau = np.exp(x)
    a = np.exp(p.bg[:, capi.BG_LN_A])
    assert abs(a[-1] - 1.0) < 1e-9
    assert 13000 < p.tau0 < 15000                       # conformal age of the flat LCDM model [Mpc]
    kappa = p.bg[:, capi.BG_KAPPA]
    i = np.argmin(np.abs(kappa - 1.0))
    assert 1000 < 1 / a[i] - 1 < 1200                   # last scattering around z ~ 1090
    assert 250 < tau[i] < 320
    Hc = np.exp(p.bg[:, capi.BG_LN_HC])
    assert np.allclose(Hc[:50] * tau[:50], 1.0, rtol=2e-3)   # radiation era: aH = 1/tau
    assert np.all(np.diff(kappa) <= 0)                  # optical depth decreases with time


def test_start_time_bisection(lib):
    import ctypes as C
    p = problem()
    err = capi.errbuf()
    ti = C.c_double()
    assert lib.song2_start_time(C.byref(p.spec), C.byref(p.tables), 0.1, 200.0, C.byref(ti), err) == 0
    # k/aH = 0.07 at the start for large k: tau_ini ~ 0.7 Mpc in the radiation era
    assert 0.5 < ti.value < 0.8


def test_ionisation_history_with_helium(lib):
    """x_e = n_e / n_H from the tabulated kappa' = a n_e sigma_T (n_H scales as
    a^-3): the plateaux of fully ionised helium (1 + 2 f_He), singly ionised
    helium (1 + f_He) and neutral helium with ionised hydrogen (1), f_He =
    Y_He / (3.9715 (1 - Y_He)) for Y_He = 0.24, then hydrogen recombination."""
    p = problem()
    a = np.exp(p.bg[:, capi.BG_LN_A])
    z = 1 / a - 1
    xr = np.exp(p.bg[:, capi.BG_LN_KAPPA_DOT]) * a * a   # proportional to x_e
    f_he = 0.24 / (3.9715 * 0.76)

    def xe_at(zz):
        return np.interp(zz, z[::-1], xr[::-1])
    norm = xe_at(9500.0) / (1 + 2 * f_he)                # z = 9500: everything ionised
    assert abs(xe_at(3500.0) / norm - (1 + f_he)) < 2e-3 * (1 + f_he)
    assert abs(xe_at(1800.0) / norm - 1.0) < 5e-3
    assert xe_at(800.0) / norm < 0.01


def test_reionisation_optical_depth(lib):
    """z_reio = 7.7 (CLASS's reio_camb): x_e = 1 + 2 f_He today, 1 + f_He at
    z = 5, the recombination value at z = 30, and an optical depth to z = 30 of
    about 0.055 (Planck's tau_reio for that redshift); z_reio = 0 leaves the
    history untouched."""
    from song_gb300.problem import DEFAULT_COSMO
    base = problem()
    cosmo = dict(DEFAULT_COSMO, z_reio=7.7)
    p = problem(cosmo=cosmo)
    a = np.exp(p.bg[:, capi.BG_LN_A])
    z = 1 / a - 1
    xr = np.exp(p.bg[:, capi.BG_LN_KAPPA_DOT]) * a * a
    xr0 = np.exp(base.bg[:, capi.BG_LN_KAPPA_DOT]) * a * a
    f_he = 0.24 / (3.9715 * 0.76)
    norm = np.interp(9500.0, z[::-1], xr0[::-1]) / (1 + 2 * f_he)

    def at(arr, zz):
        return np.interp(zz, z[::-1], arr[::-1]) / norm
    assert abs(at(xr, 0.0) - (1 + 2 * f_he)) < 1e-3
    assert abs(at(xr, 5.0) - (1 + f_he)) < 5e-3
    assert abs(at(xr, 30.0) - at(xr0, 30.0)) < 1e-6
    i30 = np.argmin(np.abs(z - 30.0))
    tau_reio = p.bg[i30, capi.BG_KAPPA] - base.bg[i30, capi.BG_KAPPA]
    assert 0.045 < tau_reio < 0.065, tau_reio
    assert np.array_equal(problem().bg, base.bg)
