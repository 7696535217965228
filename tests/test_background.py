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
