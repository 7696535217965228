"""The reader of the reference's ini/pre parameter files (input2.c) for the keys
of the hot path.  The files are written by the tests; names, aliases, yes/no
rules and defaults follow input2.c:137-2016 and perturbations2.c:843-945.  CPU only."""
import ctypes as C

import pytest

from song_gb300 import capi

INI = """
# second-order run: temperature and E-mode bispectra
output = tBisp, eBisp
modes_song = 0, 1, 2
l_max_g_song = 10
l_max_pol_g_song = 9
l_max_ur_song = 8
tol_perturb_integration_song = 1e-5
ic_song = ad
include_pure_scattering_song = yes
include_quad_scattering_song = yes
include_sachs_wolfe_song = yes
include_integrated_sachs_wolfe_song = yes
include_pure_metric_song = yes          # dropped because SW and ISW are on
use_exponential_potentials = yes
sources2_k_sampling = log
k_min_custom_song = 1e-4
k_max_custom_song = 0.05
k_size_custom_song = 8
sources2_k3_sampling = lin
k3_size = 6
custom_time_sampling_song_sources = yes
custom_tau_ini_song_sources = 200
custom_tau_end_song_sources = 0
custom_tau_size_song_sources = 100
custom_tau_mode_song_sources = log
"""

PRE = """
radiation_streaming_approximation_song = 0
tight_coupling_trigger_tau_c_over_tau_h_song = 0.015
tight_coupling_trigger_tau_c_over_tau_k_2nd_order = 0.005
l_max_scalars = 2000
l_logstep = 1.25
l_linstep = 36
transfer2_k3_sampling = smart
q_linstep_song = 0.3
transfer2_tau_sampling = custom
tau_linstep_song = 0.5
bessels_interpolation = linear
sources_time_interpolation = cubic
bispectra_k3_extrapolation = flat_extrapolation
extra_k3_oscillations_right = 20
extra_k3_oscillations_left = 10
"""


def read(lib, tmp_path, ini, pre, los=True):
    pi, pp = tmp_path / "run.ini", tmp_path / "run.pre"
    pi.write_text(ini)
    pp.write_text(pre)
    s, g = capi.Spec(), capi.Params()
    ls = capi.LosSpec() if los else None
    err = capi.errbuf()
    rc = lib.song2_read_params(str(pi).encode(), str(pp).encode(), C.byref(s), C.byref(g),
                               C.byref(ls) if ls is not None else None, err)
    return rc, s, g, ls, err.value.decode()


def test_reads_the_hot_path_keys(lib, tmp_path):
    rc, s, g, ls, err = read(lib, tmp_path, INI, PRE)
    assert rc == 0, err
    assert (s.has_source_T, s.has_source_E, s.has_source_B, s.has_source_delta_cdm) == (1, 1, 1, 0)
    assert [s.m[i] for i in range(s.m_size)] == [0, 1, 2]
    assert (s.l_max_g, s.l_max_pol_g, s.l_max_ur) == (10, 9, 8)
    assert s.rtol == 1e-5 and s.ic == 0
    assert s.has_pure_scattering_in_los and s.has_quad_scattering_in_los and s.has_sw and s.has_isw
    assert s.has_pure_metric_in_los == 0 and s.use_exponential_potentials == 1
    assert s.rescale_cmb_sources == 1          # m_max > 0 and no stop_at_* output
    assert s.radiation_streaming_approximation == 0
    assert s.tca_trigger_tau_c_over_tau_h == 0.015 and s.tca_trigger_tau_c_over_tau_k == 0.005
    assert (g.k_sampling, g.k_min, g.k_max, g.k_size) == (capi.SAMPLING_LOG, 1e-4, 0.05, 8)
    assert (g.k3_sampling, g.k3_size) == (capi.SAMPLING_LIN, 6)
    assert (g.custom_tau, g.tau_sampling, g.tau_ini, g.tau_end, g.tau_size) == (1, capi.SAMPLING_LOG, 200, 0, 100)
    assert (g.l_max_scalars, g.l_logstep, g.l_linstep) == (2000, 1.25, 36)
    assert ls.k3_sampling == capi.K3_SAMPLING_CLASS and ls.q_linstep == 0.3
    assert ls.tau_sampling == capi.TAU_SAMPLING_CUSTOM and ls.tau_linstep == 0.5
    assert ls.time_interpolation == capi.INTERP_CUBIC and ls.bessel_interpolation == capi.INTERP_LINEAR
    assert ls.k3_extrapolation == capi.K3_EXTRAP_FLAT
    assert (ls.extra_k3_oscillations_left, ls.extra_k3_oscillations_right) == (10, 20)
    assert abs(ls.x_max - (0.05 * 18000 + 0.2) * 1.05) < 1e-9


def test_defaults_are_the_reference_defaults(lib, tmp_path):
    rc, s, g, ls, err = read(lib, tmp_path, "output = tBisp\n", "")
    assert rc == 0, err
    ref = capi.Spec()
    lib.song2_spec_defaults(C.byref(ref))
    for f in ("l_max_g", "l_max_pol_g", "l_max_ur", "rtol", "tight_coupling", "has_quadratic_sources",
              "has_polarization2", "start_small_k_at_tau_c_over_tau_h"):
        assert getattr(s, f) == getattr(ref, f), f
    assert s.radiation_streaming_approximation == capi.SONG2_RSA_MD     # rsa2_MD, input2.c:2139
    assert (s.has_source_T, s.has_source_E, s.has_source_B) == (1, 0, 0)
    assert g.k_sampling == capi.SAMPLING_SMART and g.k3_sampling == capi.SAMPLING_SMART
    assert g.custom_tau == 0 and g.tau_size == 2000


def test_switches_and_outputs(lib, tmp_path):
    rc, s, *_ , err = read(lib, tmp_path, "output = bBisp, mBisp\nmodes_song = 0\nquadratic_sources = no\n", "")
    assert rc == 0, err
    # B output needs E sources; B sources vanish for m = 0 only runs
    assert (s.has_source_T, s.has_source_E, s.has_source_B, s.has_source_delta_cdm) == (0, 1, 0, 1)
    assert s.has_quadratic_sources == 0 and s.has_quadratic_liouville == 0 and s.has_quadratic_collision == 0
    assert s.rescale_cmb_sources == 0
    rc, s, *_ , err = read(lib, tmp_path, "output = tCl2, T2\nmodes_song = 0,2\n", "")
    assert rc == 0 and s.rescale_cmb_sources == 0          # stop_at_transfers2
    rc, s, *_ , err = read(lib, tmp_path, "ic_song = ad_first_order\n", "")
    assert rc == 0 and s.ic == capi.SONG2_IC_AD_FIRST_ORDER


def test_obsolete_alias_loses_to_the_new_name(lib, tmp_path):
    rc, s, *_ , err = read(lib, tmp_path, "l_max_g_2nd_order = 5\nl_max_g_song = 7\nl_max_ur_2nd_order = 6\n", "")
    assert rc == 0, err
    assert s.l_max_g == 7 and s.l_max_ur == 6


@pytest.mark.parametrize("ini,pre,msg", [
    ("l_max_g_song = 8\n", "l_max_g_song = 9\n", "multiple entries"),
    ("modes_song = 2, 1\n", "", "strictly ascending"),
    ("output = eBisp\npolarization_second_order = no\n", "", "polarization_second_order"),
    ("sources2_k_sampling = spiral\n", "", "sampling"),
    ("perfect_baryons = no\n", "", "perfect_baryons"),
    ("tol_perturb_integration_song = small\n", "", "not a number"),
    ("custom_time_sampling_song_sources = yes\ncustom_tau_ini_song_sources = 0\n", "", "tau_ini"),
])
def test_bad_files_are_errors(lib, tmp_path, ini, pre, msg):
    rc, *_ , err = read(lib, tmp_path, ini, pre)
    assert rc == 1 and msg in err, err


def test_missing_file_is_an_error(lib, tmp_path):
    s, g = capi.Spec(), capi.Params()
    err = capi.errbuf()
    assert lib.song2_read_params(str(tmp_path / "none.ini").encode(), None, C.byref(s), C.byref(g), None, err) == 1
    assert b"cannot open" in err.value


# ------------------------------------------------------------ smart samplings

def oracle_lib():
    import numpy as np  # noqa: F401
    import oracle
    lib = oracle.load()
    f = lib.song2_oracle_k_grid_smart
    f.restype = C.c_int
    f.argtypes = [C.c_double] * 11 + [C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, C.POINTER(C.c_double),
                                      C.c_int]
    g = lib.song2_oracle_k3_grids_smart
    g.restype = C.c_int
    g.argtypes = [C.POINTER(C.c_double), C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double)]
    h = lib.song2_oracle_sound_horizon
    h.restype = C.c_double
    h.argtypes = [C.POINTER(capi.Tables), C.c_double]
    return lib


def smart_k(lib, g, tau0, rs_rec, l_max):
    import numpy as np
    err = capi.errbuf()
    n = lib.song2_k_grid_smart(C.byref(g), tau0, rs_rec, l_max, None, err)
    assert n > 0, err.value
    k = np.zeros(n)
    assert lib.song2_k_grid_smart(C.byref(g), tau0, rs_rec, l_max, capi.dptr(k), err) == n
    return k


@pytest.mark.parametrize("cmb,lss,l_max", [(1, 0, 2000), (1, 1, 400), (0, 1, 2000)])
def test_smart_k_grid_matches_oracle(lib, cmb, lss, l_max):
    import numpy as np
    g = capi.Params()
    lib.song2_params_defaults(C.byref(g))
    g.has_cmb, g.has_lss, g.k_max_for_pk = cmb, lss, 1.0
    tau0, rs_rec = 14162.7, 145.3
    k = smart_k(lib, g, tau0, rs_rec, l_max)
    ol = oracle_lib()
    out = np.zeros(100000)
    n = ol.song2_oracle_k_grid_smart(g.k_min_tau0, g.k_max_tau0_over_l_max, g.k_step_sub, g.k_step_super,
                                     g.k_logstep_super, g.k_step_transition, g.k_per_decade_for_pk,
                                     g.k_per_decade_for_bao, g.k_bao_center, g.k_bao_width, g.k_max_for_pk,
                                     cmb, lss, tau0, rs_rec, l_max, capi.dptr(out), out.size)
    assert np.array_equal(k, out[:n])
    assert k[0] == g.k_min_tau0 / tau0 and np.all(np.diff(k) > 0)
    assert k[-1] == max(cmb * g.k_max_tau0_over_l_max * l_max / tau0, lss * 1.0)


def test_smart_k3_grids_match_oracle(lib):
    import numpy as np
    g = capi.Params()
    lib.song2_params_defaults(C.byref(g))
    g.has_cmb = 1
    k = smart_k(lib, g, 14162.7, 145.3, 600)
    n = len(k)
    sz = np.zeros(n * n, dtype=np.int32)
    err = capi.errbuf()
    assert lib.song2_k3_grids_smart(capi.dptr(k), n, g.k3_size_min, capi.iptr(sz), None, err) == 0, err.value
    k3 = np.zeros(int(sz.sum()))
    assert lib.song2_k3_grids_smart(capi.dptr(k), n, g.k3_size_min, capi.iptr(sz), capi.dptr(k3), err) == 0
    ol = oracle_lib()
    osz = np.zeros(n * (n + 1) // 2, dtype=np.int32)
    ok3 = np.zeros(k3.size)
    assert ol.song2_oracle_k3_grids_smart(capi.dptr(k), n, g.k3_size_min, capi.iptr(osz), capi.dptr(ok3)) == 0
    pair_sizes = [int(sz[i1 * n + i2]) for i1 in range(n) for i2 in range(i1 + 1)]
    assert pair_sizes == list(osz) and np.array_equal(k3, ok3)
    off = 0
    for i1 in range(n):
        for i2 in range(i1 + 1):
            grid = k3[off: off + sz[i1 * n + i2]]
            off += sz[i1 * n + i2]
            assert np.all(np.diff(grid) > 0)
            assert grid[0] >= abs(k[i1] - k[i2]) and grid[-1] <= k[i1] + k[i2] and grid[-1] <= k[-1]


def test_sound_horizon_matches_oracle(lib):
    from helpers import problem
    p = problem()
    tr = lib.song2_recombination_time(C.byref(p.tables))
    rs = lib.song2_sound_horizon(C.byref(p.tables), tr)
    ref = oracle_lib().song2_oracle_sound_horizon(C.byref(p.tables), tr)
    assert abs(rs - ref) <= 1e-6 * ref
    assert 130.0 < rs < 160.0      # the comoving sound horizon of this flat LCDM at the visibility peak


def test_reader_grids_of_a_smart_preset(lib, tmp_path):
    import numpy as np
    rc, s, g, ls, err = read(lib, tmp_path, "output = tBisp, eBisp\nmodes_song = 0,1,2\n",
                             "sources2_k_sampling = smart\nsources2_k3_sampling = smart\nk3_size_min = 7\n"
                             "l_max_scalars = 500\nk_min_tau0_song = 0.05\n")
    assert rc == 0, err
    assert g.k_sampling == capi.SAMPLING_SMART and g.k3_sampling == capi.SAMPLING_SMART and g.has_cmb == 1
    assert g.k3_size_min == 7 and g.k_min_tau0 == 0.05 and g.l_max_scalars == 500
    k = smart_k(lib, g, 14162.7, 145.3, g.l_max_scalars)
    n = len(k)
    sz = np.zeros(n * n, dtype=np.int32)
    errb = capi.errbuf()
    assert lib.song2_k3_grids_smart(capi.dptr(k), n, g.k3_size_min, capi.iptr(sz), None, errb) == 0
    assert min(int(sz[i1 * n + i2]) for i1 in range(n) for i2 in range(i1 + 1)) >= 2


# ------------------------------------------------------- source time sampling

def tau_grid(lib, p, step, boost, start, cmb):
    import numpy as np
    err = capi.errbuf()
    n = lib.song2_tau_grid_class(C.byref(p.tables), step, boost, start, 1e-10, cmb, None, err)
    assert n > 0, err.value
    out = np.zeros(n)
    assert lib.song2_tau_grid_class(C.byref(p.tables), step, boost, start, 1e-10, cmb, capi.dptr(out), err) == n
    return out


def oracle_tau(p, step, boost, start, cmb):
    import numpy as np
    ol = oracle_lib()
    f = ol.song2_oracle_tau_grid_class
    f.restype = C.c_int
    f.argtypes = [C.POINTER(capi.Tables), C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int,
                  C.POINTER(C.c_double)]
    r = ol.song2_oracle_thermo_rates
    r.restype = None
    r.argtypes = [C.POINTER(capi.Tables), C.c_double, C.POINTER(C.c_double)]
    out = np.zeros(1000000)
    n = f(C.byref(p.tables), step, boost, start, 1e-10, cmb, out.size, capi.dptr(out))
    assert n > 0

    def rates(tau):
        v = np.zeros(4)
        r(C.byref(p.tables), tau, capi.dptr(v))
        return v
    return out[:n], rates


@pytest.mark.parametrize("step,boost,start", [(0.4, 1.0, 0.008), (0.4, 16.0, 0.01), (1.5, 4.0, 0.02)])
def test_source_time_grid_matches_oracle(lib, step, boost, start):
    import numpy as np
    from helpers import problem
    p = problem()
    tau = tau_grid(lib, p, step, boost, start, 1)
    ref, rates = oracle_tau(p, step, boost, start, 1)
    assert tau.size == ref.size
    assert np.allclose(tau, ref, rtol=1e-10, atol=0)
    assert np.all(np.diff(tau) > 0) and tau[-1] == p.tables.tau0
    kd, _, aH, _ = rates(tau[0])
    assert abs(aH / kd - start) < 1e-6 * start              # the bisection's root
    # each step is stepsize / sqrt(rate^2 + boost^2 |2 a''/a - (aH)^2|) at the point before it
    for i in range(0, tau.size - 2, max(1, tau.size // 50)):
        _, rate, aH, app = rates(tau[i])
        want = step / np.sqrt(rate ** 2 + boost ** 2 * abs(2 * app - aH ** 2))
        assert abs((tau[i + 1] - tau[i]) - want) <= 1e-9 * want
    # a later start and a larger boost give more points
    assert tau.size > 20


def test_source_time_grid_without_cmb(lib):
    import numpy as np
    from helpers import problem
    p = problem()
    tau = tau_grid(lib, p, 0.4, 1.0, 0.008, 0)
    ref, rates = oracle_tau(p, 0.4, 1.0, 0.008, 0)
    # the grid starts at the visibility peak, whose location a maximum search
    # fixes only to about sqrt(machine epsilon)
    assert tau.size == ref.size and np.allclose(tau, ref, rtol=1e-7, atol=0)
    tr = lib.song2_recombination_time(C.byref(p.tables))
    assert tau[0] == tr
    # steps of stepsize / (aH): roughly logarithmic in tau
    _, _, aH, _ = rates(tau[3])
    assert abs((tau[4] - tau[3]) - 0.4 / aH) <= 1e-12 * tau[4]


def test_source_time_grid_errors(lib):
    from helpers import problem
    p = problem()
    err = capi.errbuf()
    # a start after recombination: tau_c / tau_h at the visibility peak is far below 10
    assert lib.song2_tau_grid_class(C.byref(p.tables), 0.4, 1.0, 10.0, 1e-10, 1, None, err) == -1
    assert b"after recombination" in err.value
    assert lib.song2_tau_grid_class(C.byref(p.tables), 0.4, 1.0, 1e-9, 1e-10, 1, None, err) == -1
    assert b"thermodynamics table" in err.value


def test_reader_source_time_sampling_keys(lib, tmp_path):
    rc, s, g, ls, err = read(lib, tmp_path, "output = tBisp\n",
                             "start_sources_at_tau_c_over_tau_h = 0.01\nperturb_sampling_stepsize_song = 0.3\n"
                             "perturb_sampling_late_time_boost = 16\n")
    assert rc == 0, err
    assert (g.tau_start_c_over_h, g.tau_stepsize, g.tau_late_boost) == (0.01, 0.3, 16.0)
    rc, s, g, ls, err = read(lib, tmp_path, "output = tBisp\n", "perturb_sampling_stepsize_for_2nd_order = 0.2\n")
    assert rc == 0, err
    assert (g.tau_start_c_over_h, g.tau_stepsize, g.tau_late_boost) == (0.008, 0.2, 1.0)
    rc, *_, err = read(lib, tmp_path, "output = tBisp\n", "perturb_sampling_stepsize_song = 0\n")
    assert rc == 1 and "positive" in err


def test_theta12_k3_grids_match_oracle(lib):
    import numpy as np
    k = np.geomspace(1e-4, 0.2, 12)
    n = len(k)
    sz = np.zeros(n * n, dtype=np.int32)
    err = capi.errbuf()
    assert lib.song2_k3_grids_theta12(capi.dptr(k), n, 9, capi.iptr(sz), None, err) == 0, err.value
    k3 = np.zeros(int(sz.sum()))
    assert lib.song2_k3_grids_theta12(capi.dptr(k), n, 9, capi.iptr(sz), capi.dptr(k3), err) == 0
    ol = oracle_lib()
    f = ol.song2_oracle_k3_grids_theta12
    f.restype = C.c_int
    f.argtypes = [C.POINTER(C.c_double), C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double)]
    osz = np.zeros(n * (n + 1) // 2, dtype=np.int32)
    ok3 = np.zeros(k3.size)
    assert f(capi.dptr(k), n, 9, capi.iptr(osz), capi.dptr(ok3)) == 0
    assert np.allclose(k3, ok3, rtol=1e-14, atol=0)
    off = 0
    for i1 in range(n):
        for i2 in range(i1 + 1):
            g = k3[off: off + 9]
            off += 9
            assert np.all(np.diff(g) > 0)
            lo = max(abs(k[i1] - k[i2]) + 1e-10, (k[i1] + k[i2]) / 100, k[0])
            hi = min(k[i1] + k[i2] - 1e-10, k[-1])
            # the angles are linear: the first and last k3 are the clipped limits
            # (the first moved inwards by a fifth of a step when k1 = k2)
            assert abs(g[-1] - hi) <= 1e-12 * hi
            if i1 != i2:
                assert abs(g[0] - lo) <= 1e-9 * lo
            else:
                assert g[0] > lo
            cos_t = (g ** 2 - k[i1] ** 2 - k[i2] ** 2) / (2 * k[i1] * k[i2])
            th = np.arccos(np.clip(cos_t, -1, 1))
            assert np.allclose(np.diff(th), np.diff(th)[0], rtol=1e-6, atol=1e-12)
    assert lib.song2_k3_grids_theta12(capi.dptr(k), n, 1, capi.iptr(sz), None, err) == 1


def read_cosmo(lib, tmp_path, ini, pre=""):
    pi, pp = tmp_path / "c.ini", tmp_path / "c.pre"
    pi.write_text(ini)
    pp.write_text(pre)
    c = capi.Cosmo()
    err = capi.errbuf()
    rc = lib.song2_read_cosmo(str(pi).encode(), str(pp).encode(), C.byref(c), err)
    return rc, c, err.value.decode()


def test_reader_cosmology_keys(lib, tmp_path):
    rc, c, err = read_cosmo(lib, tmp_path, "output = tBisp\nH0 = 67.0\nOmega_b = 0.05\nomega_cdm = 0.12\n"
                                          "N_ur = 3.04\nT_cmb = 2.725\nYHe = 0.25\n"
                                          "reio_parametrization = reio_camb\nz_reio = 8\n")
    assert rc == 0, err
    assert (c.h, c.omega_cdm, c.N_eff, c.T_cmb, c.YHe, c.z_reio) == (0.67, 0.12, 3.04, 2.725, 0.25, 8.0)
    assert abs(c.omega_b - 0.05 * 0.67 ** 2) < 1e-15
    rc, c, err = read_cosmo(lib, tmp_path, "output = tBisp\n")
    assert rc == 0, err
    assert (c.h, c.omega_b, c.omega_cdm, c.N_eff, c.T_cmb, c.YHe, c.z_reio) == (0.678, 0.0224, 0.12, 3.046, 2.7255,
                                                                               0.24, 0.0)


@pytest.mark.parametrize("ini,msg", [
    ("h = 0.7\nH0 = 70\n", "one of h and H0"),
    ("100*theta_s = 1.04\n", "theta_s"),
    ("N_ncdm = 1\n", "massive neutrinos"),
    ("Omega_k = 0.01\n", "curvature"),
    ("YHe = BBN\n", "BBN"),
    ("reio_parametrization = reio_camb\n", "needs z_reio"),
    ("reio_parametrization = reio_camb\ntau_reio = 0.06\nz_reio = 7\n", "tau_reio"),
    ("omega_b = 0.022\nOmega_b = 0.05\n", "one of omega_b"),
])
def test_reader_cosmology_errors(lib, tmp_path, ini, msg):
    rc, c, err = read_cosmo(lib, tmp_path, ini)
    assert rc == 1 and msg in err


def test_reader_bispectrum_settings(lib, tmp_path):
    rc, s, g, ls, err = read(lib, tmp_path, "output = tBisp\n",
                             "transfers_k1_interpolation = linear\ntransfers_k2_interpolation = cubic\nr_size = 75\n")
    assert rc == 0, err
    assert (g.bi_k1_interpolation, g.bi_k2_interpolation, g.bi_r_size) == (capi.INTERP_LINEAR, capi.INTERP_CUBIC, 75)
    rc, *_, err = read(lib, tmp_path, "output = tBisp\n", "r_size = 1\n")
    assert rc == 1 and "r_size" in err
