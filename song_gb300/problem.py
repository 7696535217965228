"""Problem set-up for the second-order evolver: cosmology, grids, tables.

This is the Python side of what SONG's perturb2_init does before its triplet
loop (source/perturbations2.c:82-283): read the hot-path parameters, build the
k1/k2 grid and the per-pair k3 grids (perturb2_get_k_lists, :1573-2530), the
custom source time sampling (perturb2_timesampling_for_sources, :2580-2598),
and obtain the background/thermodynamics and first-order tables that CLASS
would provide.  All arithmetic is done by the C library (song2_host.c); this
module only owns the numpy buffers so the pointers handed to C stay alive.
"""
import ctypes as C
import math

import numpy as np

from . import capi

# Flat LCDM of the benchmark configurations (h, omega_b, omega_cdm, N_eff, T_cmb, YHe)
DEFAULT_COSMO = dict(h=0.678, omega_b=0.0224, omega_cdm=0.120, N_eff=3.046, T_cmb=2.7255, YHe=0.24)

# The five benchmark configurations (sizes, l_max, modes, rtol, tau samples).
CONFIGS = {
    1: dict(name="config1_plain_cpu_runnable", k_min=1e-4, k_max=0.05, k_size=8, k3_size=6, l_max=8,
            m=(0, 1, 2), rtol=1e-3, tau_size=100, sources="TE"),
    2: dict(name="config2_plain_fp64_4.9k", k_min=1e-5, k_max=0.1, k_size=25, k3_size=15, l_max=12,
            m=(0, 1, 2), rtol=1e-4, tau_size=200, sources="TE"),
    3: dict(name="config3_mixed_16.4k", k_min=1e-5, k_max=0.3, k_size=40, k3_size=20, l_max=20,
            m=(0, 1, 2), rtol=1e-4, tau_size=200, sources="TE"),
    4: dict(name="config4_uneven_30k", k_min=1e-5, k_max=0.3, k_size=50, k3_size=24, l_max=40,
            m=(0, 1, 2, 3, 4), rtol=1e-4, tau_size=200, sources="TEB", uneven=dict(seed=20261203)),
    5: dict(name="config5_production_97k", k_min=1e-5, k_max=0.4, k_size=80, k3_size=30, l_max=25,
            m=(0, 1, 2), rtol=1e-5, tau_size=400, sources="TE"),
}

# Uneven batches: l_max = min(L_CAP, L_BASE + ceil(k tau_rec / 2)) with k = max(k1, k2, k3),
# m_max drawn from M_MAX_CHOICES per triplet (pair order).
L_BASE, L_CAP, M_MAX_CHOICES = 8, 40, (0, 2, 4)

TAU_START_SOURCES = 200.0   # Mpc, just before recombination (tau_rec ~ 280 Mpc)


class Problem:
    """Owns the spec, the grids and the tables of one run."""

    def __init__(self, k_min, k_max, k_size, k3_size, l_max, m=(0,), rtol=1e-4, tau_size=50,
                 tau_ini=TAU_START_SOURCES, tau_end=None, sources="TE", cosmo=None, bg_size=6000,
                 k_log=True, k3_log=False, tau_log=False, los="intrinsic", threshold=1e-6,
                 fo_dlntau=0.01, lib=None, uneven=None, **spec_overrides):
        self.lib = lib or capi.load()
        lib = self.lib
        err = capi.errbuf()
        # --- background & thermodynamics (the CLASS stand-in)
        self.cosmo = capi.Cosmo(**(cosmo or DEFAULT_COSMO))
        self.bg = np.zeros((bg_size, capi.BG_SIZE))
        self.bg_dd = np.zeros_like(self.bg)
        lt0, dlt, tau0, aeq = (C.c_double() for _ in range(4))
        if lib.song2_background_compute(C.byref(self.cosmo), bg_size, capi.dptr(self.bg), capi.dptr(self.bg_dd),
                                        C.byref(lt0), C.byref(dlt), C.byref(tau0), C.byref(aeq), err):
            raise RuntimeError(err.value.decode())
        self.tau0 = tau0.value
        # --- spec
        s = capi.Spec()
        lib.song2_spec_defaults(C.byref(s))
        s.l_max_g = s.l_max_pol_g = s.l_max_ur = l_max
        s.m_size = len(m)
        for i, mm in enumerate(m):
            s.m[i] = mm
        s.rtol = rtol
        s.threshold = threshold
        s.has_source_T = int("T" in sources)
        s.has_source_E = int("E" in sources)
        s.has_source_B = int("B" in sources)
        s.has_source_delta_cdm = int("D" in sources)
        if los == "intrinsic":
            # ini/intrinsic.ini: scattering + SW + ISW with exponential potentials
            s.has_pure_scattering_in_los = 1
            s.has_quad_scattering_in_los = 1
            s.has_sw = 1
            s.has_isw = 1
            s.use_exponential_potentials = 1
        elif los == "none":
            pass
        elif los == "all":
            for f in ("has_pure_scattering_in_los", "has_quad_scattering_in_los", "has_pure_metric_in_los",
                      "has_quad_metric_in_los", "has_time_delay_in_los", "has_redshift_in_los",
                      "has_lensing_in_los"):
                setattr(s, f, 1)
        for key, val in spec_overrides.items():
            setattr(s, key, val)
        # --- grids
        self.k = np.zeros(k_size)
        if lib.song2_k_grid(int(k_log), k_min, k_max, k_size, capi.dptr(self.k)):
            raise RuntimeError("bad k grid")
        self.k3_size = np.zeros(k_size * k_size, dtype=np.int32)
        if lib.song2_k3_grids(capi.dptr(self.k), k_size, k3_size, int(k3_log), capi.iptr(self.k3_size), None, err):
            raise RuntimeError(err.value.decode())
        self.k3 = np.zeros(int(self.k3_size.sum()))
        lib.song2_k3_grids(capi.dptr(self.k), k_size, k3_size, int(k3_log), capi.iptr(self.k3_size),
                           capi.dptr(self.k3), err)
        if tau_end is None:
            tau_end = self.tau0
        self.tau = np.zeros(tau_size)
        lib.song2_tau_grid(int(tau_log), tau_ini, tau_end, tau_size, capi.dptr(self.tau))
        s.k_size = k_size
        s.k = capi.dptr(self.k)
        s.k3_size = capi.iptr(self.k3_size)
        s.k3 = capi.dptr(self.k3)
        s.tau_size = tau_size
        s.tau = capi.dptr(self.tau)
        self.spec = s
        # --- tables (first-order part filled by set_first_order)
        t = capi.Tables()
        t.tau0 = self.tau0
        t.a_eq = aeq.value
        t.bg_size = bg_size
        t.bg_lntau0 = lt0.value
        t.bg_dlntau = dlt.value
        t.bg = capi.dptr(self.bg)
        t.bg_dd = capi.dptr(self.bg_dd)
        t.tau_free_streaming = lib.song2_free_streaming_time(C.byref(t), capi.RSA_TRIGGER_TAU_C_OVER_TAU)
        self.tables = t
        self.fo_l_max = max(l_max, s.l_max_los_t, s.l_max_los_p) + 1
        self.classes = None
        if uneven:
            self.set_uneven(**uneven)
        # first-order time grid: uniform in ln tau from before the earliest start time to tau0
        kmax_all = 2.0 * float(self.k[-1])
        tau_ini_min = C.c_double()
        if lib.song2_start_time(C.byref(s), C.byref(t), kmax_all, float(self.tau[0]), C.byref(tau_ini_min), err):
            raise RuntimeError(err.value.decode())
        lo = math.log(0.9 * tau_ini_min.value)
        hi = math.log(self.tau0)
        self.fo_tau_size = int(math.ceil((hi - lo) / fo_dlntau)) + 1
        self.fo_lntau0 = lo
        self.fo_dlntau = (hi - lo) / (self.fo_tau_size - 1)
        self.fo = None

    # ------------------------------------------------------------------ uneven batches
    def tau_rec(self):
        """Conformal time of the visibility peak (kappa' e^-kappa) on the background grid."""
        lnkd = self.bg[:, capi.BG_LN_KAPPA_DOT]
        kap = self.bg[:, capi.BG_KAPPA]
        i = int(np.argmax(lnkd - kap))
        return float(np.exp(self.tables.bg_lntau0 + i * self.tables.bg_dlntau))

    def set_uneven(self, seed=20261203, l_base=None, l_cap=None, m_choices=None, l_max_fn=None):
        """Give every triplet (pair order) its hierarchy class: l_max from its largest
        wavenumber, m_max drawn from the choices with a seeded generator."""
        l_base = L_BASE if l_base is None else l_base
        l_cap = L_CAP if l_cap is None else l_cap
        m_choices = M_MAX_CHOICES if m_choices is None else m_choices
        trec = self.tau_rec()
        n = len(self.k)
        kmax = []
        off = 0
        for i1 in range(n):
            for i2 in range(i1 + 1):
                nk3 = int(self.k3_size[i1 * n + i2])
                for i3 in range(nk3):
                    kmax.append(max(self.k[i1], self.k[i2], self.k3[off + i3]))
                off += nk3
        kmax = np.array(kmax)
        if l_max_fn is None:
            lmax = np.minimum(l_cap, l_base + np.ceil(kmax * trec / 2.0)).astype(int)
        else:
            lmax = np.array([l_max_fn(k) for k in kmax], dtype=int)
        lmax = np.minimum(lmax, self.spec.l_max_g)
        rng = np.random.default_rng(seed)
        mmax = rng.choice(np.array(m_choices), size=len(kmax))
        mmax = np.minimum(mmax, max(self.spec.m[i] for i in range(self.spec.m_size)))
        pairs = sorted(set(zip(lmax.tolist(), mmax.tolist())))
        index = {pq: i for i, pq in enumerate(pairs)}
        self.class_l_max = np.array([a for a, _ in pairs], dtype=np.int32)
        self.class_m_max = np.array([b for _, b in pairs], dtype=np.int32)
        self.triplet_class = np.array([index[(a, b)] for a, b in zip(lmax.tolist(), mmax.tolist())], dtype=np.int32)
        self.classes = pairs
        s = self.spec
        s.n_classes = len(pairs)
        s.class_l_max = capi.iptr(self.class_l_max)
        s.class_m_max = capi.iptr(self.class_m_max)
        s.triplet_class = capi.iptr(self.triplet_class)

    def class_sizes(self):
        """Number of equations (outside tight coupling) of every triplet's class."""
        if self.classes is None:
            return None
        out = []
        for L, mm in self.classes:
            nh = sum(1 for l in range(L + 1) for m in range(mm + 1) if m <= l)
            ne = sum(1 for l in range(2, L + 1) for m in range(mm + 1) if m <= l)
            nb = sum(1 for l in range(2, L + 1) for m in range(1, mm + 1) if m <= l)
            extra = 4 + (3 if mm >= 1 else 0) + (2 if mm >= 2 else 0)
            out.append(2 * nh + ne + nb + extra)
        return np.array(out)[self.triplet_class]

    # ------------------------------------------------------------------ sizes
    @property
    def n_triplets(self):
        return int(self.lib.song2_n_triplets(C.byref(self.spec)))

    @property
    def tp2_size(self):
        return int(self.lib.song2_tp2_size(C.byref(self.spec)))

    @property
    def per_type(self):
        return int(self.lib.song2_sources_per_type(C.byref(self.spec)))

    @property
    def fo_size(self):
        return capi.fo_size(self.fo_l_max)

    def fo_shape(self):
        return (len(self.k), self.fo_tau_size, self.fo_size)

    def fo_tau_grid(self):
        return np.exp(self.fo_lntau0 + self.fo_dlntau * np.arange(self.fo_tau_size))

    # ------------------------------------------------------------ first order
    def set_first_order(self, fo):
        """Install first-order values fo[k][tau][q] and compute their spline table."""
        fo = np.ascontiguousarray(fo, dtype=np.float64).reshape(self.fo_shape())
        dd = np.zeros_like(fo)
        nk, nt, nq = fo.shape
        for ik in range(nk):
            sub = np.ascontiguousarray(fo[ik])
            out = np.zeros_like(sub)
            self.lib.song2_spline_uniform(nt, nq, self.fo_dlntau, capi.dptr(sub), capi.dptr(out))
            dd[ik] = out
        self.fo, self.fo_dd = fo, dd
        t = self.tables
        t.fo_k_size = nk
        t.fo_tau_size = nt
        t.fo_lntau0 = self.fo_lntau0
        t.fo_dlntau = self.fo_dlntau
        t.fo_l_max = self.fo_l_max
        t.fo_size = nq
        t.fo = capi.dptr(self.fo)
        t.fo_dd = capi.dptr(self.fo_dd)

    def first_order_gpu(self):
        """Fill the first-order table with the GPU evolver in first-order mode."""
        fo = np.zeros(self.fo_shape())
        err = capi.errbuf()
        if self.lib.song2_gpu_first_order(C.byref(self.spec), C.byref(self.tables), self.fo_l_max,
                                          self.fo_tau_size, self.fo_lntau0, self.fo_dlntau,
                                          capi.dptr(fo), err):
            raise RuntimeError(err.value.decode())
        self.set_first_order(fo)
        return fo

    # ---------------------------------------------------------------- layout
    def pair_offset(self, i1, i2):
        return int(self.lib.song2_pair_offset(C.byref(self.spec), i1, i2))

    def work_order(self):
        """(i1, i2, i3) of every triplet in work order: k1 descending, k2 <= k1, k3."""
        out = []
        n = len(self.k)
        for i1 in range(n - 1, -1, -1):
            for i2 in range(i1 + 1):
                for i3 in range(int(self.k3_size[i1 * n + i2])):
                    out.append((i1, i2, i3))
        return out

    def triplet_view(self, flat, i1, i2, i3):
        """sources[tp][tau] of one triplet from a flat buffer [tp2][per_type]."""
        n = len(self.k)
        nk3 = int(self.k3_size[i1 * n + i2])
        off = self.pair_offset(i1, i2)
        flat = flat.reshape(self.tp2_size, self.per_type)
        return flat[:, off + i3: off + len(self.tau) * nk3: nk3]

    def tp_list(self):
        """(kind, l, m) of every source type in the reference order: T, E, B by
        lm(l, m) up to l_max_los_t / l_max_los_p, then delta_cdm (kind 'D', -1, 0)."""
        s = self.spec
        ms = [s.m[i] for i in range(s.m_size)]
        out = []
        for kind, flag, lmax in (("T", s.has_source_T, s.l_max_los_t), ("E", s.has_source_E, s.l_max_los_p),
                                 ("B", s.has_source_B, s.l_max_los_p)):
            if flag:
                out += [(kind, l, m) for l in range(lmax + 1) for m in ms if m <= l]
        if s.has_source_delta_cdm:
            out.append(("D", -1, 0))
        return out

    def triplet_k(self, i1, i2, i3):
        """(k1, k2, k) of one triplet."""
        n = len(self.k)
        off = 0
        for j1 in range(n):
            for j2 in range(j1 + 1):
                if (j1, j2) == (i1, i2):
                    return self.k[i1], self.k[i2], self.k3[off + i3]
                off += int(self.k3_size[j1 * n + j2])
        raise IndexError((i1, i2, i3))

    def to_nested(self, flat):
        """The reference layout sources[tp2][k1][k2<=k1] -> array (tau*k3_size + k3)."""
        flat = flat.reshape(self.tp2_size, self.per_type)
        n = len(self.k)
        out = []
        for tp in range(self.tp2_size):
            rows = []
            for i1 in range(n):
                row = []
                for i2 in range(i1 + 1):
                    off = self.pair_offset(i1, i2)
                    ln = len(self.tau) * int(self.k3_size[i1 * n + i2])
                    row.append(flat[tp, off:off + ln])
                rows.append(row)
            out.append(rows)
        return out


def config_problem(num, **overrides):
    cfg = dict(CONFIGS[num])
    cfg.pop("name")
    cfg.update(overrides)
    return Problem(**cfg)


def source_errors(test, ref, prob):
    """Per (source type, triplet) error max_tau |S - S_ref| / max_tau |S_ref|."""
    a = test.reshape(prob.tp2_size, prob.per_type)
    b = ref.reshape(prob.tp2_size, prob.per_type)
    errs = []
    for (i1, i2, i3) in prob.work_order():
        ta = prob.triplet_view(a, i1, i2, i3)
        tb = prob.triplet_view(b, i1, i2, i3)
        den = np.max(np.abs(tb), axis=1)
        num = np.max(np.abs(ta - tb), axis=1)
        with np.errstate(divide="ignore", invalid="ignore"):
            e = np.where(den > 0, num / np.where(den > 0, den, 1), np.where(num > 0, np.inf, 0.0))
        errs.append(e)
    return np.array(errs)
