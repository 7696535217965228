/*
 * song2_host.c - host-side C of the GB300 second-order evolver.
 *
 * Contents:
 *  - spec helpers: triplet counting, pair offsets of the flat source buffer;
 *  - defaults of the hot-path parameters (source/input2.c:2027-2371);
 *  - a flat LCDM background and a Peebles-type hydrogen recombination, the
 *    stand-in for CLASS background_init/thermodynamics_init, which SONG calls
 *    before perturb2_init (main/song.c:55-69) but which is not part of the
 *    reference tree (the CLASS submodule is empty);
 *  - uniform-grid natural cubic splines (both the device evolver and the
 *    first-order provider interpolate with them);
 *  - the coupling coefficients C and D used by perturb2_get_lm_lists
 *    (perturbations2.c:1236-1271), written as closed forms of the
 *    Clebsch-Gordan coefficients <l' m1; 1 q | l m>;
 *  - the start-time bisection of perturb2_start_time_evolution
 *    (perturbations2.c:3388-3524).
 */
#include "song2.h"
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ------------------------------------------------------------------ spec */

int song2_fo_size(int fo_l_max) {
  /* scalars + I_l, E_l, N_l, collision_g_l for l = 0..fo_l_max */
  return SONG2_FO_I + 4 * (fo_l_max + 1);
}

int64_t song2_n_triplets(const song2_spec *s) {
  int64_t n = 0;
  for (int i1 = 0; i1 < s->k_size; ++i1)
    for (int i2 = 0; i2 <= i1; ++i2) n += s->k3_size[i1 * s->k_size + i2];
  return n;
}

static int size_l_indexm(int l_max, const int *m, int m_size) {
  /* number of (l,m) pairs with l <= l_max, m in the list, m <= l */
  int n = 0;
  for (int l = 0; l <= l_max; ++l)
    for (int i = 0; i < m_size; ++i)
      if (m[i] <= l) ++n;
  return n;
}

int song2_tp2_size(const song2_spec *s) {
  /* perturb2_indices_of_perturbs (perturbations2.c:667-1075): T, E, B blocks
     of size_l_indexm(l_max_los) each, then delta_cdm. */
  int n = 0;
  if (s->has_source_T) n += size_l_indexm(s->l_max_los_t, s->m, s->m_size);
  if (s->has_source_E) n += size_l_indexm(s->l_max_los_p, s->m, s->m_size);
  if (s->has_source_B) n += size_l_indexm(s->l_max_los_p, s->m, s->m_size);
  if (s->has_source_delta_cdm) n += 1;
  return n;
}

int64_t song2_pair_offset(const song2_spec *s, int index_k1, int index_k2) {
  int64_t off = 0;
  for (int i1 = 0; i1 < s->k_size; ++i1)
    for (int i2 = 0; i2 <= i1; ++i2) {
      if (i1 == index_k1 && i2 == index_k2) return off;
      off += (int64_t)s->tau_size * s->k3_size[i1 * s->k_size + i2];
    }
  return off;
}

int64_t song2_sources_per_type(const song2_spec *s) {
  return (int64_t)s->tau_size * song2_n_triplets(s);
}

/* Bytes of the k1 slab of every source type in the flat buffer: the pairs
   (k1, k2 <= k1) are consecutive, so it is one contiguous run per type. */
static int64_t k1_run(const song2_spec *s, int index_k1) {
  int64_t n = 0;
  for (int i2 = 0; i2 <= index_k1; ++i2) n += (int64_t)s->tau_size * s->k3_size[index_k1 * s->k_size + i2];
  return n;
}

int song2_store_sources(const song2_spec *s, const double *flat, const char *dir, int index_k1, char *err) {
  if (index_k1 < 0 || index_k1 >= s->k_size) {
    snprintf(err, SONG2_ERRLEN, "index_k1 %d outside 0..%d", index_k1, s->k_size - 1);
    return 1;
  }
  char path[4096];
  snprintf(path, sizeof(path), "%s/sources_%03d.dat", dir, index_k1);
  FILE *f = fopen(path, "wb");
  if (!f) {
    snprintf(err, SONG2_ERRLEN, "cannot open %.900s for writing", path);
    return 1;
  }
  int tp2 = song2_tp2_size(s);
  int64_t per_type = song2_sources_per_type(s), off = song2_pair_offset(s, index_k1, 0), n = k1_run(s, index_k1);
  for (int tp = 0; tp < tp2; ++tp)
    if (n > 0 && fwrite(flat + (int64_t)tp * per_type + off, sizeof(double), (size_t)n, f) != (size_t)n) {
      fclose(f);
      snprintf(err, SONG2_ERRLEN, "short write to %.900s", path);
      return 1;
    }
  if (fclose(f)) {
    snprintf(err, SONG2_ERRLEN, "error closing %.900s", path);
    return 1;
  }
  return 0;
}

int song2_load_sources(const song2_spec *s, double *flat, const char *dir, int index_k1, char *err) {
  if (index_k1 < 0 || index_k1 >= s->k_size) {
    snprintf(err, SONG2_ERRLEN, "index_k1 %d outside 0..%d", index_k1, s->k_size - 1);
    return 1;
  }
  char path[4096];
  snprintf(path, sizeof(path), "%s/sources_%03d.dat", dir, index_k1);
  FILE *f = fopen(path, "rb");
  if (!f) {
    snprintf(err, SONG2_ERRLEN, "cannot open %.900s for reading", path);
    return 1;
  }
  int tp2 = song2_tp2_size(s);
  int64_t per_type = song2_sources_per_type(s), off = song2_pair_offset(s, index_k1, 0), n = k1_run(s, index_k1);
  for (int tp = 0; tp < tp2; ++tp)
    if (n > 0 && fread(flat + (int64_t)tp * per_type + off, sizeof(double), (size_t)n, f) != (size_t)n) {
      fclose(f);
      snprintf(err, SONG2_ERRLEN, "Error reading from %.900s: fewer entries than tau_size*k3_size per (type, k2)", path);
      return 1;
    }
  fclose(f);
  return 0;
}

void song2_spec_defaults(song2_spec *s) {
  memset(s, 0, sizeof(*s));
  s->l_max_g = s->l_max_pol_g = s->l_max_ur = 8;         /* input2.c:2257-2259 */
  s->l_max_los_t = s->l_max_los_p = 2;                   /* input2.c:2265-2266 */
  s->l_max_los_quadratic_t = s->l_max_los_quadratic_p = 2;
  s->radiation_streaming_trigger_tau_over_tau_k = 90;    /* input2.c:2140 */
  s->m_size = 1; s->m[0] = 0;                            /* input2.c:2268-2270 */
  s->has_polarization2 = 1;
  s->has_quadratic_sources = 1;
  s->has_quadratic_liouville = 1;
  s->has_quadratic_collision = 1;
  s->tight_coupling = 1;                                 /* tca2_first_order_pitrou */
  s->tca_trigger_tau_c_over_tau_h = 0.01;                /* input2.c:2136 */
  s->tca_trigger_tau_c_over_tau_k = 0.007;               /* input2.c:2137 */
  s->ic = SONG2_IC_AD;
  s->has_source_T = 1; s->has_source_E = 1; s->has_source_B = 0;
  s->rtol = 1e-4;                                        /* input2.c:2248 */
  s->threshold = 1e-6;
  s->max_steps = 200000;
  s->start_small_k_at_tau_c_over_tau_h = 0.0015;         /* input2.c:2280 */
  s->start_large_k_at_tau_h_over_tau_k = 0.07;           /* input2.c:2281 */
  s->tol_tau_approx = 1e-10;
}

/* ------------------------------------------------------------- splines */

void song2_spline_uniform(int n, int ncol, double dx, const double *y, double *dd) {
  /* Natural cubic spline on a uniform grid: solve the tridiagonal system
     dd[i-1] + 4 dd[i] + dd[i+1] = 6 (y[i+1]-2y[i]+y[i-1])/dx^2, dd[0]=dd[n-1]=0,
     column by column with the Thomas algorithm. */
  double *c = (double *)malloc(sizeof(double) * (size_t)n);
  for (int q = 0; q < ncol; ++q) {
    dd[q] = 0.0;
    if (n < 3) { for (int i = 0; i < n; ++i) dd[(size_t)i * ncol + q] = 0.0; continue; }
    c[0] = 0.0;
    double prev = 0.0; /* modified rhs of the previous row */
    for (int i = 1; i < n - 1; ++i) {
      double r = 6.0 * (y[(size_t)(i + 1) * ncol + q] - 2.0 * y[(size_t)i * ncol + q] +
                        y[(size_t)(i - 1) * ncol + q]) / (dx * dx);
      double b = 4.0 - c[i - 1];
      c[i] = 1.0 / b;
      prev = (r - prev) / b;
      dd[(size_t)i * ncol + q] = prev;
    }
    dd[(size_t)(n - 1) * ncol + q] = 0.0;
    for (int i = n - 2; i >= 1; --i)
      dd[(size_t)i * ncol + q] -= c[i] * dd[(size_t)(i + 1) * ncol + q];
  }
  free(c);
}

static double spline_eval_uniform(int n, int ncol, double x0, double dx, const double *y,
                                  const double *dd, int q, double x) {
  double u = (x - x0) / dx;
  int i = (int)floor(u);
  if (i < 0) i = 0;
  if (i > n - 2) i = n - 2;
  double b = u - i, a = 1.0 - b;
  return a * y[(size_t)i * ncol + q] + b * y[(size_t)(i + 1) * ncol + q] +
         ((a * a * a - a) * dd[(size_t)i * ncol + q] + (b * b * b - b) * dd[(size_t)(i + 1) * ncol + q]) *
             (dx * dx) / 6.0;
}

/* --------------------------------------------------------- background */

/* Physical constants (SI) */
#define C_LIGHT 2.99792458e8
#define MPC_M 3.0856775814913673e22
#define SIGMA_T 6.6524587158e-29
#define K_B 1.380649e-23
#define M_ELECTRON 9.1093837015e-31
#define H_PLANCK 6.62607015e-34
#define M_H 1.673575e-27
#define EV 1.602176634e-19
#define RHO_CRIT_H2 1.87834e-26 /* kg/m^3 for h = 1 */

typedef struct {
  double rho_g0, rho_ur0, rho_b0, rho_cdm0, rho_L0; /* CLASS units, Mpc^-2 */
} bg_params;

static void bg_rhos(const bg_params *p, double a, double *rg, double *rur, double *rb, double *rc, double *rl) {
  double a2 = a * a, a3 = a2 * a, a4 = a2 * a2;
  *rg = p->rho_g0 / a4; *rur = p->rho_ur0 / a4;
  *rb = p->rho_b0 / a3; *rc = p->rho_cdm0 / a3; *rl = p->rho_L0;
}

static double bg_H(const bg_params *p, double a) {
  double rg, rur, rb, rc, rl;
  bg_rhos(p, a, &rg, &rur, &rb, &rc, &rl);
  return sqrt(rg + rur + rb + rc + rl);
}

/* dtau / dln a = 1 / (a H) */
static double dtau_dlna(const bg_params *p, double lna) {
  double a = exp(lna);
  return 1.0 / (a * bg_H(p, a));
}

/* Peebles three-level hydrogen recombination (Peebles 1968, with the
   case-B recombination fit of Pequignot et al. 1991 and the fudge factor 1.14
   of Seager, Sasselov & Scott 1999), helium in Saha equilibrium for both of
   its ionisations (He III -> He II at 54.4 eV, He II -> He I at 24.6 eV, the
   way RECFAST starts its history), and the matter temperature equal to the
   radiation temperature.  Returns x_e(z) = n_e / n_H on a table of z. */
typedef struct { int n; double z0, dz; double *xe; } xe_table;


/* Saha factors (2 pi m_e k T / h^2)^{3/2} e^{-E/kT} times the ratio of the
   statistical weights, for hydrogen (1), He II -> He III (1) and He I -> He II (4) */
typedef struct { double H, He2, He1; } saha_s;

static saha_s saha_factors(double T) {
  double q = pow(2.0 * M_PI * M_ELECTRON * K_B * T / (H_PLANCK * H_PLANCK), 1.5);
  saha_s f;
  f.H = q * exp(-13.605693 * EV / (K_B * T));
  f.He2 = q * exp(-54.4177650 * EV / (K_B * T));
  f.He1 = 4.0 * q * exp(-24.5873876 * EV / (K_B * T));
  return f;
}

/* electrons per hydrogen nucleus from helium at electron density ne (m^-3) */
static double helium_electrons(const saha_s *f, double ne, double fHe) {
  double r1 = f->He1 / ne, r2 = f->He2 / ne; /* n_HeII/n_HeI, n_HeIII/n_HeII */
  if (!(r1 < 1e300)) return 2.0 * fHe;
  double den = 1.0 + r1 + r1 * r2;
  if (!(den < 1e300)) return 2.0 * fHe;
  return fHe * (r1 + 2.0 * r1 * r2) / den;
}

/* x_e with hydrogen and helium all in Saha equilibrium: bisection on the
   increasing x - (x_HII(x) + helium(x)) over [0, 1 + 2 fHe]; also returns x_HII */
static double saha_all(const saha_s *f, double nH, double fHe, double *xH_out) {
  double lo = 0.0, hi = 1.0 + 2.0 * fHe;
  for (int it = 0; it < 200; ++it) {
    double x = 0.5 * (lo + hi);
    double ne = x * nH;
    double xH = 1.0 / (1.0 + ne / f->H);
    double g = x - (xH + helium_electrons(f, ne, fHe));
    if (g > 0) hi = x;
    else lo = x;
  }
  double x = 0.5 * (lo + hi);
  *xH_out = 1.0 / (1.0 + x * nH / f->H);
  return x;
}

static int recombination(const song2_cosmo *c, const bg_params *bp, xe_table *tab) {
  double h = c->h;
  double nH0 = (1.0 - c->YHe) * c->omega_b * RHO_CRIT_H2 / M_H; /* m^-3 (omega_b = Omega_b h^2) */
  /* helium nuclei per hydrogen nucleus, with RECFAST's m_He / m_H */
  double fHe = c->YHe / (3.9715 * (1.0 - c->YHe));
  tab->n = 40001; tab->z0 = 0.0; tab->dz = 0.25; /* z in [0, 10000] */
  tab->xe = (double *)malloc(sizeof(double) * tab->n);
  if (!tab->xe) return 1;
  (void)h;
  const double lambda_a = 121.5682e-9, Lambda2s = 8.2245809, E2s = 13.605693 * EV / 4.0;
  const double Ealpha = 13.605693 * EV * 0.75;
  /* march from z = 10000 down; everything in Saha equilibrium until x_HII
     drops below 0.985, then Peebles for x = x_HII with a backward-Euler step
     solved by Newton iteration, helium in Saha at the electron density of the
     step */
  int peebles = 0;
  double x = 1.0;
  for (int i = tab->n - 1; i >= 0; --i) {
    double z = tab->z0 + i * tab->dz;
    double T = c->T_cmb * (1.0 + z);
    double nH = nH0 * pow(1.0 + z, 3);
    saha_s sf = saha_factors(T);
    if (!peebles) {
      double xH;
      double xe = saha_all(&sf, nH, fHe, &xH);
      x = xH;
      tab->xe[i] = xe;
      if (xH <= 0.985) peebles = 1;
      continue;
    }
    /* one backward-Euler step from z+dz to z: x_new = x_old - dz * f(z, x_new) where
       f = dx/dz of the Peebles equation */
    double a = 1.0 / (1.0 + z);
    double H_si = bg_H(bp, a) * C_LIGHT / MPC_M; /* 1/s */
    double tt = T / 1e4;
    double alphaB = 1.14 * 1e-19 * 4.309 * pow(tt, -0.6166) / (1.0 + 0.6703 * pow(tt, 0.5300)); /* m^3/s */
    double betaB = alphaB * pow(2.0 * M_PI * M_ELECTRON * K_B * T / (H_PLANCK * H_PLANCK), 1.5) * exp(-E2s / (K_B * T));
    double K = pow(lambda_a, 3) / (8.0 * M_PI * H_si);
    double boltz = exp(-Ealpha / (K_B * T));
    double xold = x, xn = x;
    for (int it = 0; it < 50; ++it) {
      double one_m = 1.0 - xn;
      double Cr = (1.0 + K * Lambda2s * nH * one_m) / (1.0 + K * (Lambda2s + betaB) * nH * one_m);
      double rate = Cr * (alphaB * nH * xn * xn - betaB * one_m * boltz); /* -dx/dt [1/s] */
      double f = rate / (H_si * (1.0 + z)); /* dx/dz */
      double g = xn - xold + tab->dz * f;   /* going down in z: x(z) = x(z+dz) - dz*dx/dz */
      /* derivative of g wrt xn (numerical) */
      double eps = 1e-7 * (fabs(xn) + 1e-12);
      double xp = xn + eps, om2 = 1.0 - xp;
      double Cr2 = (1.0 + K * Lambda2s * nH * om2) / (1.0 + K * (Lambda2s + betaB) * nH * om2);
      double f2 = Cr2 * (alphaB * nH * xp * xp - betaB * om2 * boltz) / (H_si * (1.0 + z));
      double dg = 1.0 + tab->dz * (f2 - f) / eps;
      double step = g / dg;
      xn -= step;
      if (xn < 1e-12) xn = 1e-12;
      if (xn > 1.0) xn = 1.0;
      if (fabs(step) < 1e-14 * fabs(xn)) break;
    }
    x = xn;
    tab->xe[i] = x + helium_electrons(&sf, x * nH, fHe);
  }
  return 0;
}

/* reionisation (CLASS's reio_camb with its default widths): x_e rises from its
   recombination value to 1 + f_He around z_reio along a tanh in (1+z)^{3/2},
   and by f_He more around z = 3.5 as helium ionises again */
static double xe_reio(double xe_rec, double z, double z_reio, double fHe) {
  const double ex = 1.5, width = 0.5, z_he = 3.5, width_he = 0.5;
  double arg = (pow(1.0 + z_reio, ex) - pow(1.0 + z, ex)) / (ex * pow(1.0 + z_reio, ex - 1.0)) / width;
  double xe = (1.0 + fHe - xe_rec) * (tanh(arg) + 1.0) / 2.0 + xe_rec;
  xe += fHe * (tanh((z_he - z) / width_he) + 1.0) / 2.0;
  return xe;
}

static double xe_at_z(const xe_table *t, double z) {
  if (z >= t->z0 + (t->n - 1) * t->dz) return t->xe[t->n - 1];
  if (z <= t->z0) return t->xe[0];
  double u = (z - t->z0) / t->dz;
  int i = (int)u;
  double f = u - i;
  return (1 - f) * t->xe[i] + f * t->xe[i + 1];
}

int song2_background_compute(const song2_cosmo *c, int bg_size, double *bg, double *bg_dd,
                             double *lntau0_out, double *dlntau_out, double *tau0_out,
                             double *a_eq_out, char *err) {
  if (bg_size < 16) { snprintf(err, SONG2_ERRLEN, "bg_size too small"); return 1; }
  bg_params p;
  double H0 = c->h / 2997.92458; /* 1/Mpc */
  double Og = 2.472819e-5 * pow(c->T_cmb / 2.7255, 4) / (c->h * c->h);
  double Our = c->N_eff * 7.0 / 8.0 * pow(4.0 / 11.0, 4.0 / 3.0) * Og;
  double Ob = c->omega_b / (c->h * c->h), Oc = c->omega_cdm / (c->h * c->h);
  double OL = 1.0 - Og - Our - Ob - Oc;
  p.rho_g0 = H0 * H0 * Og; p.rho_ur0 = H0 * H0 * Our;
  p.rho_b0 = H0 * H0 * Ob; p.rho_cdm0 = H0 * H0 * Oc; p.rho_L0 = H0 * H0 * OL;
  *a_eq_out = (Og + Our) / (Ob + Oc);

  /* tau(a) by Simpson integration on a fine ln a grid, starting from the
     radiation-era limit tau = a / sqrt(rho_r0). */
  const int NA = 200001;
  const double lna_min = log(1e-12), lna_max = 0.0;
  double dl = (lna_max - lna_min) / (NA - 1);
  double *lntau_a = (double *)malloc(sizeof(double) * NA);
  double tau = exp(lna_min) / sqrt(p.rho_g0 + p.rho_ur0);
  lntau_a[0] = log(tau);
  for (int i = 1; i < NA; ++i) {
    double l0 = lna_min + (i - 1) * dl;
    tau += dl / 6.0 * (dtau_dlna(&p, l0) + 4.0 * dtau_dlna(&p, l0 + 0.5 * dl) + dtau_dlna(&p, l0 + dl));
    lntau_a[i] = log(tau);
  }
  double tau0 = tau;
  *tau0_out = tau0;

  xe_table xt;
  if (recombination(c, &p, &xt)) { free(lntau_a); snprintf(err, SONG2_ERRLEN, "recombination alloc"); return 1; }

  /* ln tau grid from tau = 1e-3 Mpc to tau0 */
  double lt0 = log(1e-3), lt1 = log(tau0);
  double dlt = (lt1 - lt0) / (bg_size - 1);
  *lntau0_out = lt0; *dlntau_out = dlt;
  double nH0 = (1.0 - c->YHe) * c->omega_b * RHO_CRIT_H2 / M_H;
  double *kdot = (double *)malloc(sizeof(double) * bg_size);
  int j = 0;
  for (int i = 0; i < bg_size; ++i) {
    double lt = lt0 + i * dlt;
    if (i == bg_size - 1) lt = lt1;
    /* invert ln tau(ln a): bracket, then cubic Hermite with d ln tau / d ln a = 1/(tau a H) */
    while (j < NA - 2 && lntau_a[j + 1] < lt) ++j;
    double lna;
    if (lt <= lntau_a[0]) {
      lna = lna_min + (lt - lntau_a[0]); /* radiation era: a proportional to tau */
    } else {
      double x0 = lntau_a[j], x1 = lntau_a[j + 1];
      double y0 = lna_min + j * dl, y1 = y0 + dl;
      double d0 = exp(x0) / dtau_dlna(&p, y0), d1 = exp(x1) / dtau_dlna(&p, y1); /* dln a/dln tau */
      double hh = x1 - x0, t = (lt - x0) / hh;
      double h00 = 2 * t * t * t - 3 * t * t + 1, h10 = t * t * t - 2 * t * t + t;
      double h01 = -2 * t * t * t + 3 * t * t, h11 = t * t * t - t * t;
      lna = h00 * y0 + h10 * hh * d0 + h01 * y1 + h11 * hh * d1;
    }
    double a = exp(lna);
    double rg, rur, rb, rc, rl;
    bg_rhos(&p, a, &rg, &rur, &rb, &rc, &rl);
    double H = sqrt(rg + rur + rb + rc + rl);
    double Hc = a * H;
    /* d(aH)/dtau = a^2 H^2 - 3/2 a^2 sum (rho + p) */
    double Hcp = a * a * H * H - 1.5 * a * a * (4.0 / 3.0 * (rg + rur) + rb + rc);
    double taun = exp(lt);
    double z = 1.0 / a - 1.0;
    double xe = xe_at_z(&xt, z);
    if (c->z_reio > 0) xe = xe_reio(xe, z, c->z_reio, c->YHe / (3.9715 * (1.0 - c->YHe)));
    double ne = xe * nH0 / (a * a * a);
    kdot[i] = a * ne * SIGMA_T * MPC_M;
    double *row = bg + (size_t)i * SONG2_BG_SIZE;
    row[SONG2_BG_LN_A] = lna;
    row[SONG2_BG_LN_HC] = log(Hc);
    row[SONG2_BG_HC_PRIME_TAU2] = Hcp * taun * taun;
    row[SONG2_BG_LN_RHO_G] = log(rg);
    row[SONG2_BG_LN_RHO_B] = log(rb);
    row[SONG2_BG_LN_RHO_CDM] = log(rc);
    row[SONG2_BG_LN_RHO_UR] = log(rur);
    row[SONG2_BG_LN_KAPPA_DOT] = log(kdot[i]);
  }
  /* optical depth kappa(tau) = int_tau^tau0 kappa_dot dtau' (trapezoid in ln tau) */
  double kap = 0.0;
  bg[(size_t)(bg_size - 1) * SONG2_BG_SIZE + SONG2_BG_KAPPA] = 0.0;
  for (int i = bg_size - 2; i >= 0; --i) {
    double t0 = exp(lt0 + i * dlt), t1 = exp(lt0 + (i + 1) * dlt);
    kap += 0.5 * dlt * (kdot[i] * t0 + kdot[i + 1] * t1);
    bg[(size_t)i * SONG2_BG_SIZE + SONG2_BG_KAPPA] = kap;
  }
  song2_spline_uniform(bg_size, SONG2_BG_SIZE, dlt, bg, bg_dd);
  free(kdot); free(lntau_a); free(xt.xe);
  return 0;
}

/* ---------------------------------------------------- coupling coefficients */
/* With the SONG multipole convention f(n) = sum_lm (-i)^l sqrt(4pi/(2l+1)) f_lm Y_lm(n)
   the (l,m) multipole of (n . v) f, v = sum_q v_[q] n_[q]-components, is
   sum_q v_[q] [ c_minus(l,m-q,m) f_{l-1,m-q} - c_plus(l,m-q,m) f_{l+1,m-q} ] (times i),
   with c_minus = <l-1 0;1 0|l 0><l-1 m1;1 q|l m> and
        c_plus  = <l+1 0;1 0|l 0><l+1 m1;1 q|l m>  (Condon-Shortley phases).
   The spin-2 coefficients differ by the ratio of the spin-2 and spin-0 3j symbols,
   and d_zero is the l' = l coupling of the spin-2 harmonics that mixes E and B. */

double song2_coupling_c_minus(int l, int m1, int m) {
  if (l < 1 || abs(m) > l || abs(m1) > l - 1) return 0.0;
  double L = l;
  if (m1 == m) return sqrt(L * L - (double)m * m) / (2 * L - 1);
  if (m1 == m - 1) return sqrt((L + m - 1) * (L + m) / 2.0) / (2 * L - 1);
  if (m1 == m + 1) return sqrt((L - m - 1) * (L - m) / 2.0) / (2 * L - 1);
  return 0.0;
}

double song2_coupling_c_plus(int l, int m1, int m) {
  if (l < 0 || abs(m) > l || abs(m1) > l + 1) return 0.0;
  double L = l;
  if (m1 == m) return sqrt((L + 1) * (L + 1) - (double)m * m) / (2 * L + 3);
  if (m1 == m - 1) return -sqrt((L - m + 1) * (L - m + 2) / 2.0) / (2 * L + 3);
  if (m1 == m + 1) return -sqrt((L + m + 1) * (L + m + 2) / 2.0) / (2 * L + 3);
  return 0.0;
}

double song2_coupling_d_minus(int l, int m1, int m) {
  if (l <= 2) return 0.0;
  return song2_coupling_c_minus(l, m1, m) * sqrt((double)l * l - 4.0) / l;
}

double song2_coupling_d_plus(int l, int m1, int m) {
  if (l < 2) return 0.0;
  return song2_coupling_c_plus(l, m1, m) * sqrt((double)(l + 1) * (l + 1) - 4.0) / (l + 1);
}

double song2_coupling_d_zero(int l, int m1, int m) {
  if (l < 2 || abs(m) > l || abs(m1) > l) return 0.0;
  double L = l, pre = 2.0 / (L * (L + 1));
  if (m1 == m) return pre * m;
  if (m1 == m - 1) return -pre * sqrt((L + m) * (L - m + 1) / 2.0);
  if (m1 == m + 1) return pre * sqrt((L - m) * (L + m + 1) / 2.0);
  return 0.0;
}

/* Wigner 3j symbol (j1 j2 j3; m1 m2 m3) by the Racah sum, with the factorials as
   plain doubles (exact up to 22!, and the arguments stay below 40 for the
   delta-tilde couplings, whose l, l1, l2 are bounded by twice the quadratic
   LOS multipole cut). */
static double threej(int j1, int j2, int j3, int m1, int m2, int m3) {
  if (m1 + m2 + m3 != 0 || j3 < abs(j1 - j2) || j3 > j1 + j2) return 0.0;
  if (abs(m1) > j1 || abs(m2) > j2 || abs(m3) > j3 || j1 + j2 + j3 + 1 > 170) return 0.0;
  double f[171];
  f[0] = 1.0;
  for (int i = 1; i <= j1 + j2 + j3 + 1; ++i) f[i] = f[i - 1] * (double)i;
  double tri = f[j1 + j2 - j3] * f[j1 - j2 + j3] * f[-j1 + j2 + j3] / f[j1 + j2 + j3 + 1];
  double ms = f[j1 + m1] * f[j1 - m1] * f[j2 + m2] * f[j2 - m2] * f[j3 + m3] * f[j3 - m3];
  int kmin = 0, kmax = j1 + j2 - j3;
  if (j2 - j3 - m1 > kmin) kmin = j2 - j3 - m1;
  if (j1 - j3 + m2 > kmin) kmin = j1 - j3 + m2;
  if (j1 - m1 < kmax) kmax = j1 - m1;
  if (j2 + m2 < kmax) kmax = j2 + m2;
  double sum = 0.0;
  for (int k = kmin; k <= kmax; ++k) {
    double d = f[k] * f[j3 - j2 + k + m1] * f[j3 - j1 + k - m2] * f[j1 + j2 - j3 - k] * f[j1 - k - m1] * f[j2 - k + m2];
    sum += (k & 1) ? -1.0 / d : 1.0 / d;
  }
  double v = sqrt(tri * ms) * sum;
  return ((j1 - j2 - m3) & 1) ? -v : v;
}

double song2_delta_tilde_coupling(int field, int l, int m, int l1, int m1, int l2) {
  if (field < 0 || field > 2 || l < 0 || l1 < 0 || l2 < 0) return 0.0;
  int F = field == 0 ? 0 : 2;
  double pre = field == 0 ? 0.5 : 1.0;
  if (l2 < F || l < F) return 0.0;
  int L = l - l1 - l2;
  int odd_field = field == 2;
  if ((abs(L) % 2 != 0) != odd_field) return 0.0;
  int e = odd_field ? abs(L - 1) / 2 : abs(L) / 2;
  double sign = (e & 1) ? -1.0 : 1.0;
  int m2 = m - m1;
  double v = threej(l1, l2, l, 0, F, -F) * threej(l1, l2, l, m1, m2, -m);
  if (v == 0.0) return 0.0;
  return pre * sign * ((m & 1) ? -1.0 : 1.0) * (2.0 * l + 1) * v;
}

double song2_free_streaming_time(const song2_tables *tab, double trigger) {
  /* g(x) = ln(tau_c/tau) - ln(trigger) = -ln kappa'(tau) - x - ln(trigger), x = ln tau:
     negative until photon decoupling, positive after (no reionisation) */
  double lo = tab->bg_lntau0, hi = tab->bg_lntau0 + (tab->bg_size - 1) * tab->bg_dlntau;
  double lt = log(trigger);
#define G(x) (-spline_eval_uniform(tab->bg_size, SONG2_BG_SIZE, tab->bg_lntau0, tab->bg_dlntau, tab->bg, tab->bg_dd, \
                                   SONG2_BG_LN_KAPPA_DOT, (x)) - (x) - lt)
  if (G(hi) <= 0) return tab->tau0;
  if (G(lo) > 0) return exp(lo);
  for (int it = 0; it < 200 && hi - lo > 1e-13; ++it) {
    double mid = 0.5 * (lo + hi);
    if (G(mid) > 0) hi = mid; else lo = mid;
  }
#undef G
  return exp(0.5 * (lo + hi));
}

/* ------------------------------------------------------------ start time */

static void bg_eval_host(const song2_tables *t, double tau, double *Hc, double *kappa_dot) {
  double x = log(tau);
  *Hc = exp(spline_eval_uniform(t->bg_size, SONG2_BG_SIZE, t->bg_lntau0, t->bg_dlntau, t->bg, t->bg_dd,
                                SONG2_BG_LN_HC, x));
  *kappa_dot = exp(spline_eval_uniform(t->bg_size, SONG2_BG_SIZE, t->bg_lntau0, t->bg_dlntau, t->bg,
                                       t->bg_dd, SONG2_BG_LN_KAPPA_DOT, x));
}

int song2_start_time(const song2_spec *s, const song2_tables *t, double k, double tau_upper,
                     double *tau_ini, char *err) {
  double tau_lower = exp(t->bg_lntau0);
  double Hc, kd;
  bg_eval_host(t, tau_lower, &Hc, &kd);
  if (Hc / kd > s->start_small_k_at_tau_c_over_tau_h || k / Hc > s->start_large_k_at_tau_h_over_tau_k) {
    snprintf(err, SONG2_ERRLEN, "start time: background table starts too late for k=%g (tau_c/tau_h=%g, k/aH=%g)",
             k, Hc / kd, k / Hc);
    return 1;
  }
  double tau_mid = 0.5 * (tau_lower + tau_upper);
  int it = 0;
  while ((tau_upper - tau_lower) / tau_lower > s->tol_tau_approx && it < 200) {
    bg_eval_host(t, tau_mid, &Hc, &kd);
    if (Hc / kd > s->start_small_k_at_tau_c_over_tau_h || k / Hc > s->start_large_k_at_tau_h_over_tau_k)
      tau_upper = tau_mid;
    else
      tau_lower = tau_mid;
    tau_mid = 0.5 * (tau_lower + tau_upper);
    ++it;
  }
  *tau_ini = tau_mid;
  return 0;
}

/* --------------------------------------------------------------- grids */
/* perturb2_get_k_lists (perturbations2.c:1573-2530), lin/log sampling only,
   and the custom time sampling of perturb2_timesampling_for_sources
   (perturbations2.c:2580-2598). */

static void lin_space(double *out, double a, double b, int n) {
  for (int i = 0; i < n; ++i) out[i] = (n > 1) ? a + i * (b - a) / (n - 1) : a;
}

static void log_space(double *out, double a, double b, int n) {
  double la = log(a), lb = log(b);
  for (int i = 0; i < n; ++i) out[i] = (n > 1) ? exp(la + i * (lb - la) / (n - 1)) : a;
}

int song2_k_grid(int log_sampling, double k_min, double k_max, int k_size, double *k_out) {
  if (k_size < 1 || k_min <= 0 || k_max < k_min) return 1;
  if (log_sampling) log_space(k_out, k_min, k_max, k_size);
  else lin_space(k_out, k_min, k_max, k_size);
  return 0;
}

int song2_k3_grids(const double *k, int k_size, int k3_size, int log_sampling, int *k3_size_out,
                   double *k3_out, char *err) {
  /* k3 in [max(|k1-k2| + 1e-10, (k1+k2)/100, k_min), min(k1+k2 - 1e-10, k_max)]
     (perturbations2.c:1973-1984, _MIN_K3_DISTANCE_ and _MIN_K3_RATIO_ of
     include/perturbations2.h:178,187) */
  int64_t off = 0;
  for (int i1 = 0; i1 < k_size; ++i1)
    for (int i2 = 0; i2 < k_size; ++i2) k3_size_out[i1 * k_size + i2] = 0;
  for (int i1 = 0; i1 < k_size; ++i1)
    for (int i2 = 0; i2 <= i1; ++i2) {
      double k1 = k[i1], k2 = k[i2];
      double k3_min = fabs(k1 - k2) + 1e-10, k3_max = k1 + k2 - 1e-10;
      if ((k1 + k2) / 100 > k3_min) k3_min = (k1 + k2) / 100;
      if (k[0] > k3_min) k3_min = k[0];
      if (k[k_size - 1] < k3_max) k3_max = k[k_size - 1];
      if (k3_min >= k3_max) {
        snprintf(err, SONG2_ERRLEN, "found k3_min=%g>k3_max=%g for k1(%d)=%g and k2(%d)=%g", k3_min, k3_max,
                 i1, k1, i2, k2);
        return 1;
      }
      k3_size_out[i1 * k_size + i2] = k3_size;
      if (k3_out) {
        if (log_sampling) log_space(k3_out + off, k3_min, k3_max, k3_size);
        else lin_space(k3_out + off, k3_min, k3_max, k3_size);
      }
      off += k3_size;
    }
  return 0;
}

int song2_tau_grid(int log_sampling, double tau_ini, double tau_end, int tau_size, double *out) {
  if (tau_size < 1 || tau_ini <= 0 || tau_end < tau_ini) return 1;
  if (log_sampling) log_space(out, tau_ini, tau_end, tau_size);
  else lin_space(out, tau_ini, tau_end, tau_size);
  return 0;
}

/* ------------------------------------------------------------ table providers */

int song2_first_order_from_provider(const song2_spec *spec, int fo_l_max, int fo_tau_size, double fo_lntau0,
                                    double fo_dlntau, song2_fo_provider provider, void *user, int n_provided,
                                    const int *qs_map, double *fo_out, double *fo_dd_out, song2_tables *tab,
                                    char *err) {
  int nq = song2_fo_size(fo_l_max);
  if (!spec || !provider || !qs_map || !fo_out || !fo_dd_out || !tab || fo_tau_size < 3 || n_provided < 1 ||
      !(fo_dlntau > 0)) {
    snprintf(err, SONG2_ERRLEN, "first-order provider: bad arguments");
    return 1;
  }
  for (int q = 0; q < nq; ++q)
    if (qs_map[q] >= n_provided) {
      snprintf(err, SONG2_ERRLEN, "first-order provider: quantity %d maps to %d, beyond the %d provided", q,
               qs_map[q], n_provided);
      return 1;
    }
  double *row = (double *)malloc(sizeof(double) * (size_t)n_provided);
  if (!row) {
    snprintf(err, SONG2_ERRLEN, "first-order provider: out of host memory");
    return 1;
  }
  for (int ik = 0; ik < spec->k_size; ++ik) {
    double *blk = fo_out + (size_t)ik * fo_tau_size * nq;
    for (int j = 0; j < fo_tau_size; ++j) {
      double tau = exp(fo_lntau0 + j * fo_dlntau);
      if (provider(user, ik, spec->k[ik], tau, row)) {
        snprintf(err, SONG2_ERRLEN, "first-order provider failed at k[%d] = %g, tau = %g", ik, spec->k[ik], tau);
        free(row);
        return 1;
      }
      for (int q = 0; q < nq; ++q) blk[(size_t)j * nq + q] = qs_map[q] < 0 ? 0.0 : row[qs_map[q]];
    }
    song2_spline_uniform(fo_tau_size, nq, fo_dlntau, blk, fo_dd_out + (size_t)ik * fo_tau_size * nq);
  }
  free(row);
  tab->fo_k_size = spec->k_size;
  tab->fo_tau_size = fo_tau_size;
  tab->fo_lntau0 = fo_lntau0;
  tab->fo_dlntau = fo_dlntau;
  tab->fo_l_max = fo_l_max;
  tab->fo_size = nq;
  tab->fo = fo_out;
  tab->fo_dd = fo_dd_out;
  return 0;
}

int song2_background_from_provider(int bg_size, double bg_lntau0, double bg_dlntau, song2_bg_provider provider,
                                   void *user, double *bg_out, double *bg_dd_out, song2_tables *tab, char *err) {
  if (!provider || !bg_out || !bg_dd_out || !tab || bg_size < 3 || !(bg_dlntau > 0)) {
    snprintf(err, SONG2_ERRLEN, "background provider: bad arguments");
    return 1;
  }
  for (int j = 0; j < bg_size; ++j) {
    double tau = exp(bg_lntau0 + j * bg_dlntau);
    if (provider(user, tau, bg_out + (size_t)j * SONG2_BG_SIZE)) {
      snprintf(err, SONG2_ERRLEN, "background provider failed at tau = %g", tau);
      return 1;
    }
  }
  song2_spline_uniform(bg_size, SONG2_BG_SIZE, bg_dlntau, bg_out, bg_dd_out);
  tab->bg_size = bg_size;
  tab->bg_lntau0 = bg_lntau0;
  tab->bg_dlntau = bg_dlntau;
  tab->bg = bg_out;
  tab->bg_dd = bg_dd_out;
  return 0;
}
