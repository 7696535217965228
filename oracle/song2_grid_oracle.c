/*
 * song2_grid_oracle.c - CPU restatement of the smart k samplings of
 * perturb2_get_k_lists (source/perturbations2.c:1610-1766 for k1/k2,
 * :1960-2178 for k3) and of the sound horizon at recombination that sets their
 * scale (CLASS's pth->rs_rec; CLASS is absent from the reference tree).
 *
 * TEST INFRASTRUCTURE ONLY: the checker of the product's grid builders
 * (song_gb300/csrc/song2_params.c); only tests/ load it.  It shares no code
 * with the product.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "song2.h"

#define O_PI 3.141592653589793238462643383279502884

/* smart k1/k2 grid; the same step rules, CMB leg then LSS leg */
int song2_oracle_k_grid_smart(double k_min_tau0, double k_max_tau0_over_l_max, double k_step_sub, double k_step_super,
                              double k_logstep_super, double k_step_transition, double k_per_decade_for_pk,
                              double k_per_decade_for_bao, double k_bao_center, double k_bao_width,
                              double k_max_for_pk, int has_cmb, int has_lss, double tau0, double rs_rec,
                              int l_scalar_max, double *out, int cap) {
  int i = 0;
  out[i++] = k_min_tau0 / tau0;
  double k = out[0];
  double k_rec = 2 * O_PI / rs_rec;
  double kmax_cmb = 0, kmax_lss = 0;
  if (has_cmb) {
    kmax_cmb = k_max_tau0_over_l_max * l_scalar_max / tau0;
    while (k < kmax_cmb) {
      double lin = k_step_super + 0.5 * (tanh((out[i - 1] - k_rec) / k_rec / k_step_transition) + 1) *
                                      (k_step_sub - k_step_super);
      double lg = out[i - 1] * (k_logstep_super - 1.);
      if ((lg > (lin * k_rec)) || (out[i - 1] > k_rec))
        k = out[i - 1] + lin * k_rec;
      else
        k = out[i - 1] * k_logstep_super;
      if (i >= cap) return -1;
      out[i++] = k;
    }
  }
  if (has_lss) {
    kmax_lss = k_max_for_pk;
    while (k < kmax_lss) {
      k *= pow(10, 1 / (k_per_decade_for_pk + (k_per_decade_for_bao - k_per_decade_for_pk) *
                                                  (1 - tanh(pow((log(k) - log(k_bao_center * k_rec)) /
                                                                    log(k_bao_width), 4)))));
      if (i >= cap) return -1;
      out[i++] = k;
    }
  }
  out[i - 1] = kmax_cmb > kmax_lss ? kmax_cmb : kmax_lss;
  return i;
}

static int o_cmp(const void *a, const void *b) {
  double x = *(const double *)a, y = *(const double *)b;
  return x < y ? -1 : (x > y ? 1 : 0);
}

static int o_merge(double *a, int n) {
  qsort(a, n, sizeof(double), o_cmp);
  int m = 0;
  for (int i = 0; i < n; ++i)
    if (!m || a[i] != a[m - 1]) a[m++] = a[i];
  return m;
}

/* smart k3 grids, pair order (k1 ascending, k2 <= k1), sizes into sizes[pair] */
int song2_oracle_k3_grids_smart(const double *k, int nk, int k3_size_min, int *sizes, double *out) {
  int64_t off = 0;
  int p = 0;
  double *tmp = (double *)malloc(sizeof(double) * (nk + k3_size_min + 8));
  for (int a = 0; a < nk; ++a)
    for (int b = 0; b <= a; ++b, ++p) {
      double k1 = k[a], k2 = k[b];
      double lo = fabs(k1 - k2) + fabs(1e-10), hi = k1 + k2 - fabs(1e-10);
      lo = fmax(lo, (k1 + k2) / 100);
      lo = fmax(lo, k[0]);
      hi = fmin(hi, k[nk - 1]);
      if (lo >= hi) {
        free(tmp);
        return 1;
      }
      int i0 = 0;
      while (k[i0] < lo) ++i0;
      int i1 = nk - 1;
      while (k[i1] > hi) --i1;
      int n = 0;
      for (int j = i0; j <= i1; ++j) tmp[n++] = k[j];
      tmp[n++] = lo;
      tmp[n++] = hi;
      n = o_merge(tmp, n);
      if (n < k3_size_min) {
        int e = k3_size_min - n + 2;
        for (int j = 0; j < e; ++j) tmp[n + j] = lo + j * (hi - lo) / (e - 1);
        n = o_merge(tmp, n + e);
      }
      sizes[p] = n;
      if (out) memcpy(out + off, tmp, sizeof(double) * n);
      off += n;
    }
  free(tmp);
  return 0;
}

/* sound horizon by the trapezoid rule on a fine ln tau grid (independent of the
   product's Simpson on the table spacing) */
double song2_oracle_sound_horizon(const song2_tables *t, double tau) {
  double x0 = t->bg_lntau0, x1 = log(tau);
  int n = 20000;
  double h = (x1 - x0) / n, s = 0;
  for (int i = 0; i <= n; ++i) {
    double x = x0 + i * h;
    double u = (x - t->bg_lntau0) / t->bg_dlntau;
    int j = (int)u;
    if (j > t->bg_size - 2) j = t->bg_size - 2;
    double b = u - j, a = 1 - b;
    const double *y0 = t->bg + (size_t)j * SONG2_BG_SIZE, *y1 = y0 + SONG2_BG_SIZE;
    const double *d0 = t->bg_dd + (size_t)j * SONG2_BG_SIZE, *d1 = d0 + SONG2_BG_SIZE;
    double lrb = a * y0[SONG2_BG_LN_RHO_B] + b * y1[SONG2_BG_LN_RHO_B] +
                 ((a * a * a - a) * d0[SONG2_BG_LN_RHO_B] + (b * b * b - b) * d1[SONG2_BG_LN_RHO_B]) * t->bg_dlntau *
                     t->bg_dlntau / 6;
    double lrg = a * y0[SONG2_BG_LN_RHO_G] + b * y1[SONG2_BG_LN_RHO_G] +
                 ((a * a * a - a) * d0[SONG2_BG_LN_RHO_G] + (b * b * b - b) * d1[SONG2_BG_LN_RHO_G]) * t->bg_dlntau *
                     t->bg_dlntau / 6;
    double cs = 1 / sqrt(3 * (1 + 0.75 * exp(lrb - lrg)));
    s += (i == 0 || i == n ? 0.5 : 1.0) * exp(x) * cs;
  }
  /* before the table: c_s = 1/sqrt(3) to the precision of R -> 0 */
  double u0 = 0.0;
  {
    const double *y0 = t->bg;
    double cs0 = 1 / sqrt(3 * (1 + 0.75 * exp(y0[SONG2_BG_LN_RHO_B] - y0[SONG2_BG_LN_RHO_G])));
    u0 = exp(x0) * cs0;
  }
  return u0 + s * h;
}

/* ------------------------------------------- source time sampling
   perturb2_timesampling_for_sources without a custom grid
   (source/perturbations2.c:2620-2869).  The splines of the background table are
   evaluated here in polynomial form on each interval,
   s(x) = y0 + c1 t + M0 t^2 / 2 + (M1 - M0) t^3 / (6 h), t = x - x_i, so that the
   derivatives come from the coefficients rather than the product's a/b basis. */
static void o_poly(const song2_tables *t, int col, double x, double *s, double *s1, double *s2) {
  double h = t->bg_dlntau;
  int i = (int)floor((x - t->bg_lntau0) / h);
  if (i < 0) i = 0;
  if (i > t->bg_size - 2) i = t->bg_size - 2;
  double u = x - (t->bg_lntau0 + i * h);
  double y0 = t->bg[(size_t)i * SONG2_BG_SIZE + col], y1 = t->bg[(size_t)(i + 1) * SONG2_BG_SIZE + col];
  double m0 = t->bg_dd[(size_t)i * SONG2_BG_SIZE + col], m1 = t->bg_dd[(size_t)(i + 1) * SONG2_BG_SIZE + col];
  double c1 = (y1 - y0) / h - h * (2 * m0 + m1) / 6, c2 = m0 / 2, c3 = (m1 - m0) / (6 * h);
  *s = y0 + u * (c1 + u * (c2 + u * c3));
  *s1 = c1 + u * (2 * c2 + 3 * c3 * u);
  *s2 = 2 * c2 + 6 * c3 * u;
}

/* kappa' = dkappa/dtau, CLASS's thermodynamics variation rate
   sqrt(kappa'^2 + (kappa''/kappa')^2 + |kappa'''/kappa'|), aH and a''/a at tau */
void song2_oracle_thermo_rates(const song2_tables *t, double tau, double *out4) {
  double x = log(tau), l, lx, lxx, h, hx, hxx;
  o_poly(t, SONG2_BG_LN_KAPPA_DOT, x, &l, &lx, &lxx);
  o_poly(t, SONG2_BG_LN_HC, x, &h, &hx, &hxx);
  /* f(tau) = e^{l(ln tau)}: f'/f = lx/tau, f''/f = (lx^2 - lx + lxx)/tau^2 */
  double kd = exp(l);
  double r1 = lx / tau;                                   /* kappa''/kappa' */
  double r2 = (lxx - lx + lx * lx) / (tau * tau);         /* kappa'''/kappa' */
  double aH = exp(h);
  out4[0] = kd;
  out4[1] = sqrt(kd * kd + r1 * r1 + fabs(r2));
  out4[2] = aH;
  out4[3] = aH * hx / tau + aH * aH; /* a''/a = (aH)' + (aH)^2 */
}

/* visibility peak: the maximum of g = kappa' e^{-kappa} on a fine ln tau scan,
   refined by parabolic steps (independent of the product's golden section) */
static double o_tau_rec(const song2_tables *t) {
  int n = 20000, best = 0;
  double x0 = t->bg_lntau0, x1 = t->bg_lntau0 + (t->bg_size - 1) * t->bg_dlntau, bestv = -1e300;
  double dx = (x1 - x0) / n;
  for (int i = 0; i <= n; ++i) {
    double x = x0 + i * dx, a, b, c, d, e, f;
    o_poly(t, SONG2_BG_LN_KAPPA_DOT, x, &a, &b, &c);
    o_poly(t, SONG2_BG_KAPPA, x, &d, &e, &f);
    double v = a - d;
    if (v > bestv) bestv = v, best = i;
  }
  double lo = x0 + (best - 1) * dx, hi = x0 + (best + 1) * dx;
  for (int it = 0; it < 200; ++it) { /* ternary search on a unimodal bracket */
    double m1 = lo + (hi - lo) / 3, m2 = hi - (hi - lo) / 3, a, b, c, d, e, f;
    o_poly(t, SONG2_BG_LN_KAPPA_DOT, m1, &a, &b, &c);
    o_poly(t, SONG2_BG_KAPPA, m1, &d, &e, &f);
    double v1 = a - d;
    o_poly(t, SONG2_BG_LN_KAPPA_DOT, m2, &a, &b, &c);
    o_poly(t, SONG2_BG_KAPPA, m2, &d, &e, &f);
    if (v1 < a - d) lo = m1;
    else hi = m2;
  }
  return exp(0.5 * (lo + hi));
}

int song2_oracle_tau_grid_class(const song2_tables *t, double stepsize, double boost, double start, double tol,
                                int has_cmb, int cap, double *out) {
  double tau;
  if (has_cmb) {
    /* the thermodynamics table starts at z = 1e4: a = 1 / (1 + 1e4) */
    double lo = t->bg_lntau0, hi = log(o_tau_rec(t));
    for (int it = 0; it < 300; ++it) {
      double mid = 0.5 * (lo + hi), a, b, c;
      o_poly(t, SONG2_BG_LN_A, mid, &a, &b, &c);
      if (a < -log(1.0 + 1e4)) lo = mid;
      else hi = mid;
    }
    double tl = exp(0.5 * (lo + hi)), tu = o_tau_rec(t), r[4];
    song2_oracle_thermo_rates(t, tl, r);
    if (r[2] / r[0] > start) return -1;
    song2_oracle_thermo_rates(t, tu, r);
    if (r[2] / r[0] < start) return -1;
    while (tu - tl > tol) {
      double tm = 0.5 * (tl + tu);
      song2_oracle_thermo_rates(t, tm, r);
      if (r[2] / r[0] > start) tu = tm;
      else tl = tm;
    }
    tau = 0.5 * (tl + tu);
  } else {
    tau = o_tau_rec(t);
  }
  int n = 0;
  out[n++] = tau;
  while (tau < t->tau0 && n < cap) {
    double r[4];
    song2_oracle_thermo_rates(t, tau, r);
    double dt = has_cmb ? stepsize / sqrt(r[1] * r[1] + boost * boost * fabs(2 * r[3] - r[2] * r[2]))
                        : stepsize / r[2];
    tau += dt;
    out[n++] = tau;
  }
  if (tau < t->tau0) return -1;
  out[n - 1] = t->tau0;
  return n;
}

/* theta_12 k3 sampling (perturbations2.c:2029-2060): angles linear between
   the angles of the clipped limits, written with the law of cosines */
int song2_oracle_k3_grids_theta12(const double *k, int nk, int n3, int *sizes, double *out) {
  int off = 0, p = 0;
  for (int i1 = 0; i1 < nk; ++i1)
    for (int i2 = 0; i2 <= i1; ++i2, ++p) {
      double a = k[i1], b = k[i2];
      double lo = fabs(a - b) + 1e-10, hi = a + b - 1e-10;
      if ((a + b) / 100 > lo) lo = (a + b) / 100;
      if (k[0] > lo) lo = k[0];
      if (k[nk - 1] < hi) hi = k[nk - 1];
      if (!(lo < hi)) return 1;
      double t0 = acos((lo * lo - a * a - b * b) / (2 * a * b));
      double t1 = acos((hi * hi - a * a - b * b) / (2 * a * b));
      double dt = (t1 - t0) / (n3 - 1);
      if (i1 == i2) {
        t0 = t0 + dt / 5;
        dt = (t1 - t0) / (n3 - 1);
      }
      sizes[p] = n3;
      for (int j = 0; j < n3; ++j) out[off + j] = sqrt(a * a + b * b + 2 * cos(t0 + j * dt) * a * b);
      off += n3;
    }
  return 0;
}
