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
