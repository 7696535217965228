/*
 * song2_los_oracle.c - CPU restatement of SONG's line-of-sight integration
 * (source/transfer2.c, source/bessel2.c): second-order transfer functions from
 * the second-order sources.
 *
 * TEST INFRASTRUCTURE ONLY: the parity checker of the GPU line-of-sight
 * kernels (song_gb300/csrc/song2_los.cu); only tests/, __graft_entry__.smoke()
 * and bench.py's CPU leg load it.  It shares no code with the product.
 *
 * Followed function by function:
 *   transfer2_get_k3_size / _get_k3_sizes / _get_k3_list   transfer2.c:1329-1860
 *   transfer2_get_lm_lists (type, l, m order)                transfer2.c:1121-1320
 *   transfer2_get_time_grid                                  transfer2.c:2366-2610
 *   transfer2_interpolate_sources_in_k / _in_time            transfer2.c:2612-2926
 *   transfer2_integrate / transfer2_compute                  transfer2.c:1861-2365
 *   bessel2_get_l1_list / _get_xx_list                       bessel2.c:832-1000
 *   bessel2_J_for_Llm / bessel2_J_Llm / bessel2_j_for_l1     bessel2.c:1041-1800
 *   array_spline_table_* (CLASS, absent from the reference tree): the cubic
 *   spline with natural or estimated (3-point) end derivatives.
 * Third-party pieces restated from their published algorithms: the spherical
 * Bessel functions (CLASS bessel_j; here Miller's downward recurrence in long
 * double), the 3j symbols (SLATEC drc3jj; here the Racah formula), CLASS's l
 * list (transfer_get_l_list).  Parity with the reference itself is unpinned
 * (the reference needs CLASS, which is absent); the Bessel functions and 3j
 * symbols are pinned by the tests against scipy and sympy.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "song2.h"

#define O_PI 3.141592653589793238462643383279502884

/* ------------------------------------------------------------ helpers */

static void o_lin_space(double *out, double a, double b, int n) {
  for (int i = 0; i < n; ++i) out[i] = a + i * (b - a) / (n - 1);
}

static double o_lf(int n) { return lgamma((double)n + 1.0); }

/* Wigner 3j by the Racah formula (log-factorials) */
double song2_oracle_wigner3j(int j1, int j2, int j3, int m1, int m2, int m3) {
  if (m1 + m2 + m3 != 0) return 0.0;
  if (j3 < abs(j1 - j2) || j3 > j1 + j2) return 0.0;
  if (abs(m1) > j1 || abs(m2) > j2 || abs(m3) > j3) return 0.0;
  double pre = 0.5 * (o_lf(j1 + j2 - j3) + o_lf(j1 - j2 + j3) + o_lf(-j1 + j2 + j3) - o_lf(j1 + j2 + j3 + 1) +
                      o_lf(j1 + m1) + o_lf(j1 - m1) + o_lf(j2 + m2) + o_lf(j2 - m2) + o_lf(j3 + m3) + o_lf(j3 - m3));
  int tmin = 0;
  if (j2 - j3 - m1 > tmin) tmin = j2 - j3 - m1;
  if (j1 - j3 + m2 > tmin) tmin = j1 - j3 + m2;
  int tmax = j1 + j2 - j3;
  if (j1 - m1 < tmax) tmax = j1 - m1;
  if (j2 + m2 < tmax) tmax = j2 + m2;
  double sum = 0.0;
  for (int t = tmin; t <= tmax; ++t) {
    double v = exp(pre - (o_lf(t) + o_lf(j3 - j2 + t + m1) + o_lf(j3 - j1 + t - m2) + o_lf(j1 + j2 - j3 - t) +
                          o_lf(j1 - t - m1) + o_lf(j2 - t + m2)));
    sum += (t % 2 ? -v : v);
  }
  return ((j1 - j2 - m3) % 2 != 0) ? -sum : sum;
}

/* j_l(x) for l = 0..lmax by downward recurrence in long double from well above
   max(lmax, x), normalised to j_0 or j_1; the stored values are rescaled
   together whenever the recurrence nears the top of the long double range. */
void song2_oracle_bessel_all(double x, int lmax, double *out) {
  if (x == 0.0) {
    for (int l = 0; l <= lmax; ++l) out[l] = (l == 0);
    return;
  }
  double m = x > lmax ? x : lmax;
  int top = (int)(m + 40.0 + 2.5 * sqrt(m));
  long double *f = (long double *)malloc(sizeof(long double) * (top + 2));
  long double X = x;
  f[top + 1] = 0.0L;
  f[top] = 1e-30L;
  for (int l = top; l > 0; --l) {
    f[l - 1] = (2.0L * l + 1.0L) / X * f[l] - f[l + 1];
    if (fabsl(f[l - 1]) > 1e4000L)
      for (int j = l - 1; j <= top; ++j) f[j] *= 1e-4000L;
  }
  long double s = sinl(X), c = cosl(X), j0 = s / X, j1;
  if (x < 0.05) {
    long double x2 = X * X;
    j1 = X / 3.0L * (1.0L - x2 / 10.0L * (1.0L - x2 / 28.0L * (1.0L - x2 / 54.0L * (1.0L - x2 / 88.0L))));
  } else {
    j1 = (s / X - c) / X;
  }
  long double norm = (fabsl(j0) >= fabsl(j1)) ? j0 / f[0] : j1 / f[1];
  for (int l = 0; l <= lmax; ++l) out[l] = (double)(f[l] * norm);
  free(f);
}

static double o_bessel(int l, double x) {
  double *buf = (double *)malloc(sizeof(double) * (l + 1));
  song2_oracle_bessel_all(x, l, buf);
  double v = buf[l];
  free(buf);
  return v;
}

/* cubic spline second derivatives on x[0..n-1] (stride-1 y), natural (est = 0)
   or with end derivatives estimated from the parabola through three points */
static void o_spline(const double *x, const double *y, int n, int est, double *y2) {
  double *u = (double *)malloc(sizeof(double) * n);
  if (est) {
    double dy = ((x[2] - x[0]) * (x[2] - x[0]) * (y[1] - y[0]) - (x[1] - x[0]) * (x[1] - x[0]) * (y[2] - y[0])) /
                ((x[2] - x[0]) * (x[1] - x[0]) * (x[2] - x[1]));
    y2[0] = -0.5;
    u[0] = (3. / (x[1] - x[0])) * ((y[1] - y[0]) / (x[1] - x[0]) - dy);
  } else {
    y2[0] = u[0] = 0.0;
  }
  for (int i = 1; i < n - 1; ++i) {
    double sig = (x[i] - x[i - 1]) / (x[i + 1] - x[i - 1]);
    double p = sig * y2[i - 1] + 2.0;
    y2[i] = (sig - 1.0) / p;
    u[i] = (y[i + 1] - y[i]) / (x[i + 1] - x[i]) - (y[i] - y[i - 1]) / (x[i] - x[i - 1]);
    u[i] = (6.0 * u[i] / (x[i + 1] - x[i - 1]) - sig * u[i - 1]) / p;
  }
  double qn, un;
  if (est) {
    double a = x[n - 3], b = x[n - 2], c = x[n - 1];
    double dy = ((a - c) * (a - c) * (y[n - 2] - y[n - 1]) - (b - c) * (b - c) * (y[n - 3] - y[n - 1])) /
                ((a - c) * (b - c) * (a - b));
    qn = 0.5;
    un = (3. / (c - b)) * (dy - (y[n - 1] - y[n - 2]) / (c - b));
  } else {
    qn = un = 0.0;
  }
  y2[n - 1] = (un - qn * u[n - 2]) / (qn * y2[n - 2] + 1.0);
  for (int k = n - 2; k >= 0; --k) y2[k] = y2[k] * y2[k + 1] + u[k];
  free(u);
}

/* ------------------------------------------------------------ l list */

int song2_oracle_l_list(int l_max, double l_logstep, int l_linstep, int *out) {
  int n = 0, l = 2;
  if (l_max < 2) {
    out[0] = l_max;
    return 1;
  }
  out[n++] = l;
  int inc = (int)(l * (l_logstep - 1.));
  if (inc < 1) inc = 1;
  while ((l + inc) < l_max && inc < l_linstep) {
    l += inc;
    out[n++] = l;
    inc = (int)(l * (l_logstep - 1.));
    if (inc < 1) inc = 1;
  }
  inc = l_linstep;
  while ((l + inc) <= l_max) {
    l += inc;
    out[n++] = l;
  }
  if (l != l_max) out[n++] = l_max;
  return n;
}

/* ------------------------------------------------------ k3 transfer grid */

typedef struct {
  int size, phys_start, phys_size;
  double kmin, kmax, step;
} o_kgrid;

/* transfer2_get_k3_size */
static int o_k3_size(const song2_spec *s, const song2_los_spec *los, const double *k3, int kn, o_kgrid *g,
                     char *err) {
  double kmin_pt = k3[0], kmax_pt = k3[kn - 1];
  double kmin_tr = kmin_pt, kmax_tr = kmax_pt;
  if (los->k3_extrapolation != SONG2_K3_EXTRAP_NONE) {
    double phys = kmax_pt - kmin_pt;
    double ext_r = 2. * O_PI * los->extra_k3_oscillations_right / (los->tau0 - los->tau_rec);
    double ext_l = 2. * O_PI * los->extra_k3_oscillations_left / (los->tau0 - los->tau_rec);
    if (phys < ext_r) kmax_tr += (ext_r - phys);
    kmax_tr = fmin(kmax_tr, s->k[s->k_size - 1]);
    if (phys < ext_l) kmin_tr -= (ext_l - phys);
    kmin_tr = fmax(kmin_tr, fmin(s->k[0], kmin_pt));
    if (los->extra_k3_oscillations_left < 0) kmin_tr = s->k[0];
    if (los->extra_k3_oscillations_right < 0) kmax_tr = s->k[s->k_size - 1];
  }
  g->kmin = kmin_tr;
  g->kmax = kmax_tr;
  if (kmax_tr > los->x_max / los->tau0) {
    snprintf(err, SONG2_ERRLEN, "x_max too small for k_max=%g", kmax_tr);
    return 1;
  }
  double step = (los->k3_sampling == SONG2_K3_SAMPLING_CLASS) ? 2. * O_PI / (los->tau0 - los->tau_rec) * los->q_linstep
                                                              : los->x_step / los->tau0;
  g->step = step;
  int ipt = 0, itr = 0;
  double k = kmin_tr;
  itr++;
  if (los->k3_extrapolation != SONG2_K3_EXTRAP_NONE) {
    while (k < kmin_pt) {
      k += step;
      itr++;
    }
    if (k != kmin_pt) k = kmin_pt;
  }
  ipt++;
  g->phys_start = itr - 1;
  while (ipt < kn && (k3[ipt] - k) < step) {
    k = k3[ipt];
    ipt++;
    itr++;
  }
  g->phys_size = ipt;
  while (k < kmax_tr) {
    k += step;
    itr++;
    if (k <= kmax_pt && k >= kmin_pt) g->phys_size++;
  }
  g->size = (k > kmax_tr) ? itr - 1 : itr;
  if (g->size < 2) {
    snprintf(err, SONG2_ERRLEN, "fewer than 2 transfer k values");
    return 1;
  }
  return 0;
}

/* transfer2_get_k3_list */
static void o_k3_list(const song2_los_spec *los, const double *k3, int kn, const o_kgrid *g, double *out) {
  double kmin_pt = k3[0];
  int ipt = 0, itr = 0;
  double k = g->kmin;
  out[0] = g->kmin;
  itr++;
  if (los->k3_extrapolation != SONG2_K3_EXTRAP_NONE) {
    while (k < kmin_pt) {
      k += g->step;
      out[itr] = k;
      itr++;
    }
    if (k != kmin_pt) {
      k = kmin_pt;
      out[itr - 1] = k;
    }
  }
  ipt++;
  while (ipt < kn && (k3[ipt] - k) < g->step) {
    k = k3[ipt];
    out[itr] = k;
    ipt++;
    itr++;
  }
  while (itr < g->size && k < g->kmax) {
    k += g->step;
    out[itr] = k;
    itr++;
  }
}

int64_t song2_oracle_transfer_k_grids(const song2_spec *s, const song2_los_spec *los, int *sizes, int *pstart,
                                      int *psize, double *k_out, char *err) {
  int64_t tot = 0, off = 0;
  int p = 0;
  for (int i1 = 0; i1 < s->k_size; ++i1)
    for (int i2 = 0; i2 <= i1; ++i2, ++p) {
      int kn = s->k3_size[i1 * s->k_size + i2];
      o_kgrid g;
      if (o_k3_size(s, los, s->k3 + off, kn, &g, err)) return -1;
      if (sizes) sizes[p] = g.size;
      if (pstart) pstart[p] = g.phys_start;
      if (psize) psize[p] = g.phys_size;
      if (k_out) o_k3_list(los, s->k3 + off, kn, &g, k_out + tot);
      tot += g.size;
      off += kn;
    }
  return tot;
}

/* ----------------------------------------------------------- tables */

typedef struct {
  int x_size;
  double *xx;
  int L_size, m_size, l_size, n_rows, n_l1;
  int *l1, *l1_index, *jxmin, *jneg;
  double **j;       /* [n_l1][x_size - jxmin] */
  double *J;        /* [n_rows][x_size], zero below the row's x_min */
  double *ddJ;      /* cubic */
  int *Jxmin;
} o_tables;

static int o_index_m_max(const song2_spec *s, int l) {
  int im = -1;
  for (int i = 0; i < s->m_size; ++i)
    if (s->m[i] <= l) im = i;
  return im;
}

/* bessel2_j_for_l1: x_min by bisection and the storage of j_l1 from there on
   (the values themselves are filled x by x, one recurrence per x, in
   o_fill_j) */
static void o_j_for_l1(const song2_los_spec *los, o_tables *t, int r) {
  int l1 = t->l1[r];
  double x_min;
  if (l1 == 0) {
    x_min = 0;
    t->jxmin[r] = 0;
  } else {
    double down = 0, up = l1 + 0.5;
    while ((up - down) / down > los->bessel_tol_x_min) {
      if ((up - down) < 1e-16) {
        x_min = up = down;
        break;
      }
      double j = o_bessel(l1, 0.5 * (up + down));
      if (j >= los->j_cut) up = 0.5 * (up + down);
      else down = 0.5 * (up + down);
    }
    x_min = down;
    if (x_min < los->x_max) {
      t->jxmin[r] = 0;
      while (t->xx[t->jxmin[r]] < x_min) t->jxmin[r]++;
      if (t->jxmin[r] != 0) --t->jxmin[r];
    }
  }
  int n;
  if (x_min >= los->x_max) {
    t->jxmin[r] = t->x_size - 1;
    n = 1;
    t->j[r] = (double *)calloc(1, sizeof(double));
    t->jneg[r] = 1;
    return;
  }
  n = t->x_size - t->jxmin[r];
  t->j[r] = (double *)malloc(sizeof(double) * n);
}

static void o_fill_j(const song2_los_spec *los, o_tables *t) {
  int lmax = t->l1[t->n_l1 - 1];
#pragma omp parallel
  {
    double *buf = (double *)malloc(sizeof(double) * (lmax + 1));
#pragma omp for schedule(dynamic, 16)
    for (int i = 0; i < t->x_size; ++i) {
      song2_oracle_bessel_all(t->xx[i], lmax, buf);
      for (int r = 0; r < t->n_l1; ++r) {
        int ij = i - t->jxmin[r];
        if (ij < 0) continue;
        if (t->jneg[r]) continue;  /* negligible everywhere: the single stored value stays zero */
        t->j[r][ij] = buf[t->l1[r]];
      }
    }
    free(buf);
  }
  (void)los;
}

/* bessel2_J_Llm at one x index */
static double o_J_Llm(const o_tables *t, int Jt, int L, int l, int m, int ix, const double *f1, const double *f2,
                      int lo, int n) {
  double J = 0;
  for (int i = 0; i < n; ++i) {
    if (f1[i] == 0) continue;
    int l1 = lo + i;
    int r = t->l1_index[l1];
    int ixj = ix - t->jxmin[r];
    if (ixj < 0) continue;
    int even = ((l - l1 - L) % 2 == 0);
    double pref;
    if (Jt != 2) {
      if (!even) continue;
      pref = (((l - l1 - L) / 2) % 2 == 0) ? 1 : -1;
    } else {
      if (even) continue;
      pref = (((l - l1 - L - 1) / 2) % 2 == 0) ? 1 : -1;
    }
    J += pref * (2 * l1 + 1) * f1[i] * f2[i] * t->j[r][ixj];
  }
  J *= ((m % 2 == 0) ? 1 : -1) * (2 * l + 1);
  return J;
}

static int o_build_tables(const song2_spec *s, const song2_los_spec *los, o_tables *t, char *err) {
  memset(t, 0, sizeof(*t));
  double x_max = los->x_max;
  t->x_size = (int)(x_max / los->x_step + 1);
  t->xx = (double *)malloc(sizeof(double) * t->x_size);
  o_lin_space(t->xx, 0, x_max, t->x_size);
  int m_max = 0;
  for (int i = 0; i < s->m_size; ++i)
    if (s->m[i] > m_max) m_max = s->m[i];
  int l_los = 0;
  if (s->has_source_T && s->l_max_los_t > l_los) l_los = s->l_max_los_t;
  if ((s->has_source_E || s->has_source_B) && s->l_max_los_p > l_los) l_los = s->l_max_los_p;
  int L_max = l_los > m_max ? l_los : m_max;
  t->L_size = L_max + 1;
  t->m_size = s->m_size;
  t->l_size = los->l_size;
  t->n_rows = 3 * t->L_size * t->l_size * t->m_size;
  /* l1 list */
  int Lx = L_max + m_max;
  int top = los->l[los->l_size - 1] + Lx;
  t->l1 = (int *)malloc(sizeof(int) * (top + 1));
  t->l1_index = (int *)malloc(sizeof(int) * (top + 1));
  t->n_l1 = 0;
  for (int l1 = 0; l1 <= top; ++l1) {
    int keep = 0;
    for (int i = 0; i < los->l_size; ++i)
      if (l1 >= los->l[i] - Lx && l1 <= los->l[i] + Lx) keep = 1;
    t->l1_index[l1] = keep ? t->n_l1 : -1;
    if (keep) t->l1[t->n_l1++] = l1;
  }
  t->jxmin = (int *)calloc(t->n_l1, sizeof(int));
  t->jneg = (int *)calloc(t->n_l1, sizeof(int));
  t->j = (double **)calloc(t->n_l1, sizeof(double *));
#pragma omp parallel for schedule(dynamic)
  for (int r = 0; r < t->n_l1; ++r) o_j_for_l1(los, t, r);
  o_fill_j(los, t);
  /* projection rows */
  t->J = (double *)calloc((size_t)t->n_rows * t->x_size, sizeof(double));
  t->Jxmin = (int *)malloc(sizeof(int) * t->n_rows);
  int needT = s->has_source_T, needP = s->has_source_E || s->has_source_B;
  int bad = 0;
#pragma omp parallel for schedule(dynamic) collapse(2)
  for (int Jt = 0; Jt < 3; ++Jt)
    for (int L = 0; L < t->L_size; ++L)
      for (int il = 0; il < t->l_size; ++il)
        for (int im = 0; im < t->m_size; ++im) {
          int row = ((Jt * t->L_size + L) * t->l_size + il) * t->m_size + im;
          int l = los->l[il], m = s->m[im];
          int S = Jt == 0 ? 0 : 2;
          int needed = Jt == 0 ? needT : (needP && (Jt == 1 || m_max > 0));
          double *Jr = t->J + (size_t)row * t->x_size;
          t->Jxmin[row] = t->x_size - 1;
          if (!needed || m > (L < l ? L : l) || S > l || S > L || (Jt == 2 && m == 0)) continue;
          int lo = abs(L - l), hi = L + l, n = hi - lo + 1;
          double f1[64], f2[64];
          for (int i = 0; i < n; ++i) {
            f1[i] = song2_oracle_wigner3j(lo + i, L, l, 0, S, -S);
            f2[i] = song2_oracle_wigner3j(lo + i, L, l, 0, -m, m);
          }
          int xmin;
          if (L == l) {
            xmin = 0;
          } else {
            double xu = lo + 0.5;
            int up;
            if (xu >= los->x_max) {
              up = t->x_size - 1;
              xu = los->x_max;
            } else {
              up = 0;
              while (t->xx[up] < xu) up++;
              xu = t->xx[up];
            }
            double J = o_J_Llm(t, Jt, L, l, m, up, f1, f2, lo, n);
            if (fabs(J) < los->J_cut) {
              if (xu < los->x_max) bad = 1;
              continue;
            }
            int down = 0;
            while (down != up - 1) {
              int mid = (up + down) / 2;
              J = o_J_Llm(t, Jt, L, l, m, mid, f1, f2, lo, n);
              if (fabs(J) >= los->J_cut) up = mid;
              else down = mid;
            }
            xmin = down;
          }
          t->Jxmin[row] = xmin;
          for (int ix = xmin; ix < t->x_size; ++ix) Jr[ix] = o_J_Llm(t, Jt, L, l, m, ix, f1, f2, lo, n);
        }
  if (bad) {
    snprintf(err, SONG2_ERRLEN, "projection function negligible at its first peak");
    return 1;
  }
  if (los->bessel_interpolation == SONG2_INTERP_CUBIC) {
    t->ddJ = (double *)calloc((size_t)t->n_rows * t->x_size, sizeof(double));
#pragma omp parallel for schedule(dynamic)
    for (int row = 0; row < t->n_rows; ++row) {
      int x0 = t->Jxmin[row], n = t->x_size - x0;
      int il = (row / t->m_size) % t->l_size;
      if (n >= 3)
        o_spline(t->xx + x0, t->J + (size_t)row * t->x_size + x0, n, los->l[il] == 2,
                 t->ddJ + (size_t)row * t->x_size + x0);
    }
  }
  return 0;
}

static void o_free_tables(o_tables *t) {
  if (t->j)
    for (int r = 0; r < t->n_l1; ++r) free(t->j[r]);
  free(t->j);
  free(t->xx);
  free(t->l1);
  free(t->l1_index);
  free(t->jxmin);
  free(t->jneg);
  free(t->J);
  free(t->ddJ);
  free(t->Jxmin);
}

int song2_oracle_los_table_sizes(const song2_spec *s, const song2_los_spec *los, int *x_size, int *n_l1,
                                 int *n_rows) {
  char err[SONG2_ERRLEN];
  o_tables t;
  if (o_build_tables(s, los, &t, err)) return 1;
  *x_size = t.x_size;
  *n_l1 = t.n_l1;
  *n_rows = t.n_rows;
  o_free_tables(&t);
  return 0;
}

/* The tables in the product's full-row layout: j_l1 [n_l1][x_size] (zero below
   the l1's x_min), J [n_rows][x_size] (zero below the row's x_min). */
int song2_oracle_los_tables(const song2_spec *s, const song2_los_spec *los, int *l1, double *jtab, double *J,
                            int *Jxmin, char *err) {
  o_tables t;
  if (o_build_tables(s, los, &t, err)) return 1;
  for (int r = 0; r < t.n_l1; ++r) {
    l1[r] = t.l1[r];
    for (int i = 0; i < t.x_size; ++i) {
      int ij = i - t.jxmin[r];
      jtab[(size_t)r * t.x_size + i] = (ij >= 0 && (t.jxmin[r] < t.x_size - 1 || ij == 0)) ? t.j[r][ij] : 0.0;
    }
  }
  memcpy(J, t.J, sizeof(double) * (size_t)t.n_rows * t.x_size);
  memcpy(Jxmin, t.Jxmin, sizeof(int) * t.n_rows);
  o_free_tables(&t);
  return 0;
}

/* --------------------------------------------------------- transfers */

static int o_lm(const song2_spec *s, int L, int im) {
  int n = 0;
  for (int l = 0; l < L; ++l)
    for (int i = 0; i < s->m_size; ++i)
      if (s->m[i] <= l) ++n;
  return n + im;
}

/* Transfers of the pairs pair_lo <= p < pair_hi (pair order: k1 ascending,
   k2 <= k1); the other pairs' entries of out are left untouched.  The tables
   are built first (their time is not separable from the call). */
int song2_oracle_transfer_pairs(const song2_spec *s, const song2_los_spec *los, const double *sources, double *out,
                                int pair_lo, int pair_hi, int nthreads, char *err) {
  o_tables t;
  if (o_build_tables(s, los, &t, err)) return 1;
  int n_pairs = s->k_size * (s->k_size + 1) / 2;
  int *ksz = (int *)malloc(sizeof(int) * n_pairs), *kps = (int *)malloc(sizeof(int) * n_pairs),
      *kpn = (int *)malloc(sizeof(int) * n_pairs);
  int64_t nu = song2_oracle_transfer_k_grids(s, los, ksz, kps, kpn, NULL, err);
  if (nu < 0) {
    o_free_tables(&t);
    return 1;
  }
  double *kall = (double *)malloc(sizeof(double) * nu);
  song2_oracle_transfer_k_grids(s, los, NULL, NULL, NULL, kall, err);
  /* source type blocks */
  int base_T = 0, base_E = 0, base_B = 0, b = 0;
  if (s->has_source_T) {
    base_T = b;
    b += o_lm(s, s->l_max_los_t + 1, 0);
  }
  if (s->has_source_E) {
    base_E = b;
    b += o_lm(s, s->l_max_los_p + 1, 0);
  }
  if (s->has_source_B) {
    base_B = b;
    b += o_lm(s, s->l_max_los_p + 1, 0);
  }
  /* transfer types: T, E, B x (index_l, index_m), l major */
  int n_tt = 0;
  int has[3] = {s->has_source_T, s->has_source_E, s->has_source_B};
  for (int ty = 0; ty < 3; ++ty)
    if (has[ty])
      for (int il = 0; il < los->l_size; ++il) n_tt += o_index_m_max(s, los->l[il]) + 1;
  int *tt_ty = (int *)malloc(sizeof(int) * n_tt), *tt_il = (int *)malloc(sizeof(int) * n_tt),
      *tt_im = (int *)malloc(sizeof(int) * n_tt);
  {
    int o = 0;
    for (int ty = 0; ty < 3; ++ty)
      if (has[ty])
        for (int il = 0; il < los->l_size; ++il)
          for (int im = 0; im <= o_index_m_max(s, los->l[il]); ++im) {
            tt_ty[o] = ty;
            tt_il[o] = il;
            tt_im[o] = im;
            ++o;
          }
  }
  int tp2 = song2_tp2_size(s);
  int64_t per_type = song2_sources_per_type(s);
  int ts = s->tau_size;
  const double *tau_pt = s->tau;
  /* pair offsets */
  int64_t *src_off = (int64_t *)malloc(sizeof(int64_t) * n_pairs), *k3_off = (int64_t *)malloc(sizeof(int64_t) * n_pairs),
          *u_off = (int64_t *)malloc(sizeof(int64_t) * n_pairs);
  {
    int64_t so = 0, ko = 0, uo = 0;
    int p = 0;
    for (int i1 = 0; i1 < s->k_size; ++i1)
      for (int i2 = 0; i2 <= i1; ++i2, ++p) {
        int kn = s->k3_size[i1 * s->k_size + i2];
        src_off[p] = so;
        k3_off[p] = ko;
        u_off[p] = uo;
        so += (int64_t)ts * kn;
        ko += kn;
        uo += ksz[p];
      }
  }
  double x_step = los->x_step;
  int L_T = s->l_max_los_t, L_P = s->l_max_los_p;
#pragma omp parallel for schedule(dynamic) num_threads(nthreads > 0 ? nthreads : 1)
  for (int p = pair_lo; p < (pair_hi < n_pairs ? pair_hi : n_pairs); ++p) {
    int kn = 0;
    {
      int q = 0;
      for (int i1 = 0; i1 < s->k_size; ++i1)
        for (int i2 = 0; i2 <= i1; ++i2, ++q)
          if (q == p) kn = s->k3_size[i1 * s->k_size + i2];
    }
    const double *kpt = s->k3 + k3_off[p];
    int n_k = ksz[p];
    const double *ktr = kall + u_off[p];
    /* interpolation in k for every source type (transfer2_interpolate_sources_in_k) */
    double *sk = (double *)calloc((size_t)tp2 * n_k * ts, sizeof(double)); /* [tp][k][tau] */
    double *spl = (double *)malloc(sizeof(double) * (size_t)ts * kn);
    double *col = (double *)malloc(sizeof(double) * kn), *colspl = (double *)malloc(sizeof(double) * kn);
    for (int tp = 0; tp < tp2; ++tp) {
      const double *S = sources + (int64_t)tp * per_type + src_off[p];
      if (los->k3_interpolation == SONG2_INTERP_CUBIC)
        for (int it = 0; it < ts; ++it) {
          for (int j = 0; j < kn; ++j) col[j] = S[it * kn + j];
          o_spline(kpt, col, kn, 1, colspl);
          for (int j = 0; j < kn; ++j) spl[it * kn + j] = colspl[j];
        }
      int first = kps[p], last = kps[p] + kpn[p] - 1;
      int ik = 0;
      double h = kpt[1] - kpt[0];
      for (int itr = first; itr <= last; ++itr) {
        while (ik + 1 < kn && kpt[ik + 1] < ktr[itr]) {
          ik++;
          h = kpt[ik + 1] - kpt[ik];
        }
        double bb = (ktr[itr] - kpt[ik]) / h, aa = 1 - bb;
        for (int it = 0; it < ts; ++it) {
          double v = aa * S[it * kn + ik] + bb * S[it * kn + ik + 1];
          if (los->k3_interpolation == SONG2_INTERP_CUBIC)
            v += ((aa * aa * aa - aa) * spl[it * kn + ik] + (bb * bb * bb - bb) * spl[it * kn + ik + 1]) * h * h / 6.0;
          sk[((size_t)tp * n_k + itr) * ts + it] = v;
        }
      }
      if (los->k3_extrapolation == SONG2_K3_EXTRAP_FLAT) {
        for (int itr = last + 1; itr < n_k; ++itr)
          for (int it = 0; it < ts; ++it) sk[((size_t)tp * n_k + itr) * ts + it] = sk[((size_t)tp * n_k + last) * ts + it];
        for (int itr = 0; itr < first; ++itr)
          for (int it = 0; it < ts; ++it) sk[((size_t)tp * n_k + itr) * ts + it] = sk[((size_t)tp * n_k + first) * ts + it];
      }
    }
    free(col);
    free(colspl);
    free(spl);
    /* per k */
    for (int ik = 0; ik < n_k; ++ik) {
      double k = ktr[ik];
      /* time grid (transfer2_get_time_grid) */
      int G;
      double *grid, *dtau;
      int *left;
      if (los->tau_sampling == SONG2_TAU_SAMPLING_SOURCES) {
        G = ts;
        grid = (double *)malloc(sizeof(double) * G);
        left = (int *)malloc(sizeof(int) * G);
        for (int i = 0; i < G; ++i) {
          grid[i] = tau_pt[i];
          left[i] = i;
        }
      } else {
        double step = (los->tau_sampling == SONG2_TAU_SAMPLING_CUSTOM) ? 2 * O_PI / k * los->tau_linstep : x_step / k;
        int itr = 0, ipt = 0;
        double tau = tau_pt[0];
        itr++;
        ipt++;
        while (ipt < ts) {
          while ((tau_pt[ipt] - tau) > step) {
            tau += step;
            itr++;
          }
          tau = tau_pt[ipt];
          ++itr;
          ++ipt;
        }
        G = itr;
        grid = (double *)malloc(sizeof(double) * G);
        left = (int *)malloc(sizeof(int) * G);
        itr = ipt = 0;
        tau = tau_pt[0];
        grid[0] = tau;
        itr++;
        ipt++;
        left[0] = 0;
        while (ipt < ts) {
          while ((tau_pt[ipt] - tau) > step) {
            tau += step;
            grid[itr] = tau;
            left[itr] = ipt;
            itr++;
          }
          tau = tau_pt[ipt];
          grid[itr] = tau;
          left[itr] = ipt;
          itr++;
          ipt++;
        }
        for (int i = 0; i < G; ++i)
          if (left[i] == ts - 1) left[i] = ts - 2;
      }
      dtau = (double *)malloc(sizeof(double) * G);
      dtau[0] = grid[1] - grid[0];
      for (int i = 1; i < G - 1; ++i) dtau[i] = grid[i + 1] - grid[i - 1];
      dtau[G - 1] = grid[G - 1] - grid[G - 2];
      /* sources at the grid times (transfer2_interpolate_sources_in_time) */
      double *st = (double *)malloc(sizeof(double) * (size_t)tp2 * G);
      double *tspl = (double *)malloc(sizeof(double) * ts);
      for (int tp = 0; tp < tp2; ++tp) {
        const double *row = sk + ((size_t)tp * n_k + ik) * ts;
        if (los->tau_sampling == SONG2_TAU_SAMPLING_SOURCES) {
          for (int i = 0; i < G; ++i) st[(size_t)tp * G + i] = row[i];
          continue;
        }
        if (los->time_interpolation == SONG2_INTERP_CUBIC) o_spline(tau_pt, row, ts, 1, tspl);
        for (int i = 0; i < G; ++i) {
          int it = left[i];
          double hh = tau_pt[it + 1] - tau_pt[it];
          double bb = (grid[i] - tau_pt[it]) / hh, aa = 1 - bb;
          double v = aa * row[it] + bb * row[it + 1];
          if (los->time_interpolation == SONG2_INTERP_CUBIC)
            v += ((aa * aa * aa - aa) * tspl[it] + (bb * bb * bb - bb) * tspl[it + 1]) * hh * hh / 6.0;
          st[(size_t)tp * G + i] = v;
        }
      }
      free(tspl);
      /* transfer2_compute / transfer2_integrate for every type */
      for (int o = 0; o < n_tt; ++o) {
        int ty = tt_ty[o], il = tt_il[o], im = tt_im[o];
        int l = los->l[il], m = s->m[im];
        /* (J, source base, sign) pieces */
        int nq = 0, Jq[2], Bq[2];
        double Sq[2];
        int Lmax;
        if (ty == 0) {
          Lmax = L_T;
          Jq[0] = 0; Bq[0] = base_T; Sq[0] = 1; nq = 1;
        } else if (ty == 1) {
          Lmax = L_P;
          Jq[0] = 1; Bq[0] = base_E; Sq[0] = 1; nq = 1;
          if (m != 0 && s->has_source_B) { Jq[1] = 2; Bq[1] = base_B; Sq[1] = 1; nq = 2; }
        } else {
          Lmax = L_P;
          Jq[0] = 1; Bq[0] = base_B; Sq[0] = 1; nq = 1;
          if (s->has_source_E) { Jq[1] = 2; Bq[1] = base_E; Sq[1] = -1; nq = 2; }
        }
        double contrib[2] = {0, 0};
        for (int q = 0; q < nq; ++q) {
          double integral = 0;
          for (int i = 0; i < G; ++i) {
            double x = k * (los->tau0 - grid[i]);
            int ix = (int)(x / x_step);
            double aJ = (t.xx[ix + 1] - x) / x_step;
            double integrand = 0;
            for (int L = 0; L <= Lmax; ++L) {
              if (m > (L < l ? L : l)) continue;
              int row = ((Jq[q] * t.L_size + L) * t.l_size + il) * t.m_size + im;
              int xmin = t.Jxmin[row];
              if (ix < xmin) continue;
              const double *Jr = t.J + (size_t)row * t.x_size;
              double Jv;
              if (los->bessel_interpolation == SONG2_INTERP_LINEAR) {
                Jv = aJ * Jr[ix] + (1 - aJ) * Jr[ix + 1];
              } else {
                const double *dd = t.ddJ + (size_t)row * t.x_size;
                Jv = (aJ * Jr[ix] + (1. - aJ) * (Jr[ix + 1] - aJ * ((aJ + 1.) * dd[ix] + (2. - aJ) * dd[ix + 1]) *
                                                                    x_step * x_step / 6.0));
              }
              int tp = Bq[q] + o_lm(s, L, im);
              integrand += Jv * st[(size_t)tp * G + i];
            }
            integral += integrand * dtau[i];
          }
          contrib[q] = integral * 0.5;
        }
        double tr = (nq == 2) ? (Sq[1] < 0 ? contrib[0] - contrib[1] : contrib[0] + contrib[1]) : contrib[0];
        tr /= 4.;
        tr /= (2. * l + 1);
        tr /= 2.;
        out[(int64_t)o * nu + u_off[p] + ik] = tr;
      }
      free(st);
      free(grid);
      free(left);
      free(dtau);
    }
    free(sk);
  }
  free(ksz);
  free(kps);
  free(kpn);
  free(kall);
  free(tt_ty);
  free(tt_il);
  free(tt_im);
  free(src_off);
  free(k3_off);
  free(u_off);
  o_free_tables(&t);
  return 0;
}

int song2_oracle_transfer(const song2_spec *s, const song2_los_spec *los, const double *sources, double *out,
                          int nthreads, char *err) {
  return song2_oracle_transfer_pairs(s, los, sources, out, 0, 1 << 30, nthreads, err);
}

/* ================================================== intrinsic bispectrum
   bispectra2_intrinsic_init and its integrals, in the reference's order
   (bispectra2.c:300-3030): for each second-order field X, M3 of the m list
   and parity-allowed offset_L3, the k3 integral on every (l3, r, k1, k2 <= k1)
   (bispectra2_intrinsic_integrate_over_k3, :1107-1447); for each field Y the
   interpolation of I_l3 in k2 onto q (bispectra2_interpolate_over_k2,
   :1448-1612) and its Bessel convolution with T1_l2 (:1613-1849); for each
   even offset_L1 and field Z the interpolation in k1 (:1850-1994), the
   convolution with T1_l1 (:1995-2292), the r integral (:2293-2455) and the
   geometrical factors (:2456-2880); then the symmetrisation (:760-790).
   The first-order convolution uses the same Bessel table (CLASS's bessel
   module is absent from the reference tree).  3j and 6j symbols by Racah's
   formulas in long double (the reference calls SLATEC's drc3jj/drc6j). */

static long double o_lfl(int n) { return lgammal((long double)n + 1.0L); }

static int o_tri(int a, int b, int c) { return c >= abs(a - b) && c <= a + b; }

static long double o_w3j000(int a, int b, int c) {
  if (!o_tri(a, b, c)) return 0;
  int J = a + b + c;
  if (J % 2) return 0;
  int g = J / 2;
  long double v = expl(0.5L * (o_lfl(J - 2 * a) + o_lfl(J - 2 * b) + o_lfl(J - 2 * c) - o_lfl(J + 1)) + o_lfl(g) -
                       o_lfl(g - a) - o_lfl(g - b) - o_lfl(g - c));
  return (g % 2) ? -v : v;
}

static long double o_w3j(int j1, int j2, int j3, int m1, int m2, int m3) {
  if (m1 + m2 + m3 != 0 || !o_tri(j1, j2, j3) || abs(m1) > j1 || abs(m2) > j2 || abs(m3) > j3) return 0;
  if (m1 == 0 && m2 == 0) return o_w3j000(j1, j2, j3);
  long double pre = 0.5L * (o_lfl(j1 + j2 - j3) + o_lfl(j1 - j2 + j3) + o_lfl(-j1 + j2 + j3) -
                            o_lfl(j1 + j2 + j3 + 1) + o_lfl(j1 + m1) + o_lfl(j1 - m1) + o_lfl(j2 + m2) +
                            o_lfl(j2 - m2) + o_lfl(j3 + m3) + o_lfl(j3 - m3));
  int lo = 0, hi = j1 + j2 - j3;
  if (j2 - j3 - m1 > lo) lo = j2 - j3 - m1;
  if (j1 - j3 + m2 > lo) lo = j1 - j3 + m2;
  if (j1 - m1 < hi) hi = j1 - m1;
  if (j2 + m2 < hi) hi = j2 + m2;
  long double s = 0;
  for (int k = lo; k <= hi; ++k) {
    long double v = expl(pre - (o_lfl(k) + o_lfl(j3 - j2 + k + m1) + o_lfl(j3 - j1 + k - m2) +
                                o_lfl(j1 + j2 - j3 - k) + o_lfl(j1 - k - m1) + o_lfl(j2 - k + m2)));
    s += (k % 2) ? -v : v;
  }
  return ((j1 - j2 - m3) % 2) ? -s : s;
}

static long double o_ldelta(int a, int b, int c) {
  return o_lfl(a + b - c) + o_lfl(a - b + c) + o_lfl(-a + b + c) - o_lfl(a + b + c + 1);
}

/* {a b c; d e f} */
long double song2_oracle_wigner6j_l(int a, int b, int c, int d, int e, int f) {
  if (!o_tri(a, b, c) || !o_tri(a, e, f) || !o_tri(d, b, f) || !o_tri(d, e, c)) return 0;
  long double ld = 0.5L * (o_ldelta(a, b, c) + o_ldelta(a, e, f) + o_ldelta(d, b, f) + o_ldelta(d, e, c));
  int lo = a + b + c;
  if (a + e + f > lo) lo = a + e + f;
  if (d + b + f > lo) lo = d + b + f;
  if (d + e + c > lo) lo = d + e + c;
  int hi = a + b + d + e;
  if (b + c + e + f < hi) hi = b + c + e + f;
  if (c + a + f + d < hi) hi = c + a + f + d;
  long double s = 0;
  for (int t = lo; t <= hi; ++t) {
    long double v = expl(ld + o_lfl(t + 1) -
                         (o_lfl(t - a - b - c) + o_lfl(t - a - e - f) + o_lfl(t - d - b - f) + o_lfl(t - d - e - c) +
                          o_lfl(a + b + d + e - t) + o_lfl(b + c + e + f - t) + o_lfl(c + a + f + d - t)));
    s += (t % 2) ? -v : v;
  }
  return s;
}

double song2_oracle_wigner6j(int a, int b, int c, int d, int e, int f) {
  return (double)song2_oracle_wigner6j_l(a, b, c, d, e, f);
}

typedef struct {
  const o_tables *t;
  double x_step;
  double **ddj;  /* cubic */
  int cubic;
  int bad;
} o_bes;

/* bessel2_convolution (bessel2.c:499-600) */
static double o_convolve(o_bes *B, const double *kk, const double *dk, int n, const double *f, const double *g, int L,
                         double r) {
  const o_tables *t = B->t;
  int row = t->l1_index[L];
  double xmin = t->jneg[row] ? t->xx[t->x_size - 1] : t->xx[t->jxmin[row]];
  int nx = t->jneg[row] ? 1 : t->x_size - t->jxmin[row];
  double s = 0;
  for (int i = 0; i < n; ++i) {
    double fv = f[i];
    if (fv == 0.) continue;
    double gv = 1.;
    if (g) {
      gv = g[i];
      if (gv == 0.) continue;
    }
    double k = kk[i], x = k * r;
    if (x < xmin) continue;
    int ix = (int)((x - xmin) / B->x_step);
    if (ix + 1 >= nx) {
      B->bad = 1;
      continue;
    }
    double a = (xmin + B->x_step * (ix + 1) - x) / B->x_step;
    const double *jr = t->j[row];
    double j;
    if (!B->cubic) {
      j = a * jr[ix] + (1. - a) * jr[ix + 1];
    } else {
      const double *dd = B->ddj[row];
      j = a * jr[ix] + (1. - a) * (jr[ix + 1] - a * ((a + 1.) * dd[ix] + (2. - a) * dd[ix + 1]) * B->x_step *
                                                    B->x_step / 6.0);
    }
    s += k * k * j * fv * gv * dk[i];
  }
  return 0.5 * s;
}

static void o_trap(const double *x, int n, double *d) {
  d[0] = x[1] - x[0];
  for (int i = 1; i < n - 1; ++i) d[i] = x[i + 1] - x[i - 1];
  d[n - 1] = x[n - 1] - x[n - 2];
}

/* interpolation of f (times the window 1/k^2) from the k grid onto q, times q^2
   and P(q) (bispectra2_interpolate_over_k2/k1) */
static int o_interp_k(const double *k, int K, double *f, int cubic, const double *q, int Q, const double *pk,
                      double *out) {
  double *spl = NULL;
  if (cubic) {
    spl = (double *)malloc(sizeof(double) * K);
    o_spline(k, f, K, 1, spl);
  }
  int ik = 0;
  double h = k[1] - k[0];
  for (int iq = 0; iq < Q; ++iq) {
    while (ik + 1 < K && k[ik + 1] < q[iq]) {
      ik++;
      h = k[ik + 1] - k[ik];
    }
    if (ik + 1 >= K) {
      free(spl);
      return 1;
    }
    double b = (q[iq] - k[ik]) / h, a = 1. - b;
    double v = a * f[ik] + b * f[ik + 1];
    if (cubic) v += ((a * a * a - a) * spl[ik] + (b * b * b - b) * spl[ik + 1]) * h * h / 6.0;
    v *= q[iq] * q[iq];
    v *= pk[iq];
    out[iq] = v;
  }
  free(spl);
  return 0;
}

int song2_oracle_bispectra(const song2_spec *s, const song2_los_spec *los, const song2_bispectra_spec *bs,
                           const double *T2, double *out, char *err) {
  o_tables t;
  if (o_build_tables(s, los, &t, err)) return 1;
  o_bes B = {&t, los->x_step, NULL, los->bessel_interpolation == SONG2_INTERP_CUBIC, 0};
  if (B.cubic) {
    B.ddj = (double **)calloc(t.n_l1, sizeof(double *));
    for (int r = 0; r < t.n_l1; ++r) {
      int n = t.jneg[r] ? 1 : t.x_size - t.jxmin[r];
      B.ddj[r] = (double *)calloc(n, sizeof(double));
      if (n >= 3) o_spline(t.xx + t.jxmin[r], t.j[r], n, 0, B.ddj[r]);
    }
  }
  const int L = los->l_size, R = bs->r_size, Q = bs->q_size, K = s->k_size, bf = bs->bf_size;
  const int *l = los->l;
  int n_pairs = K * (K + 1) / 2;
  int *ksz = (int *)malloc(sizeof(int) * n_pairs);
  int64_t nu = song2_oracle_transfer_k_grids(s, los, ksz, NULL, NULL, NULL, err);
  double *kall = (double *)malloc(sizeof(double) * nu), *dkall = (double *)malloc(sizeof(double) * nu);
  song2_oracle_transfer_k_grids(s, los, NULL, NULL, NULL, kall, err);
  int64_t *uoff = (int64_t *)malloc(sizeof(int64_t) * n_pairs);
  {
    int64_t o = 0;
    for (int p = 0; p < n_pairs; ++p) {
      uoff[p] = o;
      o_trap(kall + o, ksz[p], dkall + o);
      o += ksz[p];
    }
  }
  /* transfer types: T, E, B blocks; (l, m <= l) inside (transfer2_get_lm_lists) */
  int has[3] = {s->has_source_T, s->has_source_E, s->has_source_B};
  int tt_base[3] = {0, 0, 0}, per_type = 0;
  for (int il = 0; il < L; ++il) per_type += o_index_m_max(s, l[il]) + 1;
  {
    int b = 0;
    for (int f = 0; f < 3; ++f)
      if (has[f]) {
        tt_base[f] = b;
        b += per_type;
      }
  }
  int *lm_off = (int *)malloc(sizeof(int) * L);
  {
    int o = 0;
    for (int il = 0; il < L; ++il) {
      lm_off[il] = o;
      o += o_index_m_max(s, l[il]) + 1;
    }
  }
  /* triangles */
  int *tmin = (int *)malloc(sizeof(int) * L * L), *tmax = (int *)malloc(sizeof(int) * L * L);
  for (int a = 0; a < L; ++a)
    for (int b = 0; b < L; ++b) {
      int lo = 0, hi = L - 1;
      while (lo < L && l[lo] < abs(l[a] - l[b])) lo++;
      while (hi >= 0 && l[hi] > l[a] + l[b]) hi--;
      tmin[a * L + b] = lo;
      tmax[a * L + b] = hi;
    }
  /* grids */
  const double *kp = s->k, *q = bs->q, *r = bs->r;
  double *dq = (double *)malloc(sizeof(double) * Q), *dr = (double *)malloc(sizeof(double) * R);
  o_trap(q, Q, dq);
  o_trap(r, R, dr);
  int m_max = 0;
  for (int i = 0; i < s->m_size; ++i)
    if (s->m[i] > m_max) m_max = s->m[i];
  int fpar[3] = {0, 0, 1};
  int parity = (3 * fpar[bs->bf[bf - 1]]) % 2;  /* set once, from the last combination (bispectra2.c:967) */
  /* unsymmetrised bispectrum U[X][Y][Z][a][b][c - tmin(a, b)], c up to L */
  size_t ucount = (size_t)bf * bf * bf * L * L * L;
  double *U = (double *)calloc(ucount, sizeof(double));
#define UIDX(X, Y, Z, a, b, c) (((((size_t)((X) * bf + (Y)) * bf + (Z)) * L + (a)) * L + (b)) * L + (c))
  double *I3 = (double *)malloc(sizeof(double) * (size_t)L * R * K * K);
  double *I2 = (double *)malloc(sizeof(double) * (size_t)L * L * R * K);
  double *I1 = (double *)malloc(sizeof(double) * (size_t)L * L * L * R);
  double *Ir = (double *)malloc(sizeof(double) * (size_t)L * L * L);
  int rc = 0;
  for (int X = 0; X < bf && !rc; ++X)
    for (int im = 0; im < s->m_size && !rc; ++im) {
      int M3 = s->m[im];
      double fa = 1, f2a = 1;
      for (int c = M3; c > 0; --c) fa *= c;
      for (int c = 2 * M3; c > 0; --c) f2a *= c;
      double coef = pow(2., M3) * fa / sqrt(f2a);
      for (int oL3 = 0; oL3 < 2 * M3 + 1 && !rc; ++oL3) {
        if (parity == 0 ? (oL3 % 2 != 0) : (oL3 % 2 == 0)) continue;
        /* k3 */
        memset(I3, 0, sizeof(double) * (size_t)L * R * K * K);
#pragma omp parallel for schedule(dynamic)
        for (int il3 = 0; il3 < L; ++il3) {
          int l3 = l[il3], L3 = abs(l3 - M3) + oL3;
          if (M3 > l3 || L3 > l3 + M3) continue;
          int tt = tt_base[bs->bf[X]] + lm_off[il3] + im;
          int p = 0;
          for (int k1 = 0; k1 < K; ++k1)
            for (int k2 = 0; k2 <= k1; ++k2, ++p) {
              const double *T = T2 + (size_t)tt * nu + uoff[p];
              for (int ir = 0; ir < R; ++ir) {
                double v = o_convolve(&B, kall + uoff[p], dkall + uoff[p], ksz[p], T, NULL, L3, r[ir]);
                if (M3 != 0) v *= coef;
                v *= 2;
                I3[(((size_t)il3 * R + ir) * K + k1) * K + k2] = v;
              }
            }
        }
        for (int Y = 0; Y < bf && !rc; ++Y) {
          /* k2 */
          memset(I2, 0, sizeof(double) * (size_t)L * L * R * K);
          int bad2 = 0;
#pragma omp parallel for schedule(dynamic) reduction(| : bad2)
          for (int ir = 0; ir < R; ++ir) {
            double *f = (double *)malloc(sizeof(double) * K), *ip = (double *)malloc(sizeof(double) * Q);
            for (int il3 = 0; il3 < L && !bad2; ++il3) {
              if (M3 > l[il3]) continue;
              for (int k1 = 0; k1 < K && !bad2; ++k1) {
                for (int k2 = 0; k2 < K; ++k2) {
                  if (k1 > k2) f[k2] = I3[(((size_t)il3 * R + ir) * K + k1) * K + k2];
                  else f[k2] = I3[(((size_t)il3 * R + ir) * K + k2) * K + k1] * pow(-kp[k1] / kp[k2], M3);
                  f[k2] *= 1 / pow(kp[k2], 2);
                }
                if (o_interp_k(kp, K, f, bs->k2_interpolation == SONG2_INTERP_CUBIC, q, Q, bs->pk, ip)) {
                  bad2 = 1;
                  break;
                }
                for (int il2 = 0; il2 < L; ++il2) {
                  const double *T1 = bs->transfer1 + ((size_t)Y * L + il2) * Q;
                  I2[(((size_t)il3 * L + il2) * R + ir) * K + k1] = o_convolve(&B, q, dq, Q, ip, T1, l[il2], r[ir]);
                }
              }
            }
            free(f);
            free(ip);
          }
          if (bad2) {
            snprintf(err, SONG2_ERRLEN, "q beyond the largest k");
            rc = 1;
          }
          for (int oL1 = 0; oL1 < 2 * M3 + 1 && !rc; ++oL1) {
            if (oL1 % 2 != 0) continue;
            for (int Z = 0; Z < bf && !rc; ++Z) {
              /* k1 */
              int bad1 = 0;
#pragma omp parallel for schedule(dynamic) reduction(| : bad1)
              for (int ir = 0; ir < R; ++ir) {
                double *f = (double *)malloc(sizeof(double) * K), *ip = (double *)malloc(sizeof(double) * Q);
                for (int il3 = 0; il3 < L && !bad1; ++il3) {
                  if (M3 > l[il3]) continue;
                  for (int il2 = 0; il2 < L && !bad1; ++il2) {
                    int a = tmin[il3 * L + il2], b = tmax[il3 * L + il2];
                    if (b < a) continue;
                    for (int k1 = 0; k1 < K; ++k1)
                      f[k1] = I2[(((size_t)il3 * L + il2) * R + ir) * K + k1] * (1 / pow(kp[k1], 2));
                    if (o_interp_k(kp, K, f, bs->k1_interpolation == SONG2_INTERP_CUBIC, q, Q, bs->pk, ip)) {
                      bad1 = 1;
                      break;
                    }
                    for (int il1 = a; il1 <= b; ++il1) {
                      int l1 = l[il1], L1 = abs(l1 - M3) + oL1;
                      double v = 0;
                      if (L1 <= l1 + M3) {
                        const double *T1 = bs->transfer1 + ((size_t)Z * L + il1) * Q;
                        v = o_convolve(&B, q, dq, Q, ip, T1, L1, r[ir]);
                      }
                      I1[(((size_t)il3 * L + il2) * L + il1) * R + ir] = v;
                    }
                  }
                }
                free(f);
                free(ip);
              }
              if (bad1) {
                snprintf(err, SONG2_ERRLEN, "q beyond the largest k");
                rc = 1;
                continue;
              }
              /* r */
              for (int il3 = 0; il3 < L; ++il3)
                for (int il2 = 0; il2 < L; ++il2)
                  for (int il1 = tmin[il3 * L + il2]; il1 <= tmax[il3 * L + il2]; ++il1) {
                    const double *I = I1 + (((size_t)il3 * L + il2) * L + il1) * R;
                    double sum = 0;
                    for (int ir = 0; ir < R; ++ir) {
                      double v = r[ir] * r[ir] * I[ir];
                      if (v == 0.) continue;
                      sum += v * dr[ir];
                    }
                    Ir[((size_t)il3 * L + il2) * L + il1] = 0.5 * sum;
                  }
              /* geometry */
              for (int il3 = 0; il3 < L; ++il3) {
                int l3 = l[il3], L3 = abs(l3 - M3) + oL3;
                if (L3 > l3 + M3 || M3 > l3) continue;
                long double F3 = o_w3j(L3, M3, l3, 0, -M3, M3), S3 = F3;
                if (M3 != 0) {
                  long double sg = (oL3 % 2) ? -1 : 1;
                  S3 = parity == 0 ? F3 + sg * F3 : F3 - sg * F3;
                }
                for (int il2 = 0; il2 < L; ++il2) {
                  int l2 = l[il2];
                  for (int il1 = tmin[il3 * L + il2]; il1 <= tmax[il3 * L + il2]; ++il1) {
                    int l1 = l[il1], L1 = abs(l1 - M3) + oL1;
                    if (L1 > l1 + M3) continue;
                    if (!o_tri(L1, l2, L3)) continue;
                    int even_conf = ((l1 + l2 + l3) % 2 == 0);
                    long double F123 = o_w3j000(l1, l2, l3), FL1 = o_w3j000(L1, l2, L3),
                                F1 = o_w3j000(L1, l1, M3), F6 = song2_oracle_wigner6j_l(L1, L3, l2, l3, l1, M3);
                    double integral = Ir[((size_t)il3 * L + il2) * L + il1];
                    long double pref = parity == 0
                                           ? 8 / (O_PI * O_PI * O_PI) * (2 * L1 + 1.) * (2 * L3 + 1.)
                                           : -0.5 / (4 * O_PI * O_PI * O_PI * O_PI) * (2 * L1 + 1.) * (2 * L3 + 1.) *
                                                 (2 * l1 + 1) * (2 * l2 + 1);
                    long double geo = S3 * F1 * FL1 * F6;
                    if (parity == 0 && even_conf) geo /= F123;
                    int ex = parity == 0 ? l3 + L3 - l1 - L1 : l3 + L3 - l1 - L1 - 1;
                    double sg = ((ex / 2) % 2 == 0) ? 1 : -1;
                    double *dst = U + UIDX(X, Y, Z, il3, il2, il1);
                    if (parity == 0 && m_max == 0) *dst = 8 / (O_PI * O_PI * O_PI) * integral;
                    else *dst += (double)(sg * pref * geo * integral);
                  }
                }
              }
            }
          }
        }
      }
    }
  if (!rc && B.bad) {
    snprintf(err, SONG2_ERRLEN, "a Bessel argument fell outside the table");
    rc = 1;
  }
  if (!rc) {
    /* symmetrisation over the position of the second-order field */
    int64_t n = 0;
    for (int a = 0; a < L; ++a)
      for (int b = 0; b <= a; ++b) {
        int lo = tmin[a * L + b], hi = tmax[a * L + b] < b ? tmax[a * L + b] : b;
        for (int c = lo; c <= hi; ++c) ++n;
      }
    int64_t ci = 0;
    for (int a = 0; a < L; ++a)
      for (int b = 0; b <= a; ++b) {
        int lo = tmin[a * L + b], hi = tmax[a * L + b] < b ? tmax[a * L + b] : b;
        for (int c = lo; c <= hi; ++c, ++ci)
          for (int X = 0; X < bf; ++X)
            for (int Y = 0; Y < bf; ++Y)
              for (int Z = 0; Z < bf; ++Z)
                out[((size_t)(X * bf + Y) * bf + Z) * n + ci] =
                    U[UIDX(X, Y, Z, a, b, c)] + U[UIDX(Y, X, Z, b, a, c)] + U[UIDX(Z, Y, X, c, b, a)];
      }
  }
#undef UIDX
  free(U);
  free(I3);
  free(I2);
  free(I1);
  free(Ir);
  free(dq);
  free(dr);
  free(tmin);
  free(tmax);
  free(lm_off);
  free(ksz);
  free(kall);
  free(dkall);
  free(uoff);
  if (B.ddj) {
    for (int rr = 0; rr < t.n_l1; ++rr) free(B.ddj[rr]);
    free(B.ddj);
  }
  o_free_tables(&t);
  return rc;
}
