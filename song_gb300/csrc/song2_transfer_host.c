/* song2_transfer_host.c - host side of the line-of-sight integration that turns
 * the second-order sources into transfer functions (SONG's transfer2.c and
 * bessel2.c): the multipole list, the transfer k grids, the layout of the
 * transfer types, the 3j coefficients of the projection functions and the x
 * ranges of the spherical Bessel functions.  The tables themselves and the
 * integral run on the device (song2_los.cu).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "song2.h"
#include "song2_los.h"

#define S2_PI 3.141592653589793238462643383279502884

/* ------------------------------------------------------------- defaults */

void song2_los_defaults(song2_los_spec *los, const song2_spec *spec, const song2_tables *tab) {
  memset(los, 0, sizeof(*los));
  /* transfers2 / precision2 defaults (input2.c:2206-2207, 2301-2331) */
  los->k3_sampling = SONG2_K3_SAMPLING_CLASS;
  los->q_linstep = 0.45;
  los->tau_sampling = SONG2_TAU_SAMPLING_SOURCES;
  los->tau_linstep = 0.6;
  los->k3_interpolation = SONG2_INTERP_LINEAR;
  los->time_interpolation = SONG2_INTERP_LINEAR;
  los->bessel_interpolation = SONG2_INTERP_LINEAR;
  los->k3_extrapolation = SONG2_K3_EXTRAP_NONE;
  los->extra_k3_oscillations_left = 0;
  los->extra_k3_oscillations_right = 0;
  los->x_step = 0.2;
  los->j_cut = 1e-12;
  los->J_cut = 1e-6;
  los->bessel_tol_x_min = 1e-4;
  /* pbs2->xx_max for the lin/log k samplings: k_max times a guess of tau0,
     extended by one step and 5 % (input2.c:1982-2006) */
  double k_max = 0.0;
  if (spec && spec->k && spec->k_size > 0) k_max = spec->k[spec->k_size - 1];
  los->x_max = (k_max * 18000.0 + los->x_step) * 1.05;
  if (tab) {
    los->tau0 = tab->tau0;
    los->tau_rec = song2_recombination_time(tab);
  }
}

/* -------------------------------------------------------------- l list */

int song2_l_list(int l_max, double l_logstep, int l_linstep, int *out) {
  if (l_max < 2) {
    if (out) out[0] = l_max < 0 ? 0 : l_max;
    return 1;
  }
  int n = 0, l = 2;
  if (out) out[n] = l;
  ++n;
  int inc = (int)(l * (l_logstep - 1.0));
  if (inc < 1) inc = 1;
  while (l + inc < l_max && inc < l_linstep) {
    l += inc;
    if (out) out[n] = l;
    ++n;
    inc = (int)(l * (l_logstep - 1.0));
    if (inc < 1) inc = 1;
  }
  inc = l_linstep < 1 ? 1 : l_linstep;
  while (l + inc <= l_max) {
    l += inc;
    if (out) out[n] = l;
    ++n;
  }
  if (l != l_max) {
    if (out) out[n] = l_max;
    ++n;
  }
  return n;
}

/* ------------------------------------------------------- recombination */

static double bg_col(const song2_tables *t, int col, double x) {
  /* natural cubic spline on the uniform ln tau grid */
  double u = (x - t->bg_lntau0) / t->bg_dlntau;
  int i = (int)floor(u);
  if (i < 0) i = 0;
  if (i > t->bg_size - 2) i = t->bg_size - 2;
  double b = u - i, a = 1.0 - b, h = t->bg_dlntau;
  const double *y0 = t->bg + (size_t)i * SONG2_BG_SIZE, *y1 = y0 + SONG2_BG_SIZE;
  const double *d0 = t->bg_dd + (size_t)i * SONG2_BG_SIZE, *d1 = d0 + SONG2_BG_SIZE;
  return a * y0[col] + b * y1[col] + ((a * a * a - a) * d0[col] + (b * b * b - b) * d1[col]) * h * h / 6.0;
}

/* ln of the visibility kappa' exp(-kappa) at x = ln tau */
static double ln_visibility(const song2_tables *t, double x) {
  return bg_col(t, SONG2_BG_LN_KAPPA_DOT, x) - bg_col(t, SONG2_BG_KAPPA, x);
}

double song2_recombination_time(const song2_tables *t) {
  /* coarse scan of the table nodes, then golden-section refinement */
  int best = 0;
  double vb = -INFINITY;
  for (int i = 0; i < t->bg_size; ++i) {
    double v = ln_visibility(t, t->bg_lntau0 + i * t->bg_dlntau);
    if (v > vb) {
      vb = v;
      best = i;
    }
  }
  double lo = t->bg_lntau0 + (best > 0 ? best - 1 : 0) * t->bg_dlntau;
  double hi = t->bg_lntau0 + (best < t->bg_size - 1 ? best + 1 : best) * t->bg_dlntau;
  const double g = 0.5 * (sqrt(5.0) - 1.0);
  double c = hi - g * (hi - lo), d = lo + g * (hi - lo);
  double fc = ln_visibility(t, c), fd = ln_visibility(t, d);
  for (int it = 0; it < 200 && hi - lo > 1e-14; ++it) {
    if (fc > fd) {
      hi = d;
      d = c;
      fd = fc;
      c = hi - g * (hi - lo);
      fc = ln_visibility(t, c);
    } else {
      lo = c;
      c = d;
      fc = fd;
      d = lo + g * (hi - lo);
      fd = ln_visibility(t, d);
    }
  }
  return exp(0.5 * (lo + hi));
}

/* ------------------------------------------------------- type layout */

/* index of the largest m of the spec's list with m <= l, or -1 (ppr2->index_m_max) */
int s2los_index_m_max(const song2_spec *s, int l) {
  int im = -1;
  for (int i = 0; i < s->m_size; ++i)
    if (s->m[i] <= l) im = i;
  return im;
}

int song2_transfer_types(const song2_spec *s, const song2_los_spec *los, int *type, int *l, int *m) {
  int has[3] = {s->has_source_T, s->has_source_E, s->has_source_B};
  int n = 0;
  for (int t = 0; t < 3; ++t) {
    if (!has[t]) continue;
    for (int il = 0; il < los->l_size; ++il) {
      int imx = s2los_index_m_max(s, los->l[il]);
      for (int im = 0; im <= imx; ++im) {
        if (type) type[n] = t;
        if (l) l[n] = los->l[il];
        if (m) m[n] = s->m[im];
        ++n;
      }
    }
  }
  return n;
}

/* ----------------------------------------------------- transfer k grids */

/* k3 limits and linear step of one pair (transfer2_get_k3_size, transfer2.c:1329-1564) */
static void pair_k_limits(const song2_spec *s, const song2_los_spec *los, const double *k3, int k3n, double *kmin_tr,
                          double *kmax_tr, double *step) {
  double kmin_pt = k3[0], kmax_pt = k3[k3n - 1];
  double lo = kmin_pt, hi = kmax_pt;
  if (los->k3_extrapolation != SONG2_K3_EXTRAP_NONE) {
    double range = kmax_pt - kmin_pt;
    double right = 2. * S2_PI * los->extra_k3_oscillations_right / (los->tau0 - los->tau_rec);
    double left = 2. * S2_PI * los->extra_k3_oscillations_left / (los->tau0 - los->tau_rec);
    if (range < right) hi += right - range;
    if (hi > s->k[s->k_size - 1]) hi = s->k[s->k_size - 1];
    if (range < left) lo -= left - range;
    double floor_k = s->k[0] < kmin_pt ? s->k[0] : kmin_pt;
    if (lo < floor_k) lo = floor_k;
    if (los->extra_k3_oscillations_left < 0) lo = s->k[0];
    if (los->extra_k3_oscillations_right < 0) hi = s->k[s->k_size - 1];
  }
  *kmin_tr = lo;
  *kmax_tr = hi;
  if (los->k3_sampling == SONG2_K3_SAMPLING_CLASS)
    *step = 2. * S2_PI / (los->tau0 - los->tau_rec) * los->q_linstep;
  else
    *step = los->x_step / los->tau0;
}

/* The k list of one pair (transfer2_get_k3_size for the counts, then
   transfer2_get_k3_list for the values, :1566-1680); fills k_out when non-NULL. */
static int pair_k_list(const song2_spec *s, const song2_los_spec *los, const double *k3, int k3n, int *size,
                       int *phys_start, int *phys_size, double *k_out, char *err) {
  double kmin_tr, kmax_tr, step;
  pair_k_limits(s, los, k3, k3n, &kmin_tr, &kmax_tr, &step);
  double kmin_pt = k3[0], kmax_pt = k3[k3n - 1];
  if (!(step > 0)) {
    snprintf(err, SONG2_ERRLEN, "transfer k step is %g", step);
    return 1;
  }
  if (kmax_tr > los->x_max / los->tau0) {
    snprintf(err, SONG2_ERRLEN,
             "x_max is not large enough: the projection functions J(k (tau0-tau)) do not cover k_max=%g "
             "(tau0=%g, x_max=%g)",
             kmax_tr, los->tau0, los->x_max);
    return 1;
  }
  /* sizes (transfer2_get_k3_size) */
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
  int pstart = itr - 1;
  while (ipt < k3n && (k3[ipt] - k) < step) {
    k = k3[ipt];
    ipt++;
    itr++;
  }
  int psize = ipt;
  while (k < kmax_tr) {
    k += step;
    itr++;
    if (k <= kmax_pt && k >= kmin_pt) psize++;
  }
  int n = (k > kmax_tr) ? itr - 1 : itr;
  if (n < 2) {
    snprintf(err, SONG2_ERRLEN, "fewer than 2 transfer k values for a pair with k3 in [%g, %g]", kmin_pt, kmax_pt);
    return 1;
  }
  if (los->k3_extrapolation == SONG2_K3_EXTRAP_NONE && (psize != n || pstart != 0)) {
    snprintf(err, SONG2_ERRLEN, "transfer k grid leaves the triangle without extrapolation");
    return 1;
  }
  *size = n;
  *phys_start = pstart;
  *phys_size = psize;
  if (!k_out) return 0;
  /* values (transfer2_get_k3_list) */
  ipt = 0;
  itr = 0;
  k = kmin_tr;
  k_out[0] = kmin_tr;
  itr++;
  if (los->k3_extrapolation != SONG2_K3_EXTRAP_NONE) {
    while (k < kmin_pt) {
      k += step;
      if (itr < n) k_out[itr] = k;
      itr++;
    }
    if (k != kmin_pt) {
      k = kmin_pt;
      k_out[itr - 1] = k;
    }
  }
  ipt++;
  while (ipt < k3n && (k3[ipt] - k) < step) {
    k = k3[ipt];
    if (itr < n) k_out[itr] = k;
    ipt++;
    itr++;
  }
  while (itr < n && k < kmax_tr) {
    k += step;
    k_out[itr] = k;
    itr++;
  }
  if (k_out[n - 1] > kmax_tr) {
    snprintf(err, SONG2_ERRLEN, "transfer k grid overshoots k_max=%.17g", kmax_tr);
    return 1;
  }
  return 0;
}

int64_t song2_transfer_k_grids(const song2_spec *s, const song2_los_spec *los, int *sizes, int *physical_start,
                               int *physical_size, double *k_out, char *err) {
  int64_t total = 0, k3off = 0;
  int pair = 0;
  for (int i1 = 0; i1 < s->k_size; ++i1)
    for (int i2 = 0; i2 <= i1; ++i2, ++pair) {
      int k3n = s->k3_size[i1 * s->k_size + i2];
      if (k3n < 2 || (los->k3_interpolation == SONG2_INTERP_CUBIC && k3n < 4)) {
        snprintf(err, SONG2_ERRLEN, "pair (%d,%d): cannot interpolate in k3 with k3_size=%d", i1, i2, k3n);
        return -1;
      }
      int n, ps, pn;
      if (pair_k_list(s, los, s->k3 + k3off, k3n, &n, &ps, &pn, k_out ? k_out + total : NULL, err)) return -1;
      if (sizes) sizes[pair] = n;
      if (physical_start) physical_start[pair] = ps;
      if (physical_size) physical_size[pair] = pn;
      total += n;
      k3off += k3n;
    }
  return total;
}

/* ----------------------------------------------------------- 3j symbols */

int song2_wigner3j_row(int l2, int l3, int m2, int m3, int *l1_min_out, int *l1_max_out, double *out,
                       int out_size) {
  /* (l1 l2 l3; m1 m2 m3) with m1 = -m2-m3, for l1 = l1_min..l1_max, by the
     three-term recursion of Schulten and Gordon (J. Math. Phys. 16 (1975) 1961)
       l1 A(l1+1) f(l1+1) + B(l1) f(l1) + (l1+1) A(l1) f(l1-1) = 0,
       A(l1) = sqrt((l1^2 - (l2-l3)^2) ((l2+l3+1)^2 - l1^2) (l1^2 - m1^2)),
       B(l1) = -(2 l1 + 1) (l2(l2+1) m1 - l3(l3+1) m1 - l1(l1+1)(m3 - m2)),
     run downwards from l1_max (where A(l1_max+1) = 0), normalised by
     sum (2 l1 + 1) f^2 = 1 and the sign (-1)^(l2-l3-m1) of f(l1_max). */
  int m1 = -m2 - m3;
  if (abs(m2) > l2 || abs(m3) > l3) return 1;
  int lo = abs(l2 - l3) > abs(m1) ? abs(l2 - l3) : abs(m1);
  int hi = l2 + l3;
  if (hi < lo) return 1;
  int n = hi - lo + 1;
  if (n > out_size) return 1;
  *l1_min_out = lo;
  *l1_max_out = hi;
#define A_(j) sqrt(((double)(j) * (j) - (double)(l2 - l3) * (l2 - l3)) * \
                   ((double)(l2 + l3 + 1) * (l2 + l3 + 1) - (double)(j) * (j)) * ((double)(j) * (j) - (double)m1 * m1))
#define B_(j) (-(2.0 * (j) + 1.0) * ((double)l2 * (l2 + 1) * m1 - (double)l3 * (l3 + 1) * m1 - \
                                     (double)(j) * ((j) + 1) * (double)(m3 - m2)))
  double *f = out;
  f[n - 1] = 1.0;
  if (n > 1) f[n - 2] = -B_(hi) * f[n - 1] / ((hi + 1.0) * A_(hi));
  for (int j = hi - 1; j > lo; --j) {
    int i = j - lo;
    /* f(j-1) = -(j A(j+1) f(j+1) + B(j) f(j)) / ((j+1) A(j)) */
    f[i - 1] = -(j * A_(j + 1) * f[i + 1] + B_(j) * f[i]) / ((j + 1.0) * A_(j));
  }
#undef A_
#undef B_
  double norm = 0.0;
  for (int i = 0; i < n; ++i) norm += (2.0 * (lo + i) + 1.0) * f[i] * f[i];
  double sgn = ((l2 - l3 - m1) % 2 != 0) ? -1.0 : 1.0;
  double c = sgn / sqrt(norm);
  if (f[n - 1] < 0) c = -c;
  for (int i = 0; i < n; ++i) out[i] = f[i] * c;
  return 0;
}

/* --------------------------------------------- spherical Bessel functions */

/* j_l(x) for l = 0..lmax at one x, by downward recurrence from above
   max(lmax, x) normalised to j_0 or j_1 (Miller's method); the same routine as
   the device kernel, one x at a time.  out[l] for l <= lmax. */
void s2los_bessel_all(double x, int lmax, double *out) {
  if (x == 0.0) {
    for (int l = 0; l <= lmax; ++l) out[l] = (l == 0) ? 1.0 : 0.0;
    return;
  }
  int top = s2los_miller_start(x, lmax);
  double inv = 1.0 / x;
  double fp = 0.0, f = 1.0;     /* f_{l+1}, f_l */
  int scale = 0;
  /* first pass: the scale count and the normalisation */
  for (int l = top; l > 0; --l) {
    double fm = (2.0 * l + 1.0) * inv * f - fp;
    fp = f;
    f = fm;
    if (fabs(f) > S2LOS_BIG) {
      f *= S2LOS_SMALL;
      fp *= S2LOS_SMALL;
      ++scale;
    }
  }
  int e_norm;
  double m_norm = frexp(s2los_miller_norm(x, f, fp), &e_norm);
  int final_scale = scale;
  /* second pass: the same recurrence, each stored value brought to the final
     scale and normalised exactly */
  fp = 0.0;
  f = 1.0;
  scale = 0;
  for (int l = top; l >= 0; --l) {
    if (l <= lmax) out[l] = ldexp(f * m_norm, e_norm - S2LOS_SCALE_BITS * (final_scale - scale));
    if (l == 0) break;
    double fm = (2.0 * l + 1.0) * inv * f - fp;
    fp = f;
    f = fm;
    if (fabs(f) > S2LOS_BIG) {
      f *= S2LOS_SMALL;
      fp *= S2LOS_SMALL;
      ++scale;
    }
  }
}

/* j_l(x) at one (l, x) */
static double bessel_one(int l, double x) {
  double stack[64];
  double *buf = (l < 64) ? stack : (double *)malloc(sizeof(double) * (l + 1));
  if (!buf) return 0.0;
  s2los_bessel_all(x, l, buf);
  double v = buf[l];
  if (buf != stack) free(buf);
  return v;
}

/* First index of the x grid from which j_l1 is stored (bessel2_j_for_l1,
   bessel2.c:1669-1800): bisection in x for j_l1(x) = j_cut below the first peak,
   then the grid point before it; x_size (nothing stored) when j_l1 is
   negligible everywhere, where the reference stores a single zero. */
int s2los_bessel_xmin(int l1, const song2_los_spec *los, int x_size, double x_max) {
  if (l1 == 0) return 0;
  double lo = 0.0, hi = l1 + 0.5, xmin;
  int done = 0;
  while (lo == 0.0 || (hi - lo) / lo > los->bessel_tol_x_min) {
    if (hi - lo < S2LOS_SMALLEST_VARIATION) {
      xmin = hi = lo;
      done = 1;
      break;
    }
    double mid = 0.5 * (hi + lo);
    if (bessel_one(l1, mid) >= los->j_cut) hi = mid;
    else lo = mid;
  }
  if (!done) xmin = lo;
  if (xmin >= x_max) return x_size;
  int i = 0;
  while (s2los_x_of(i, x_size, x_max) < xmin) i++;
  if (i != 0) --i;
  return i;
}
