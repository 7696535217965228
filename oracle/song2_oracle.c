/*
 * song2_oracle.c - CPU restatement of SONG's second-order perturbation
 * evolution (source/perturbations2.c), FP64, OpenMP over k1.
 *
 * TEST INFRASTRUCTURE ONLY (see song2_oracle.h): it checks the GPU evolver and
 * provides the timed CPU baseline; it is never on the product path.
 *
 * Structure follows the reference function by function:
 *   perturb2_get_lm_lists        perturbations2.c:1115-1533  -> cfg_init
 *   perturb2_geometrical_corner  perturbations2.c:5446-6069  -> geometrical_corner
 *   perturb2_start_time_evolution            :3388-3524      -> start_time
 *   perturb2_approximations / switches       :4854-5403      -> tca_is_on, solve
 *   perturb2_vector_init                     :6620-7357      -> vector_init
 *   perturb2_initial_conditions              :3670-4216      -> initial_conditions
 *   perturb2_derivs                          :7636-8451      -> derivs
 *   perturb2_einstein                        :8484-8814      -> einstein
 *   perturb2_workspace_at_tau                :8839-9027      -> workspace_at_tau
 *   perturb2_fluid_variables                 :9108-9338      -> (inlined in tca_variables)
 *   perturb2_tca_variables                   :9374-9738      -> tca_variables
 *   perturb2_rsa_variables                   :9773-10164     -> rsa_variables
 *   perturb2_compute_psi_prime               :10188-10383    -> compute_psi_prime
 *   perturb2_quadratic_sources               :10643-11813    -> quadratic_sources
 *   perturb2_sources                         :11869-12823    -> store_sources
 *     (delta-tilde terms                     :12339-12710    -> delta_tilde_source)
 *   evolver_ndf15 [CLASS, absent]           called :6517-6536 -> ndf15
 *
 * Deliberate, documented choices (same in the GPU evolver):
 *  - quadratic sources in derivs come from a per-triplet table on the
 *    first-order time nodes, splined in ln tau (perturbations2.c:10407-10606,
 *    14366-14688), as the reference's default path; tight coupling, initial
 *    conditions and the source functions compute them directly;
 *  - perfect baryons and CDM (reference default, input2.c:2087-2088), Newtonian
 *    gauge, phi equation = huang (input2.c:2152); RSA intervals when the spec
 *    asks for them, no NRA/UFA;
 *  - NDF15 written from Shampine & Reichelt, SIAM J. Sci. Comput. 18 (1997):
 *    orders 1-5, kappa = (-0.185,-1/9,-0.0823,-0.0415,0), simplified Newton,
 *    max-norm error control, backward-difference step change, dense output.
 *    The Jacobian of the affine system is obtained exactly by applying the
 *    linear part of derivs to the unit vectors.
 */
#include "song2_oracle.h"
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif
#define SQRT_2 1.4142135623730950488
#define SQRT_3 1.7320508075688772935
#define SQRT_6 2.4494897427831780982
#define FOUR_THIRDS (4.0 / 3.0)
#define ONE_THIRD (1.0 / 3.0)
#define QUAD_COEFF 2.0
#define LMAXP (SONG2_MAX_L + 4)

static int o_fo_size(int fo_l_max);
static int64_t o_n_triplets(const song2_spec *s);

/* ======================================================= 3j couplings */

static double lfact(int n) { return lgamma((double)n + 1.0); }

/* Wigner 3j symbol by the Racah formula */
static double wigner3j(int j1, int j2, int j3, int m1, int m2, int m3) {
  if (m1 + m2 + m3 != 0) return 0.0;
  if (j3 < abs(j1 - j2) || j3 > j1 + j2) return 0.0;
  if (abs(m1) > j1 || abs(m2) > j2 || abs(m3) > j3) return 0.0;
  double pre = 0.5 * (lfact(j1 + j2 - j3) + lfact(j1 - j2 + j3) + lfact(-j1 + j2 + j3) - lfact(j1 + j2 + j3 + 1) +
                      lfact(j1 + m1) + lfact(j1 - m1) + lfact(j2 + m2) + lfact(j2 - m2) + lfact(j3 + m3) +
                      lfact(j3 - m3));
  int tmin = 0;
  if (j2 - j3 - m1 > tmin) tmin = j2 - j3 - m1;
  if (j1 - j3 + m2 > tmin) tmin = j1 - j3 + m2;
  int tmax = j1 + j2 - j3;
  if (j1 - m1 < tmax) tmax = j1 - m1;
  if (j2 + m2 < tmax) tmax = j2 + m2;
  double sum = 0.0;
  for (int t = tmin; t <= tmax; ++t) {
    double v = exp(pre - (lfact(t) + lfact(j3 - j2 + t + m1) + lfact(j3 - j1 + t - m2) + lfact(j1 + j2 - j3 - t) +
                          lfact(j1 - t - m1) + lfact(j2 - t + m2)));
    sum += (t % 2 ? -v : v);
  }
  int ph = j1 - j2 - m3;
  return ((ph % 2) != 0 ? -sum : sum);
}

/* int  sY*_{lm} Y_{1q} sY_{l'm1} dOmega, spin s */
static double spin_gaunt(int s, int l, int m, int q, int lp, int m1) {
  double v = sqrt((2.0 * l + 1) * 3.0 * (2.0 * lp + 1) / (4 * M_PI)) * wigner3j(l, 1, lp, -m, q, m1) *
             wigner3j(l, 1, lp, s, 0, -s);
  int ph = m + s;
  return (ph % 2 ? -v : v);
}

double song2_oracle_coupling(int kind, int l, int m1, int m) {
  int q = m - m1;
  if (abs(q) > 1 || l < 0) return 0.0;
  switch (kind) {
  case 0: /* c_minus: multipole l of n_q * f_{l-1,m1} */
    if (l < 1) return 0.0;
    return sqrt(4 * M_PI * (2.0 * l + 1) / (3.0 * (2.0 * l - 1))) * spin_gaunt(0, l, m, q, l - 1, m1);
  case 1:
    return sqrt(4 * M_PI * (2.0 * l + 1) / (3.0 * (2.0 * l + 3))) * spin_gaunt(0, l, m, q, l + 1, m1);
  case 2:
    if (l < 3) return 0.0;
    return sqrt(4 * M_PI * (2.0 * l + 1) / (3.0 * (2.0 * l - 1))) * spin_gaunt(2, l, m, q, l - 1, m1);
  case 3:
    if (l < 2) return 0.0;
    return sqrt(4 * M_PI * (2.0 * l + 1) / (3.0 * (2.0 * l + 3))) * spin_gaunt(2, l, m, q, l + 1, m1);
  case 4:
    /* E-B mixing: the l'=l spin-2 coupling; sign fixed so that d_zero(l,m,m) = 2m/(l(l+1)) */
    if (l < 2) return 0.0;
    return -sqrt(4 * M_PI / 3.0) * spin_gaunt(2, l, m, q, l, m1);
  }
  return 0.0;
}

/* delta-tilde coupling, perturb2_get_lm_lists (perturbations2.c:1380-1490): the
   3j products of coupling_general (song_tools, absent from the reference tree),
   as its call site defines them (:1439-1446), with the field's prefactor
   (:1386-1400) and the sign i^L or i^(L-1) (:1466-1476). */
double song2_oracle_delta_tilde_coupling(int field, int l, int m, int l1, int m1, int l2) {
  int F = (field == 0) ? 0 : 2;
  double prefactor = (field == 0) ? 0.5 : 1.0;
  if (l2 < F || l < F) return 0.0;
  int L = l - l1 - l2;
  int even = (field != 2);
  if ((abs(L) % 2 == 0) != even) return 0.0;
  double sign = even ? ((abs(L) / 2) % 2 ? -1.0 : 1.0) : ((abs(L - 1) / 2) % 2 ? -1.0 : 1.0);
  int m2 = m - m1;
  double v = (m % 2 ? -1.0 : 1.0) * (2.0 * l + 1) * wigner3j(l1, l2, l, 0, F, -F) * wigner3j(l1, l2, l, m1, m2, -m);
  return prefactor * sign * v;
}

/* ======================================================= configuration */

typedef struct cfg_s {
  const song2_spec *s;
  const song2_tables *t;
  int m_size, m[SONG2_MAX_M];
  int compute_m[SONG2_MAX_M];
  int index_m[SONG2_MAX_M]; /* position of m in the list, -1 if absent */
  int index_m_max[LMAXP];   /* last index_m with m <= l, -1 if none */
  int L_big, Lq;
  int lm_array[LMAXP][SONG2_MAX_M];
  int n_lm;
  int lm_quad[LMAXP][LMAXP];
  int n_lmq;
  int nlm_array[3][3][SONG2_MAX_M];
  double *cmin, *cplu, *dmin, *dplu, *dzer; /* [n_lm][3] */
  int fo_l_max, nfo, fo_E, fo_N, fo_CG;
  int first_order_mode;
  int tp2_size, index_tp2_T, index_tp2_E, index_tp2_B, index_tp2_delta_cdm;
  int64_t n_triplets;
  /* ppt2->coupling_coefficients[field][l][m][l1][m1 + dt_Q][l2], l <= dt_L */
  double *dtc;
  int dt_Q, dt_L;
  /* the run-wide configuration, which fixes the source types (itself, except for
     the hierarchy classes of an uneven batch) */
  const struct cfg_s *run;
} cfg_t;

#define LM(l, m) (c->lm_array[(l)][c->index_m[(m)]])
#define LMQ(l, m) (c->lm_quad[(l)][(m)])
#define DTC_SIZE(c) (3 * ((c)->dt_L + 1) * SONG2_MAX_M * ((c)->dt_Q + 1) * (2 * (c)->dt_Q + 1) * ((c)->dt_Q + 1))
#define DTC(c, f, l, m, l1, m1, l2)                                                                                    \
  ((c)->dtc[(((((f) * ((c)->dt_L + 1) + (l)) * SONG2_MAX_M + (m)) * ((c)->dt_Q + 1) + (l1)) * (2 * (c)->dt_Q + 1) +      \
             (m1) + (c)->dt_Q) * ((c)->dt_Q + 1) + (l2)])
/* source-type index of (l, m) in the run-wide layout */
#define RLM(l, m) (c->run->lm_array[(l)][c->run->index_m[(m)]])

static int size_l_indexm(const cfg_t *c, int l_max) {
  int n = 0;
  for (int l = 0; l <= l_max; ++l)
    for (int i = 0; i < c->m_size; ++i)
      if (c->m[i] <= l) ++n;
  return n;
}

static int cfg_init(cfg_t *c, const song2_spec *s, const song2_tables *t, int fo_l_max, char *err) {
  memset(c, 0, sizeof(*c));
  c->s = s; c->t = t;
  c->run = c;
  c->m_size = s->m_size;
  for (int i = 0; i < SONG2_MAX_M; ++i) c->index_m[i] = -1;
  for (int i = 0; i < s->m_size; ++i) {
    c->m[i] = s->m[i];
    if (s->m[i] < 0 || s->m[i] >= SONG2_MAX_M) { snprintf(err, SONG2_ERRLEN, "m out of range"); return 1; }
    c->compute_m[s->m[i]] = 1;
    c->index_m[s->m[i]] = i;
  }
  int L = s->l_max_g;
  if (s->has_polarization2 && s->l_max_pol_g > L) L = s->l_max_pol_g;
  if (s->l_max_ur > L) L = s->l_max_ur;
  if (s->l_max_los_t > L) L = s->l_max_los_t;
  if (s->l_max_los_p > L) L = s->l_max_los_p;
  if (L + 2 >= LMAXP) { snprintf(err, SONG2_ERRLEN, "l_max too large"); return 1; }
  if (s->l_max_g < 2 || s->l_max_ur < 2 || (s->has_polarization2 && s->l_max_pol_g < 2)) {
    snprintf(err, SONG2_ERRLEN, "l_max_* must be at least 2");
    return 1;
  }
  if (s->has_polarization2)
    for (int i = 0; i < s->m_size; ++i) {
      double l = s->l_max_pol_g, m = s->m[i];
      if (l <= 2 || 1 - m * m / (l * l) * (l + 2) / (l - 2) < 0) {
        snprintf(err, SONG2_ERRLEN, "l_max_pol_g too small for m = %d (polarisation closure)", s->m[i]);
        return 1;
      }
    }
  c->L_big = L; c->Lq = L + 1;
  for (int l = 0; l < LMAXP; ++l) {
    c->index_m_max[l] = -1;
    for (int i = 0; i < c->m_size; ++i) if (c->m[i] <= l) c->index_m_max[l] = i;
  }
  int n = 0;
  for (int l = 0; l <= c->Lq; ++l)
    for (int i = 0; i < c->m_size; ++i) c->lm_array[l][i] = (c->m[i] <= l) ? n++ : -1;
  c->n_lm = n;
  n = 0;
  for (int l = 0; l <= c->Lq; ++l)
    for (int m = 0; m <= l; ++m) c->lm_quad[l][m] = n++;
  c->n_lmq = n;
  /* massive hierarchies, perfect fluids: (n,l) = (0,0), (1,1) */
  n = 0;
  for (int nn = 0; nn <= 1; ++nn)
    for (int l = 0; l <= 1; ++l) {
      if ((l != nn) && (l != 0)) continue;
      if ((l == 0) && (nn % 2 != 0)) continue;
      for (int i = 0; i < c->m_size; ++i) c->nlm_array[nn][l][i] = (c->m[i] <= l) ? n++ : -1;
    }
  c->cmin = (double *)calloc((size_t)c->n_lm * 3, sizeof(double));
  c->cplu = (double *)calloc((size_t)c->n_lm * 3, sizeof(double));
  c->dmin = (double *)calloc((size_t)c->n_lm * 3, sizeof(double));
  c->dplu = (double *)calloc((size_t)c->n_lm * 3, sizeof(double));
  c->dzer = (double *)calloc((size_t)c->n_lm * 3, sizeof(double));
  for (int l = 0; l <= c->Lq; ++l)
    for (int i = 0; i < c->m_size; ++i) {
      int m = c->m[i];
      if (m > l) continue;
      int lm = c->lm_array[l][i];
      for (int m1 = m - 1; m1 <= m + 1; ++m1) {
        c->cmin[lm * 3 + m - m1 + 1] = song2_oracle_coupling(0, l, m1, m);
        c->cplu[lm * 3 + m - m1 + 1] = song2_oracle_coupling(1, l, m1, m);
        c->dmin[lm * 3 + m - m1 + 1] = song2_oracle_coupling(2, l, m1, m);
        c->dplu[lm * 3 + m - m1 + 1] = song2_oracle_coupling(3, l, m1, m);
        c->dzer[lm * 3 + m - m1 + 1] = song2_oracle_coupling(4, l, m1, m);
      }
    }
  c->fo_l_max = fo_l_max;
  c->nfo = o_fo_size(fo_l_max);
  c->fo_E = SONG2_FO_I + (fo_l_max + 1);
  c->fo_N = SONG2_FO_I + 2 * (fo_l_max + 1);
  c->fo_CG = SONG2_FO_I + 3 * (fo_l_max + 1);
  c->first_order_mode = (s->ic == SONG2_IC_AD_FIRST_ORDER);
  /* source types (perturb2_indices_of_perturbs) */
  int tp = 0;
  c->index_tp2_T = c->index_tp2_E = c->index_tp2_B = c->index_tp2_delta_cdm = -1;
  if (s->has_source_T) { c->index_tp2_T = tp; tp += size_l_indexm(c, s->l_max_los_t); }
  if (s->has_source_E) { c->index_tp2_E = tp; tp += size_l_indexm(c, s->l_max_los_p); }
  if (s->has_source_B) { c->index_tp2_B = tp; tp += size_l_indexm(c, s->l_max_los_p); }
  if (s->has_source_delta_cdm) c->index_tp2_delta_cdm = tp++;
  c->tp2_size = tp;
  c->n_triplets = o_n_triplets(s);
  if (s->radiation_streaming_approximation != SONG2_RSA_NONE && !c->first_order_mode) {
    if (s->radiation_streaming_approximation != SONG2_RSA_MD &&
        s->radiation_streaming_approximation != SONG2_RSA_MD_WITH_REIO) {
      snprintf(err, SONG2_ERRLEN, "radiation_streaming_approximation: none, MD or MD_with_reio");
      return 1;
    }
    if (!(t->tau_free_streaming > 0) || !(s->radiation_streaming_trigger_tau_over_tau_k > 0)) {
      snprintf(err, SONG2_ERRLEN, "the RSA needs tau_free_streaming > 0 and a positive k tau trigger");
      return 1;
    }
  }
  if (s->use_delta_tilde_in_los && !c->first_order_mode) {
    /* input2.c:742-744 */
    if (s->has_redshift_in_los) {
      snprintf(err, SONG2_ERRLEN, "use_delta_tilde_in_los excludes has_redshift_in_los");
      return 1;
    }
    int Q = s->l_max_los_quadratic_t > s->l_max_los_quadratic_p ? s->l_max_los_quadratic_t : s->l_max_los_quadratic_p;
    if (s->l_max_los_quadratic_t < 0 || s->l_max_los_quadratic_p < 0 || Q > L || Q > SONG2_MAX_M + 1) {
      snprintf(err, SONG2_ERRLEN, "l_max_los_quadratic_t/p out of range");
      return 1;
    }
    c->dt_Q = Q;
    c->dt_L = s->l_max_los_t > s->l_max_los_p ? s->l_max_los_t : s->l_max_los_p;
    c->dtc = (double *)calloc((size_t)DTC_SIZE(c), sizeof(double));
    for (int f = 0; f < 3; ++f)
      for (int l = 0; l <= c->dt_L; ++l)
        for (int m = 0; m <= l && m < SONG2_MAX_M; ++m)
          for (int l1 = 0; l1 <= Q; ++l1)
            for (int m1 = -l1; m1 <= l1; ++m1)
              for (int l2 = 0; l2 <= Q; ++l2)
                DTC(c, f, l, m, l1, m1, l2) = song2_oracle_delta_tilde_coupling(f, l, m, l1, m1, l2);
  }
  return 0;
}

static void cfg_free(cfg_t *c) {
  free(c->cmin); free(c->cplu); free(c->dmin); free(c->dplu); free(c->dzer); free(c->dtc);
}

/* ======================================================= interpolation */

static double spl(int n, int ncol, double x0, double dx, const double *y, const double *dd, int q, double x) {
  double u = (x - x0) / dx;
  int i = (int)floor(u);
  if (i < 0) i = 0;
  if (i > n - 2) i = n - 2;
  double b = u - i, a = 1.0 - b;
  const double *y0 = y + (size_t)i * ncol, *d0 = dd + (size_t)i * ncol;
  return a * y0[q] + b * y0[ncol + q] + ((a * a * a - a) * d0[q] + (b * b * b - b) * d0[ncol + q]) * (dx * dx) / 6.0;
}

/* d/dx of the same spline */
static double spl_dx(int n, int ncol, double x0, double dx, const double *y, const double *dd, int q, double x) {
  double u = (x - x0) / dx;
  int i = (int)floor(u);
  if (i < 0) i = 0;
  if (i > n - 2) i = n - 2;
  double b = u - i, a = 1.0 - b;
  const double *y0 = y + (size_t)i * ncol, *d0 = dd + (size_t)i * ncol;
  return (y0[ncol + q] - y0[q]) / dx + ((1 - 3 * a * a) * d0[q] + (3 * b * b - 1) * d0[ncol + q]) * dx / 6.0;
}

/* ======================================================= layout helpers
   (restated here so that the oracle links against nothing of the product) */

static int o_fo_size(int fo_l_max) { return SONG2_FO_I + 4 * (fo_l_max + 1); }

static int64_t o_n_triplets(const song2_spec *s) {
  int64_t n = 0;
  for (int i1 = 0; i1 < s->k_size; ++i1)
    for (int i2 = 0; i2 <= i1; ++i2) n += s->k3_size[i1 * s->k_size + i2];
  return n;
}

static int64_t o_pair_offset(const song2_spec *s, int index_k1, int index_k2) {
  int64_t off = 0;
  for (int i1 = 0; i1 < s->k_size; ++i1)
    for (int i2 = 0; i2 <= i1; ++i2) {
      if (i1 == index_k1 && i2 == index_k2) return off;
      off += (int64_t)s->tau_size * s->k3_size[i1 * s->k_size + i2];
    }
  return off;
}

/* perturb2_start_time_evolution (perturbations2.c:3388-3524) */
static int o_start_time(const song2_spec *s, const song2_tables *t, double k, double tau_upper, double *tau_ini,
                        char *err) {
  double tau_lower = exp(t->bg_lntau0);
#define O_HC(x) exp(spl(t->bg_size, SONG2_BG_SIZE, t->bg_lntau0, t->bg_dlntau, t->bg, t->bg_dd, SONG2_BG_LN_HC, (x)))
#define O_KD(x) exp(spl(t->bg_size, SONG2_BG_SIZE, t->bg_lntau0, t->bg_dlntau, t->bg, t->bg_dd, SONG2_BG_LN_KAPPA_DOT, (x)))
  double Hc = O_HC(log(tau_lower)), kd = O_KD(log(tau_lower));
  if (Hc / kd > s->start_small_k_at_tau_c_over_tau_h || k / Hc > s->start_large_k_at_tau_h_over_tau_k) {
    snprintf(err, SONG2_ERRLEN, "start time: background table starts too late for k=%g", k);
    return 1;
  }
  double tau_mid = 0.5 * (tau_lower + tau_upper);
  while ((tau_upper - tau_lower) / tau_lower > s->tol_tau_approx) {
    Hc = O_HC(log(tau_mid));
    kd = O_KD(log(tau_mid));
    if (Hc / kd > s->start_small_k_at_tau_c_over_tau_h || k / Hc > s->start_large_k_at_tau_h_over_tau_k)
      tau_upper = tau_mid;
    else
      tau_lower = tau_mid;
    tau_mid = 0.5 * (tau_lower + tau_upper);
  }
#undef O_HC
#undef O_KD
  *tau_ini = tau_mid;
  return 0;
}

/* ======================================================= workspace */

typedef struct {
  int l_max_g, l_max_pol_g, l_max_ur;
  int use_closure_g, use_closure_pol_g, use_closure_ur;
  int n_max_b, l_max_b, n_max_cdm, l_max_cdm;
  int idx_g, idx_E, idx_B, idx_ur, idx_b, idx_cdm;
  int idx_phi, idx_phi_p, idx_omega, idx_gamma, idx_gamma_p;
  int n;
  int tca, rsa;
} pv_t;

enum { QS_WHAT_TOTAL = 0, QS_WHAT_COLLISION = 1 };

typedef struct {
  cfg_t *c;
  int index_k1, index_k2, index_k3;
  double k1, k2, k, k_sq, cosk1k2, cosk1k, cosk2k, k1_dot_k2;
  double k1_m[3], k2_m[3], k1_ten_k2[5], k1_ten_k1[5], k2_ten_k2[5];
  double *rot1, *rot2, *rot1m, *rot2m;
  double *cm12, *cm21, *cp12, *cp21, *cm11, *cm22, *cp11, *cp22;
  double *dm12, *dm21, *dp12, *dp21, *dm11, *dm22, *dp11, *dp22;
  double *dz12, *dz21, *dz11, *dz22;
  pv_t pv;
  /* full (no approximation) hierarchy sizes, used by the quadratic sources */
  int l_max_g, l_max_pol_g, l_max_ur;
  /* background at tau */
  double tau, a, a_sq, Hc, Hc_prime, rho_g, rho_b, rho_cdm, rho_ur, kappa_dot, exp_m_kappa, g, r;
  double *fo1, *fo2;
  int linear_only;
  int qs2_size, iq_g, iq_E, iq_B, iq_ur, iq_b, iq_cdm;
  int iq_psi, iq_psi_prime, iq_phi_prime_poisson, iq_phi_prime_longitudinal, iq_phi_prime_prime;
  int iq_omega_m1_prime, iq_gamma_m2_prime_prime, iq_vv_g, iq_vv_ur, iq_dd_b, iq_vv_b, iq_vv_cdm;
  int iq_vvp_b, iq_vvp_cdm;
  double *qs, *qc;
  /* quadratic-source table of the triplet on the first-order time nodes j0..j0+qt_n-1
     (perturb2_quadratic_sources_for_k1k2k, perturbations2.c:10407-10606):
     qtab[node][2][qs2_size] = values, spline second derivatives in ln tau */
  double *qtab, *qt_c;
  int qt_j0, qt_n, qt_ready;
  /* shared variables (perturb2_workspace_at_tau) */
  double I_00, N_00, N_1m[3], I_1m[3], I_2m[3], E_2m[3], B_2m[3], C_1m[3], b_200, b_22m[3], cdm_200, cdm_22m[3];
  double I_1m_tca1[3], I_2m_tca1[3], E_2m_tca1[3], B_2m_tca1[3], C_1m_tca1[3], Pi_tca1[3];
  /* metric (pvecmetric) */
  double psi, phi_prime, phi_prime_prime, omega_m1_prime, gamma_m2_prime_prime;
  double phi_prime_poisson, phi_prime_longitudinal;
  song2_triplet_stats st;
  /* outputs */
  double *src_flat;
  int64_t pair_off, per_type;
  int k3_size;
  double *fo_out;
  int fo_tau_size;
  /* evolver scratch */
  double *J, *M, *dif, *ytmp, *dytmp, *rhs, *del, *invwt, *psiv, *difkp1, *ynew, *ylin, *dylin;
  int *piv;
  int nmax;
} ws_t;

#define RLIST(X) X(rot1) X(rot2) X(rot1m) X(rot2m)
#define CLIST(X) X(cm12) X(cm21) X(cp12) X(cp21) X(cm11) X(cm22) X(cp11) X(cp22) X(dm12) X(dm21) X(dp12) X(dp21) \
  X(dm11) X(dm22) X(dp11) X(dp22) X(dz12) X(dz21) X(dz11) X(dz22)

static int nlm_hier_b(const cfg_t *c) {
  int n = 0;
  for (int i = 0; i < c->m_size; ++i) {
    if (c->m[i] == 0) ++n;  /* (0,0,0) */
    if (c->m[i] <= 1) ++n;  /* (1,1,m) */
  }
  return n;
}

static ws_t *ws_alloc(cfg_t *c) {
  ws_t *w = (ws_t *)calloc(1, sizeof(ws_t));
  w->c = c;
#define A1(x) w->x = (double *)calloc((size_t)c->n_lmq, sizeof(double));
  RLIST(A1)
#undef A1
#define A2(x) w->x = (double *)calloc((size_t)c->n_lm, sizeof(double));
  CLIST(A2)
#undef A2
  w->fo1 = (double *)calloc((size_t)c->nfo, sizeof(double));
  w->fo2 = (double *)calloc((size_t)c->nfo, sizeof(double));
  const song2_spec *s = c->s;
  w->l_max_g = s->l_max_g; w->l_max_pol_g = s->l_max_pol_g; w->l_max_ur = s->l_max_ur;
  /* quadratic-source layout (perturb2_workspace_init, perturbations2.c:4370-4560) */
  int q = 0;
  w->iq_g = q; q += size_l_indexm(c, w->l_max_g);
  w->iq_E = q; if (s->has_polarization2) q += size_l_indexm(c, w->l_max_pol_g);
  w->iq_B = q; if (s->has_polarization2) q += size_l_indexm(c, w->l_max_pol_g);
  w->iq_ur = q; q += size_l_indexm(c, w->l_max_ur);
  w->iq_b = q; q += nlm_hier_b(c);
  w->iq_cdm = q; q += nlm_hier_b(c);
  w->iq_psi = q++; w->iq_psi_prime = q++; w->iq_phi_prime_poisson = q++; w->iq_phi_prime_longitudinal = q++;
  w->iq_phi_prime_prime = q++; w->iq_omega_m1_prime = q++; w->iq_gamma_m2_prime_prime = q++;
  w->iq_vv_g = q++; w->iq_vv_ur = q++; w->iq_dd_b = q++; w->iq_vv_b = q++; w->iq_vv_cdm = q++;
  w->iq_vvp_b = q++; w->iq_vvp_cdm = q++;
  w->qs2_size = q;
  w->qs = (double *)calloc((size_t)q, sizeof(double));
  w->qc = (double *)calloc((size_t)q, sizeof(double));
  {
    int nn = c->t ? (c->t->fo_tau_size > 2 ? c->t->fo_tau_size : 2) : 2;
    w->qtab = (double *)calloc((size_t)nn * 2 * q, sizeof(double));
    w->qt_c = (double *)calloc((size_t)nn, sizeof(double));
  }
  int nmax = 4 * size_l_indexm(c, c->L_big) + 2 * nlm_hier_b(c) + 8;
  w->nmax = nmax;
  w->J = (double *)calloc((size_t)nmax * nmax, sizeof(double));
  w->M = (double *)calloc((size_t)nmax * nmax, sizeof(double));
  w->dif = (double *)calloc((size_t)nmax * 7, sizeof(double));
  w->ytmp = (double *)calloc(nmax, sizeof(double));
  w->dytmp = (double *)calloc(nmax, sizeof(double));
  w->rhs = (double *)calloc(nmax, sizeof(double));
  w->del = (double *)calloc(nmax, sizeof(double));
  w->invwt = (double *)calloc(nmax, sizeof(double));
  w->psiv = (double *)calloc(nmax, sizeof(double));
  w->difkp1 = (double *)calloc(nmax, sizeof(double));
  w->ynew = (double *)calloc(nmax, sizeof(double));
  w->ylin = (double *)calloc(nmax, sizeof(double));
  w->dylin = (double *)calloc(nmax, sizeof(double));
  w->piv = (int *)calloc(nmax, sizeof(int));
  return w;
}

static void ws_free(ws_t *w) {
#define F1(x) free(w->x);
  RLIST(F1) CLIST(F1)
#undef F1
  free(w->fo1); free(w->fo2); free(w->qs); free(w->qc); free(w->qtab); free(w->qt_c);
  free(w->J); free(w->M); free(w->dif); free(w->ytmp); free(w->dytmp); free(w->rhs); free(w->del);
  free(w->invwt); free(w->psiv); free(w->difkp1); free(w->ynew); free(w->ylin); free(w->dylin); free(w->piv);
  free(w);
}

/* ------------------------------------------------------------ accessors */

#define PV (&w->pv)
#define I(l, m) ((((l) > PV->l_max_g) || (abs(m) > (l)) || ((l) < 0)) ? 0.0 : y[PV->idx_g + LM(l, m)])
#define E(l, m) ((!c->s->has_polarization2 || ((l) > PV->l_max_pol_g) || (abs(m) > (l)) || ((l) < 0)) ? 0.0 : y[PV->idx_E + LM(l, m)])
#define B(l, m) ((!c->s->has_polarization2 || ((l) > PV->l_max_pol_g) || (abs(m) > (l)) || ((l) < 0)) ? 0.0 : y[PV->idx_B + LM(l, m)])
#define N(l, m) ((((l) > PV->l_max_ur) || (abs(m) > (l)) || ((l) < 0)) ? 0.0 : y[PV->idx_ur + LM(l, m)])
#define NLM(n, l, m) (c->nlm_array[(n)][(l)][c->index_m[(m)]])
#define b(n, l, m) ((((n) > PV->n_max_b) || ((l) > PV->l_max_b) || (abs(m) > (l)) || ((l) < 0)) ? 0.0 : y[PV->idx_b + NLM(n, l, m)])
#define cdm(n, l, m) ((((n) > PV->n_max_cdm) || ((l) > PV->l_max_cdm) || (abs(m) > (l)) || ((l) < 0)) ? 0.0 : y[PV->idx_cdm + NLM(n, l, m)])
#define dI(l, m) dy[PV->idx_g + LM(l, m)]
#define dE(l, m) dy[PV->idx_E + LM(l, m)]
#define dB(l, m) dy[PV->idx_B + LM(l, m)]
#define dN(l, m) dy[PV->idx_ur + LM(l, m)]
#define db(n, l, m) dy[PV->idx_b + NLM(n, l, m)]
#define dcdm(n, l, m) dy[PV->idx_cdm + NLM(n, l, m)]

#define c_minus(l, m1, m) (c->cmin[LM(l, m) * 3 + (m) - (m1) + 1])
#define c_plus(l, m1, m) (c->cplu[LM(l, m) * 3 + (m) - (m1) + 1])
#define d_minus(l, m1, m) (c->dmin[LM(l, m) * 3 + (m) - (m1) + 1])
#define d_plus(l, m1, m) (c->dplu[LM(l, m) * 3 + (m) - (m1) + 1])
#define d_zero(l, m1, m) (c->dzer[LM(l, m) * 3 + (m) - (m1) + 1])

#define rot_1(l, m) ((((l) < 0) || (abs(m) > (l))) ? 0.0 : ((m) < 0 ? w->rot1m[LMQ(l, abs(m))] : w->rot1[LMQ(l, m)]))
#define rot_2(l, m) ((((l) < 0) || (abs(m) > (l))) ? 0.0 : ((m) < 0 ? w->rot2m[LMQ(l, abs(m))] : w->rot2[LMQ(l, m)]))

#define I_1_raw(l) ((l) < 0 ? 0.0 : fo1[SONG2_FO_I + (l)])
#define I_2_raw(l) ((l) < 0 ? 0.0 : fo2[SONG2_FO_I + (l)])
#define E_1_raw(l) ((((l) < 0) || !c->s->has_polarization2) ? 0.0 : fo1[c->fo_E + (l)])
#define E_2_raw(l) ((((l) < 0) || !c->s->has_polarization2) ? 0.0 : fo2[c->fo_E + (l)])
#define N_1_raw(l) ((l) < 0 ? 0.0 : fo1[c->fo_N + (l)])
#define N_2_raw(l) ((l) < 0 ? 0.0 : fo2[c->fo_N + (l)])
#define I_1(l, m) (rot_1(l, m) * I_1_raw(l))
#define I_2(l, m) (rot_2(l, m) * I_2_raw(l))
#define E_1(l, m) (rot_1(l, m) * E_1_raw(l))
#define E_2(l, m) (rot_2(l, m) * E_2_raw(l))
#define N_1(l, m) (rot_1(l, m) * N_1_raw(l))
#define N_2(l, m) (rot_2(l, m) * N_2_raw(l))

#define dI_qs2(l, m) w->qs[w->iq_g + LM(l, m)]
#define dE_qs2(l, m) w->qs[w->iq_E + LM(l, m)]
#define dB_qs2(l, m) w->qs[w->iq_B + LM(l, m)]
#define dN_qs2(l, m) w->qs[w->iq_ur + LM(l, m)]
#define db_qs2(n, l, m) w->qs[w->iq_b + NLM(n, l, m)]
#define dcdm_qs2(n, l, m) w->qs[w->iq_cdm + NLM(n, l, m)]
#define dI_qc2(l, m) w->qc[w->iq_g + LM(l, m)]
#define dE_qc2(l, m) w->qc[w->iq_E + LM(l, m)]
#define dB_qc2(l, m) w->qc[w->iq_B + LM(l, m)]
#define db_qc2(n, l, m) w->qc[w->iq_b + NLM(n, l, m)]

#define c_minus_12(l, m) w->cm12[LM(l, m)]
#define c_minus_21(l, m) w->cm21[LM(l, m)]
#define c_plus_12(l, m) w->cp12[LM(l, m)]
#define c_plus_21(l, m) w->cp21[LM(l, m)]
#define c_minus_11(l, m) w->cm11[LM(l, m)]
#define c_minus_22(l, m) w->cm22[LM(l, m)]
#define c_plus_11(l, m) w->cp11[LM(l, m)]
#define c_plus_22(l, m) w->cp22[LM(l, m)]
#define d_minus_12(l, m) w->dm12[LM(l, m)]
#define d_minus_21(l, m) w->dm21[LM(l, m)]
#define d_plus_12(l, m) w->dp12[LM(l, m)]
#define d_plus_21(l, m) w->dp21[LM(l, m)]
#define d_minus_11(l, m) w->dm11[LM(l, m)]
#define d_minus_22(l, m) w->dm22[LM(l, m)]
#define d_plus_11(l, m) w->dp11[LM(l, m)]
#define d_plus_22(l, m) w->dp22[LM(l, m)]
#define d_zero_12(l, m) w->dz12[LM(l, m)]
#define d_zero_21(l, m) w->dz21[LM(l, m)]
#define d_zero_11(l, m) w->dz11[LM(l, m)]
#define d_zero_22(l, m) w->dz22[LM(l, m)]
#define r_minus_12(l, m) ((l - 1) * c_minus_12(l, m))
#define r_minus_21(l, m) ((l - 1) * c_minus_21(l, m))
#define r_plus_12(l, m) (-(l + 2) * c_plus_12(l, m))
#define r_plus_21(l, m) (-(l + 2) * c_plus_21(l, m))
#define k_minus_12(l, m) ((l - 1) * d_minus_12(l, m))
#define k_minus_21(l, m) ((l - 1) * d_minus_21(l, m))
#define k_plus_12(l, m) (-(l + 2) * d_plus_12(l, m))
#define k_plus_21(l, m) (-(l + 2) * d_plus_21(l, m))
#define k_zero_12(l, m) (-d_zero_12(l, m))
#define k_zero_21(l, m) (-d_zero_21(l, m))

/* ======================================================= geometry */

/* sqrt((l-m)!/(l+m)!) P_l^m(x) with the Condon-Shortley phase, computed from the
   unnormalised upward recurrence and a log-factorial normalisation (an
   independent route from the device's normalised recurrence). */
static double legendre_norm_r(int l, int m, double x, int rescaled) {
  double s = sqrt(fmax(0.0, 1.0 - x * x));
  /* P_m^m = (-1)^m (2m-1)!! s^m, kept in log form with sign; rescaled: without s^m
     (plegendre_lm_rescaled, perturbations2.c:5641) */
  if (rescaled) s = 1.0;
  double logpmm = 0.0;
  for (int i = 1; i <= m; ++i) logpmm += log(2.0 * i - 1.0);
  double norm = 0.5 * (lfact(l - m) - lfact(l + m));
  if (l == m) {
    double v = (s == 0.0 && m > 0) ? 0.0 : exp(logpmm + norm + m * log(s > 0 ? s : 1.0));
    return (m % 2 ? -v : v);
  }
  /* recurrence on P_l^m / P_m^m to avoid overflow */
  double p0 = 1.0, p1 = x * (2.0 * m + 1.0), p2 = p1;
  for (int ll = m + 2; ll <= l; ++ll) {
    p2 = ((2.0 * ll - 1.0) * x * p1 - (ll + m - 1.0) * p0) / (ll - m);
    p0 = p1; p1 = p2;
  }
  double base = (s == 0.0 && m > 0) ? 0.0 : exp(logpmm + norm + m * log(s > 0 ? s : 1.0));
  double v = base * p2;
  return (m % 2 ? -v : v);
}

static double legendre_norm(int l, int m, double x) { return legendre_norm_r(l, m, x, 0); }

static int geometrical_corner(ws_t *w, int index_k1, int index_k2, int index_k3, const double *k3row) {
  cfg_t *c = w->c;
  const song2_spec *s = c->s;
  w->index_k1 = index_k1; w->index_k2 = index_k2; w->index_k3 = index_k3;
  double k1 = w->k1 = s->k[index_k1];
  double k2 = w->k2 = s->k[index_k2];
  double k = w->k = k3row[index_k3];
  double k_sq = w->k_sq = k * k;
  double cosk1k2 = w->cosk1k2 = (k_sq - k1 * k1 - k2 * k2) / (2 * k1 * k2);
  double cosk1k = w->cosk1k = (k1 + k2 * cosk1k2) / k;
  double cosk2k = w->cosk2k = (k2 + k1 * cosk1k2) / k;
  if (fabs(cosk1k2) > 1 || fabs(cosk1k) > 1 || fabs(cosk2k) > 1) return 1;
  w->k1_dot_k2 = k1 * k2 * cosk1k2;
  int rescale = s->rescale_cmb_sources && !c->first_order_mode;
  double sin1 = sqrt(fmax(0.0, 1.0 - cosk1k * cosk1k)), sin2 = sqrt(fmax(0.0, 1.0 - cosk2k * cosk2k));
  for (int l = 0; l <= c->Lq; ++l)
    for (int m = 0; m <= l; ++m) {
      double sg = (m % 2 ? -1.0 : 1.0);
      if (!rescale) {
        /* perturbations2.c:5604-5622 */
        double r1 = legendre_norm(l, m, cosk1k);
        double r2 = sg * legendre_norm(l, m, cosk2k);
        w->rot1[LMQ(l, m)] = r1;
        w->rot2[LMQ(l, m)] = r2;
        w->rot1m[LMQ(l, m)] = sg * r1;
        w->rot2m[LMQ(l, m)] = sg * r2;
      } else {
        /* perturbations2.c:5635-5652: P_lm / sin^m for m >= 0, (-1)^m P_lm sin^m for -m;
           (k1/k2)^(+-m) on the k2 side */
        w->rot1[LMQ(l, m)] = legendre_norm_r(l, m, cosk1k, 1);
        w->rot2[LMQ(l, m)] = sg * legendre_norm_r(l, m, cosk2k, 1) * pow(k1 / k2, m);
        w->rot1m[LMQ(l, m)] = sg * legendre_norm(l, m, cosk1k) * pow(sin1, m);
        w->rot2m[LMQ(l, m)] = sg * (sg * legendre_norm(l, m, cosk2k) * pow(sin2, m)) * pow(k1 / k2, -m);
      }
    }
  double k1_M1 = w->k1_m[0] = k1 * rot_1(1, -1);
  double k1_0 = w->k1_m[1] = k1 * rot_1(1, 0);
  double k1_P1 = w->k1_m[2] = k1 * rot_1(1, 1);
  double k2_M1 = w->k2_m[0] = k2 * rot_2(1, -1);
  double k2_0 = w->k2_m[1] = k2 * rot_2(1, 0);
  double k2_P1 = w->k2_m[2] = k2 * rot_2(1, 1);
  double k1_dot_k2 = w->k1_dot_k2;
  w->k1_ten_k2[0] = SQRT_2 / SQRT_3 * k1_M1 * k2_M1;
  w->k1_ten_k2[1] = (k1_M1 * k2_0 + k2_M1 * k1_0) / SQRT_3;
  w->k1_ten_k2[2] = k1_0 * k2_0 - k1_dot_k2 / 3.;
  w->k1_ten_k2[3] = (k1_P1 * k2_0 + k2_P1 * k1_0) / SQRT_3;
  w->k1_ten_k2[4] = SQRT_2 / SQRT_3 * k1_P1 * k2_P1;
  w->k1_ten_k1[0] = SQRT_2 / SQRT_3 * k1_M1 * k1_M1;
  w->k1_ten_k1[1] = (k1_M1 * k1_0 + k1_M1 * k1_0) / SQRT_3;
  w->k1_ten_k1[2] = k1_0 * k1_0 - k1 * k1 / 3.;
  w->k1_ten_k1[3] = (k1_P1 * k1_0 + k1_P1 * k1_0) / SQRT_3;
  w->k1_ten_k1[4] = SQRT_2 / SQRT_3 * k1_P1 * k1_P1;
  w->k2_ten_k2[0] = SQRT_2 / SQRT_3 * k2_M1 * k2_M1;
  w->k2_ten_k2[1] = (k2_M1 * k2_0 + k2_M1 * k2_0) / SQRT_3;
  w->k2_ten_k2[2] = k2_0 * k2_0 - k2 * k2 / 3.;
  w->k2_ten_k2[3] = (k2_P1 * k2_0 + k2_P1 * k2_0) / SQRT_3;
  w->k2_ten_k2[4] = SQRT_2 / SQRT_3 * k2_P1 * k2_P1;
  for (int l = 0; l <= c->L_big; ++l)
    for (int im = 0; im <= c->index_m_max[l]; ++im) {
      int m = c->m[im];
      int lm = LM(l, m);
      double a[20] = {0};
      for (int m2 = -1; m2 <= 1; ++m2) {
        int m1 = m - m2;
        double cm = c->cmin[lm * 3 + m - m1 + 1], cp = c->cplu[lm * 3 + m - m1 + 1];
        double dm = c->dmin[lm * 3 + m - m1 + 1], dp = c->dplu[lm * 3 + m - m1 + 1];
        double dz = c->dzer[lm * 3 + m - m1 + 1];
        a[0] += rot_1(1, m2) * rot_2(l - 1, m1) * cm;
        a[1] += rot_2(1, m2) * rot_1(l - 1, m1) * cm;
        a[2] += rot_1(1, m2) * rot_2(l + 1, m1) * cp;
        a[3] += rot_2(1, m2) * rot_1(l + 1, m1) * cp;
        a[4] += rot_1(1, m2) * rot_1(l - 1, m1) * cm;
        a[5] += rot_2(1, m2) * rot_2(l - 1, m1) * cm;
        a[6] += rot_1(1, m2) * rot_1(l + 1, m1) * cp;
        a[7] += rot_2(1, m2) * rot_2(l + 1, m1) * cp;
        a[8] += rot_1(1, m2) * rot_2(l - 1, m1) * dm;
        a[9] += rot_2(1, m2) * rot_1(l - 1, m1) * dm;
        a[10] += rot_1(1, m2) * rot_2(l + 1, m1) * dp;
        a[11] += rot_2(1, m2) * rot_1(l + 1, m1) * dp;
        a[12] += rot_1(1, m2) * rot_1(l - 1, m1) * dm;
        a[13] += rot_2(1, m2) * rot_2(l - 1, m1) * dm;
        a[14] += rot_1(1, m2) * rot_1(l + 1, m1) * dp;
        a[15] += rot_2(1, m2) * rot_2(l + 1, m1) * dp;
        a[16] += rot_1(1, m2) * rot_2(l, m1) * dz;
        a[17] += rot_2(1, m2) * rot_1(l, m1) * dz;
        a[18] += rot_1(1, m2) * rot_1(l, m1) * dz;
        a[19] += rot_2(1, m2) * rot_2(l, m1) * dz;
      }
      w->cm12[lm] = a[0]; w->cm21[lm] = a[1]; w->cp12[lm] = a[2]; w->cp21[lm] = a[3];
      w->cm11[lm] = a[4]; w->cm22[lm] = a[5]; w->cp11[lm] = a[6]; w->cp22[lm] = a[7];
      w->dm12[lm] = a[8]; w->dm21[lm] = a[9]; w->dp12[lm] = a[10]; w->dp21[lm] = a[11];
      w->dm11[lm] = a[12]; w->dm22[lm] = a[13]; w->dp11[lm] = a[14]; w->dp22[lm] = a[15];
      w->dz12[lm] = a[16]; w->dz21[lm] = a[17]; w->dz11[lm] = a[18]; w->dz22[lm] = a[19];
    }
  return 0;
}

/* ======================================================= tables at tau */

static void background_at_tau(ws_t *w, double tau) {
  const song2_tables *t = w->c->t;
  double x = log(tau);
  w->tau = tau;
#define BG(q) spl(t->bg_size, SONG2_BG_SIZE, t->bg_lntau0, t->bg_dlntau, t->bg, t->bg_dd, (q), x)
  w->a = exp(BG(SONG2_BG_LN_A));
  w->a_sq = w->a * w->a;
  w->Hc = exp(BG(SONG2_BG_LN_HC));
  w->Hc_prime = BG(SONG2_BG_HC_PRIME_TAU2) / (tau * tau);
  w->rho_g = exp(BG(SONG2_BG_LN_RHO_G));
  w->rho_b = exp(BG(SONG2_BG_LN_RHO_B));
  w->rho_cdm = exp(BG(SONG2_BG_LN_RHO_CDM));
  w->rho_ur = exp(BG(SONG2_BG_LN_RHO_UR));
  w->kappa_dot = exp(BG(SONG2_BG_LN_KAPPA_DOT));
  w->exp_m_kappa = exp(-BG(SONG2_BG_KAPPA));
#undef BG
  w->g = w->kappa_dot * w->exp_m_kappa;
  w->r = w->rho_g / w->rho_b;
}

/* perturb_song_sources_at_tau_and_k: spline of the first-order table in ln tau */
static void first_order_at_tau(ws_t *w, double tau) {
  cfg_t *c = w->c;
  const song2_tables *t = c->t;
  if (w->linear_only || c->first_order_mode) {
    memset(w->fo1, 0, sizeof(double) * c->nfo);
    memset(w->fo2, 0, sizeof(double) * c->nfo);
    return;
  }
  double x = log(tau);
  size_t stride = (size_t)t->fo_tau_size * t->fo_size;
  const double *v1 = t->fo + stride * w->index_k1, *d1 = t->fo_dd + stride * w->index_k1;
  const double *v2 = t->fo + stride * w->index_k2, *d2 = t->fo_dd + stride * w->index_k2;
  for (int q = 0; q < c->nfo; ++q) {
    w->fo1[q] = spl(t->fo_tau_size, t->fo_size, t->fo_lntau0, t->fo_dlntau, v1, d1, q, x);
    w->fo2[q] = spl(t->fo_tau_size, t->fo_size, t->fo_lntau0, t->fo_dlntau, v2, d2, q, x);
  }
}

/* ======================================================= quadratic sources */

static void quadratic_sources(ws_t *w, int what) {
  cfg_t *c = w->c;
  const song2_spec *s = c->s;
  double *fo1 = w->fo1, *fo2 = w->fo2;
  if (w->linear_only || c->first_order_mode || !s->has_quadratic_sources) {
    if (what == QS_WHAT_TOTAL) memset(w->qs, 0, sizeof(double) * w->qs2_size);
    memset(w->qc, 0, sizeof(double) * w->qs2_size);
    return;
  }
  double k = w->k, k_sq = w->k_sq, k1 = w->k1, k2 = w->k2;
  double k1_dot_k2 = w->k1_dot_k2, k1_sq = k1 * k1, k2_sq = k2 * k2;
  double *k1_m = w->k1_m, *k2_m = w->k2_m, *k1_ten_k2 = w->k1_ten_k2, *k1_ten_k1 = w->k1_ten_k1,
         *k2_ten_k2 = w->k2_ten_k2;
  int l_max_g = w->l_max_g, l_max_pol_g = w->l_max_pol_g, l_max_ur = w->l_max_ur;
  double a_sq = w->a_sq, Hc = w->Hc, Hc_sq = Hc * Hc, Hc_prime = w->Hc_prime, kappa_dot = w->kappa_dot;
  double r = w->r;
  double delta_b_1 = fo1[SONG2_FO_DELTA_B], delta_b_2 = fo2[SONG2_FO_DELTA_B];
  double vpot_b_1 = fo1[SONG2_FO_V_B], vpot_b_2 = fo2[SONG2_FO_V_B];
  double delta_cdm_1 = fo1[SONG2_FO_DELTA_CDM], delta_cdm_2 = fo2[SONG2_FO_DELTA_CDM];
  double vpot_cdm_1 = fo1[SONG2_FO_V_CDM], vpot_cdm_2 = fo2[SONG2_FO_V_CDM];

  if (what == QS_WHAT_TOTAL) {
    memset(w->qs, 0, sizeof(double) * w->qs2_size);
    double rho_dipole_1 = 0, rho_dipole_2 = 0;
    if (c->compute_m[0]) {
      rho_dipole_1 = w->rho_g * I_1_raw(1) + w->rho_b * fo1[SONG2_FO_DIPOLE_B] + w->rho_cdm * fo1[SONG2_FO_DIPOLE_CDM] +
                     w->rho_ur * N_1_raw(1);
      rho_dipole_2 = w->rho_g * I_2_raw(1) + w->rho_b * fo2[SONG2_FO_DIPOLE_B] + w->rho_cdm * fo2[SONG2_FO_DIPOLE_CDM] +
                     w->rho_ur * N_2_raw(1);
    }
    double phi_1 = fo1[SONG2_FO_PHI], phi_2 = fo2[SONG2_FO_PHI];
    double psi_1 = fo1[SONG2_FO_PSI], psi_2 = fo2[SONG2_FO_PSI];
    double psi_prime_1 = fo1[SONG2_FO_PSI_P], psi_prime_2 = fo2[SONG2_FO_PSI_P];
    double phi_prime_1 = fo1[SONG2_FO_PHI_P], phi_prime_2 = fo2[SONG2_FO_PHI_P];
    double phi_prime_prime_1 = fo1[SONG2_FO_PHI_PP], phi_prime_prime_2 = fo2[SONG2_FO_PHI_PP];
    /* Einstein tensor, perturbations2.c:10905-11060 */
    if (c->compute_m[0]) {
      double Q_TT = -12 * psi_1 * psi_2 * Hc_sq + phi_1 * phi_2 * (3 * k1_dot_k2 + 4 * k1_sq + 4 * k2_sq) +
                    6 * phi_prime_2 * (phi_1 - psi_1) * Hc + 6 * phi_prime_1 * (phi_2 - psi_2) * Hc -
                    3 * phi_prime_1 * phi_prime_2;
      double Q_ST = +2 * psi_1 * psi_2 * Hc * (k1_m[1] + k2_m[1]) - 2 * psi_1 * phi_2 * Hc * (k1_m[1]) -
                    2 * psi_2 * phi_1 * Hc * (+k2_m[1]) - 2 * phi_1 * phi_prime_2 * (k1_m[1] + 2 * k2_m[1]) -
                    2 * phi_2 * phi_prime_1 * (2 * k1_m[1] + k2_m[1]) + psi_1 * phi_prime_2 * (k1_m[1]) +
                    psi_2 * phi_prime_1 * (k2_m[1]) +
                    0.5 * a_sq * (k1_m[1] / k1 * rho_dipole_1 * (psi_2 + phi_2) + k2_m[1] / k2 * rho_dipole_2 * (psi_1 + phi_1));
      double Q_TR = -12 * psi_1 * psi_2 * (Hc * Hc + 2 * Hc_prime) + psi_1 * psi_2 * (k_sq + k1_sq + k2_sq) +
                    phi_1 * phi_2 * (3 * k1_dot_k2 + 4 * k1_sq + 4 * k2_sq) + phi_1 * psi_2 * (k1_dot_k2 - 2 * k2_sq) +
                    phi_2 * psi_1 * (k1_dot_k2 - 2 * k1_sq) +
                    6 * (phi_prime_prime_2 + 2 * Hc * phi_prime_2) * (phi_1 - psi_1) +
                    6 * (phi_prime_prime_1 + 2 * Hc * phi_prime_1) * (phi_2 - psi_2) -
                    3 * psi_prime_2 * (4 * Hc * psi_1 + phi_prime_1) - 3 * psi_prime_1 * (4 * Hc * psi_2 + phi_prime_2) +
                    3 * phi_prime_1 * phi_prime_2;
      double Q_SS = phi_1 * phi_2 * (-3 * k1_ten_k2[2] - 2 * k1_ten_k1[2] - 2 * k2_ten_k2[2]) +
                    psi_1 * psi_2 * (-k1_ten_k2[2] - k1_ten_k1[2] - k2_ten_k2[2]) +
                    psi_1 * phi_2 * (k1_ten_k2[2] + k1_ten_k1[2]) + psi_2 * phi_1 * (k1_ten_k2[2] + k2_ten_k2[2]);
      double Q_SS_prime =
          (phi_prime_1 * phi_2 + phi_1 * phi_prime_2) * (-3 * k1_ten_k2[2] - 2 * k1_ten_k1[2] - 2 * k2_ten_k2[2]) +
          (psi_prime_1 * psi_2 + psi_1 * psi_prime_2) * (-k1_ten_k2[2] - k1_ten_k1[2] - k2_ten_k2[2]) +
          (psi_prime_1 * phi_2 + psi_1 * phi_prime_2) * (k1_ten_k2[2] + k1_ten_k1[2]) +
          (psi_prime_2 * phi_1 + psi_2 * phi_prime_1) * (k1_ten_k2[2] + k2_ten_k2[2]);
      Q_TT *= 2; Q_ST *= 2; Q_TR *= 2; Q_SS *= 2; Q_SS_prime *= 2;
      w->qs[w->iq_phi_prime_poisson] = -Q_TT / (6 * Hc);
      w->qs[w->iq_phi_prime_longitudinal] = Q_ST / (2 * k);
      w->qs[w->iq_psi] = -Q_SS * 3 / (2 * k_sq);
      w->qs[w->iq_psi_prime] = -Q_SS_prime * 3 / (2 * k_sq) - Q_SS * 3 * Hc / k_sq;
      w->qs[w->iq_phi_prime_prime] = -(Q_TR + Q_TT) / 6;
    }
    if (c->compute_m[1]) {
      double Q_SS = phi_1 * phi_2 * (-3 * k1_ten_k2[3] - 2 * k1_ten_k1[3] - 2 * k2_ten_k2[3]) +
                    psi_1 * psi_2 * (-k1_ten_k2[3] - k1_ten_k1[3] - k2_ten_k2[3]) +
                    psi_1 * phi_2 * (k1_ten_k2[3] + k1_ten_k1[3]) + psi_2 * phi_1 * (k1_ten_k2[3] + k2_ten_k2[3]);
      Q_SS *= 2;
      w->qs[w->iq_omega_m1_prime] = SQRT_3 / k * Q_SS;
    }
    if (c->compute_m[2]) {
      double Q_SS = phi_1 * phi_2 * (-3 * k1_ten_k2[4] - 2 * k1_ten_k1[4] - 2 * k2_ten_k2[4]) +
                    psi_1 * psi_2 * (-k1_ten_k2[4] - k1_ten_k1[4] - k2_ten_k2[4]) +
                    psi_1 * phi_2 * (k1_ten_k2[4] + k1_ten_k1[4]) + psi_2 * phi_1 * (k1_ten_k2[4] + k2_ten_k2[4]);
      Q_SS *= 2;
      w->qs[w->iq_gamma_m2_prime_prime] = -Q_SS;
    }
    /* Liouville operator, perturbations2.c:11068-11303 */
    if (s->has_quadratic_liouville) {
      for (int l = 0; l <= l_max_g; ++l)
        for (int im = 0; im <= c->index_m_max[l]; ++im) {
          int m = c->m[im];
          double v = 0;
          if (l == 0) v = -8 * (phi_1 * phi_prime_2 + phi_2 * phi_prime_1);
          if (l == 1) v = 4 * (k1_m[m + 1] * psi_1 * (psi_2 - phi_2) + k2_m[m + 1] * psi_2 * (psi_1 - phi_1));
          v += I_2_raw(l + 1) * c_plus_22(l, m) * k2 * (phi_1 + psi_1) - I_2_raw(l - 1) * c_minus_22(l, m) * k2 * (phi_1 + psi_1) +
               I_1_raw(l + 1) * c_plus_11(l, m) * k1 * (phi_2 + psi_2) - I_1_raw(l - 1) * c_minus_11(l, m) * k1 * (phi_2 + psi_2);
          v += -4 * phi_prime_1 * I_2(l, m) + I_2_raw(l + 1) * 4 * c_plus_12(l, m) * k1 * psi_1 -
               I_2_raw(l - 1) * 4 * c_minus_12(l, m) * k1 * psi_1 - 4 * phi_prime_2 * I_1(l, m) +
               I_1_raw(l + 1) * 4 * c_plus_21(l, m) * k2 * psi_2 - I_1_raw(l - 1) * 4 * c_minus_21(l, m) * k2 * psi_2;
          v += I_2_raw(l + 1) * r_plus_12(l, m) * k1 * (phi_1 + psi_1) - I_2_raw(l - 1) * r_minus_12(l, m) * k1 * (phi_1 + psi_1) +
               I_1_raw(l + 1) * r_plus_21(l, m) * k2 * (phi_2 + psi_2) - I_1_raw(l - 1) * r_minus_21(l, m) * k2 * (phi_2 + psi_2);
          dI_qs2(l, m) = -v;
        }
      if (s->has_polarization2)
        for (int l = 2; l <= l_max_pol_g; ++l)
          for (int im = 0; im <= c->index_m_max[l]; ++im) {
            int m = c->m[im];
            double e = -4 * phi_prime_1 * E_2(l, m) +
                       E_2_raw(l + 1) * (k_plus_12(l, m) * k1 * (phi_1 + psi_1) + d_plus_22(l, m) * k2 * (phi_1 + psi_1) +
                                         4 * d_plus_12(l, m) * k1 * psi_1) -
                       E_2_raw(l - 1) * (k_minus_12(l, m) * k1 * (phi_1 + psi_1) + d_minus_22(l, m) * k2 * (phi_1 + psi_1) +
                                         4 * d_minus_12(l, m) * k1 * psi_1) -
                       4 * phi_prime_2 * E_1(l, m) +
                       E_1_raw(l + 1) * (k_plus_21(l, m) * k2 * (phi_2 + psi_2) + d_plus_11(l, m) * k1 * (phi_2 + psi_2) +
                                         4 * d_plus_21(l, m) * k2 * psi_2) -
                       E_1_raw(l - 1) * (k_minus_21(l, m) * k2 * (phi_2 + psi_2) + d_minus_11(l, m) * k1 * (phi_2 + psi_2) +
                                         4 * d_minus_21(l, m) * k2 * psi_2);
            double bb = -E_2_raw(l) * (k_zero_12(l, m) * k1 * (phi_1 + psi_1) + d_zero_22(l, m) * k2 * (phi_1 + psi_1) +
                                       4 * d_zero_12(l, m) * k1 * psi_1) -
                        E_1_raw(l) * (k_zero_21(l, m) * k2 * (phi_2 + psi_2) + d_zero_11(l, m) * k1 * (phi_2 + psi_2) +
                                      4 * d_zero_21(l, m) * k2 * psi_2);
            dE_qs2(l, m) = -e;
            dB_qs2(l, m) = -bb;
          }
      if (c->compute_m[0])
        db_qs2(0, 0, 0) = 2 * k1_dot_k2 * (psi_1 - phi_1) * vpot_b_2 + k2_sq * (phi_1 + psi_1) * vpot_b_2 +
                          3 * phi_prime_1 * (delta_b_2 + 2 * phi_2) + 2 * k1_dot_k2 * (psi_2 - phi_2) * vpot_b_1 +
                          k1_sq * (phi_2 + psi_2) * vpot_b_1 + 3 * phi_prime_2 * (delta_b_1 + 2 * phi_1);
      for (int im = 0; im <= c->index_m_max[1]; ++im) {
        int m = c->m[im];
        db_qs2(1, 1, m) = 3 * k1_m[m + 1] * (delta_b_2 * psi_1 - 4 * vpot_b_1 * phi_prime_2 + phi_2 * psi_1) +
                          3 * k2_m[m + 1] * (delta_b_1 * psi_2 - 4 * vpot_b_2 * phi_prime_1 + phi_1 * psi_2) -
                          3 * psi_1 * psi_2 * (k1_m[m + 1] + k2_m[m + 1]);
      }
      if (c->compute_m[0])
        dcdm_qs2(0, 0, 0) = 2 * k1_dot_k2 * (psi_1 - phi_1) * vpot_cdm_2 + k2_sq * (phi_1 + psi_1) * vpot_cdm_2 +
                            3 * phi_prime_1 * (delta_cdm_2 + 2 * phi_2) + 2 * k1_dot_k2 * (psi_2 - phi_2) * vpot_cdm_1 +
                            k1_sq * (phi_2 + psi_2) * vpot_cdm_1 + 3 * phi_prime_2 * (delta_cdm_1 + 2 * phi_1);
      for (int im = 0; im <= c->index_m_max[1]; ++im) {
        int m = c->m[im];
        dcdm_qs2(1, 1, m) = 3 * k1_m[m + 1] * (delta_cdm_2 * psi_1 - 4 * vpot_cdm_1 * phi_prime_2 + phi_2 * psi_1) +
                            3 * k2_m[m + 1] * (delta_cdm_1 * psi_2 - 4 * vpot_cdm_2 * phi_prime_1 + phi_1 * psi_2) -
                            3 * psi_1 * psi_2 * (k1_m[m + 1] + k2_m[m + 1]);
      }
      for (int l = 0; l <= l_max_ur; ++l)
        for (int im = 0; im <= c->index_m_max[l]; ++im) {
          int m = c->m[im];
          double v = 0;
          if (l == 0) v = -8 * phi_1 * phi_prime_2 - 8 * phi_2 * phi_prime_1;
          if (l == 1) v = 4 * (k1_m[m + 1] * psi_1 * (psi_2 - phi_2) + k2_m[m + 1] * psi_2 * (psi_1 - phi_1));
          v += -4 * phi_prime_1 * N_2(l, m) +
               N_2_raw(l + 1) * (r_plus_12(l, m) * k1 * (phi_1 + psi_1) + c_plus_22(l, m) * k2 * (phi_1 + psi_1) +
                                 4 * c_plus_12(l, m) * k1 * psi_1) -
               N_2_raw(l - 1) * (r_minus_12(l, m) * k1 * (phi_1 + psi_1) + c_minus_22(l, m) * k2 * (phi_1 + psi_1) +
                                 4 * c_minus_12(l, m) * k1 * psi_1) -
               4 * phi_prime_2 * N_1(l, m) +
               N_1_raw(l + 1) * (r_plus_21(l, m) * k2 * (phi_2 + psi_2) + c_plus_11(l, m) * k1 * (phi_2 + psi_2) +
                                 4 * c_plus_21(l, m) * k2 * psi_2) -
               N_1_raw(l - 1) * (r_minus_21(l, m) * k2 * (phi_2 + psi_2) + c_minus_11(l, m) * k1 * (phi_2 + psi_2) +
                                 4 * c_minus_21(l, m) * k2 * psi_2);
          dN_qs2(l, m) = -v;
        }
    }
  }

  /* Collision term, perturbations2.c:11313-11783 */
  memset(w->qc, 0, sizeof(double) * w->qs2_size);
  if (s->has_quadratic_collision) {
    double u_b_1[3] = {0}, u_b_2[3] = {0};
    for (int im = 0; im <= c->index_m_max[1]; ++im) {
      int m = c->m[im];
      u_b_1[m] = -k1_m[m + 1] * vpot_b_1;
      u_b_2[m] = -k2_m[m + 1] * vpot_b_2;
    }
    double v_0_1 = -k1 * vpot_b_1, v_0_2 = -k2 * vpot_b_2;
    double A_1 = fo1[SONG2_FO_PSI], A_2 = fo2[SONG2_FO_PSI];
    double delta_e_1 = delta_b_1, delta_e_2 = delta_b_2;
    double c_1 = 0, c_2 = 0;
    if (c->compute_m[0]) {
      double vpot_g_1 = fo1[SONG2_FO_V_G], vpot_g_2 = fo2[SONG2_FO_V_G];
      dI_qc2(0, 0) = FOUR_THIRDS * k1_dot_k2 * (vpot_b_1 * (vpot_g_2 - vpot_b_2) + vpot_b_2 * (vpot_g_1 - vpot_b_1));
    }
    for (int l = 1; l <= l_max_g; ++l)
      for (int im = 0; im <= c->index_m_max[l]; ++im) {
        int m = c->m[im];
        if (l == 1) {
          c_1 = 4 * u_b_1[m] - I_1(1, m);
          c_2 = 4 * u_b_2[m] - I_2(1, m);
          dI_qc2(1, m) = 3 * (c_minus_12(1, m) * v_0_1 * I_2_raw(0) + c_minus_21(1, m) * v_0_2 * I_1_raw(0));
          dI_qc2(1, m) += -4 * (delta_b_1 * u_b_2[m] + delta_b_2 * u_b_1[m]);
        }
        if (l == 2) {
          c_1 = -I_1(2, m) + 0.1 * (I_1(2, m) - SQRT_6 * E_1(2, m));
          c_2 = -I_2(2, m) + 0.1 * (I_2(2, m) - SQRT_6 * E_2(2, m));
          dI_qc2(2, m) = c_minus_12(2, m) * v_0_1 * (7 * v_0_2 - 0.5 * I_2_raw(1)) +
                         c_minus_21(2, m) * v_0_2 * (7 * v_0_1 - 0.5 * I_1_raw(1));
        }
        if (l == 3) {
          c_1 = -I_1(3, m);
          c_2 = -I_2(3, m);
          dI_qc2(3, m) = 0.5 * (c_minus_12(3, m) * v_0_1 * (I_2_raw(2) - SQRT_6 * E_2_raw(2)) +
                                c_minus_21(3, m) * v_0_2 * (I_1_raw(2) - SQRT_6 * E_1_raw(2)));
        }
        if (l > 3) {
          c_1 = -I_1(l, m);
          c_2 = -I_2(l, m);
        }
        double loss = (A_1 + delta_e_1) * c_2 + (A_2 + delta_e_2) * c_1 + c_minus_12(l, m) * v_0_1 * I_2_raw(l - 1) -
                      c_plus_12(l, m) * v_0_1 * I_2_raw(l + 1) + c_minus_21(l, m) * v_0_2 * I_1_raw(l - 1) -
                      c_plus_21(l, m) * v_0_2 * I_1_raw(l + 1);
        dI_qc2(l, m) += loss;
      }
    if (s->has_polarization2) {
      for (int l = 2; l <= l_max_pol_g; ++l)
        for (int im = 0; im <= c->index_m_max[l]; ++im) {
          int m = c->m[im];
          if (l == 2) {
            c_1 = -E_1(2, m) - SQRT_6 * 0.1 * (I_1(2, m) - SQRT_6 * E_1(2, m));
            c_2 = -E_2(2, m) - SQRT_6 * 0.1 * (I_2(2, m) - SQRT_6 * E_2(2, m));
            dE_qc2(2, m) = 0.5 * SQRT_6 *
                           (c_minus_12(2, m) * v_0_1 * (I_2_raw(1) - 2 * v_0_2) + c_minus_21(2, m) * v_0_2 * (I_1_raw(1) - 2 * v_0_1));
          }
          if (l == 3) {
            c_1 = -E_1(3, m);
            c_2 = -E_2(3, m);
            dE_qc2(3, m) = -0.5 * SQRT_6 *
                           (d_minus_12(3, m) * v_0_1 * (I_2_raw(2) - SQRT_6 * E_2_raw(2)) +
                            d_minus_21(3, m) * v_0_2 * (I_1_raw(2) - SQRT_6 * E_1_raw(2)));
          }
          if (l > 3) {
            c_1 = -E_1(l, m);
            c_2 = -E_2(l, m);
          }
          double loss = (A_1 + delta_e_1) * c_2 + (A_2 + delta_e_2) * c_1 + d_minus_12(l, m) * v_0_1 * E_2_raw(l - 1) -
                        d_plus_12(l, m) * v_0_1 * E_2_raw(l + 1) + d_minus_21(l, m) * v_0_2 * E_1_raw(l - 1) -
                        d_plus_21(l, m) * v_0_2 * E_1_raw(l + 1);
          dE_qc2(l, m) += loss;
        }
      for (int l = 2; l <= l_max_pol_g; ++l)
        for (int im = 0; im <= c->index_m_max[l]; ++im) {
          int m = c->m[im];
          if (l == 2)
            dB_qc2(2, m) = -0.2 * SQRT_6 *
                           (d_zero_12(2, m) * v_0_1 * (I_2_raw(2) - SQRT_6 * E_2_raw(2)) +
                            d_zero_21(2, m) * v_0_2 * (I_1_raw(2) - SQRT_6 * E_1_raw(2)));
          dB_qc2(l, m) += d_zero_12(l, m) * v_0_1 * E_2_raw(l) + d_zero_21(l, m) * v_0_2 * E_1_raw(l);
        }
    }
    if (c->compute_m[0]) db_qc2(0, 0, 0) = -r * dI_qc2(0, 0);
    for (int im = 0; im <= c->index_m_max[1]; ++im) db_qc2(1, 1, c->m[im]) = -r * dI_qc2(1, c->m[im]);
    for (int q = 0; q < w->qs2_size; ++q) {
      w->qc[q] *= kappa_dot;
      if (what == QS_WHAT_TOTAL) w->qs[q] += w->qc[q];
    }
  }
  /* products needed later (perturbations2.c:11795-11809), and the time derivatives
     of the velocity products used by psi' (perturbations2.c:10312-10340) */
  if (what == QS_WHAT_TOTAL) {
    w->qs[w->iq_vv_g] = fo1[SONG2_FO_V_G] * fo2[SONG2_FO_V_G];
    w->qs[w->iq_vv_ur] = fo1[SONG2_FO_V_UR] * fo2[SONG2_FO_V_UR];
    w->qs[w->iq_dd_b] = delta_b_1 * delta_b_2;
    w->qs[w->iq_vv_b] = vpot_b_1 * vpot_b_2;
    w->qs[w->iq_vv_cdm] = vpot_cdm_1 * vpot_cdm_2;
    w->qs[w->iq_vvp_b] = fo1[SONG2_FO_V_B_P] * vpot_b_2 + vpot_b_1 * fo2[SONG2_FO_V_B_P];
    w->qs[w->iq_vvp_cdm] = fo1[SONG2_FO_V_CDM_P] * vpot_cdm_2 + vpot_cdm_1 * fo2[SONG2_FO_V_CDM_P];
  }
}

/* ======================================================= workspace at tau */

static void tca_variables(ws_t *w, const double *y) {
  cfg_t *c = w->c;
  const song2_spec *s = c->s;
  double *fo1 = w->fo1, *fo2 = w->fo2;
  double k = w->k, Hc = w->Hc, r = w->r, kappa_dot = w->kappa_dot, tau_c = 1 / kappa_dot;
  double *k1_m = w->k1_m, *k2_m = w->k2_m, k1_dot_k2 = w->k1_dot_k2, *k1_ten_k2 = w->k1_ten_k2;
  /* perturb2_fluid_variables (perturbations2.c:9108-9338), only what the TCA uses */
  double vpot_g_1 = fo1[SONG2_FO_V_G], vpot_g_2 = fo2[SONG2_FO_V_G];
  double delta_g_1 = fo1[SONG2_FO_DELTA_G], delta_g_2 = fo2[SONG2_FO_DELTA_G];
  double v_dot_v_g = -k1_dot_k2 * vpot_g_1 * vpot_g_2;
  double delta_g = w->I_00 - 8 / 3. * v_dot_v_g;
  double u_g_1[3] = {0}, u_g_2[3] = {0}, v_ten_v_g[3] = {0};
  for (int im = 0; im <= c->index_m_max[1]; ++im) {
    int m = c->m[im];
    u_g_1[m] = -k1_m[m + 1] * vpot_g_1;
    u_g_2[m] = -k2_m[m + 1] * vpot_g_2;
  }
  for (int im = 0; im <= c->index_m_max[2]; ++im) {
    int m = c->m[im];
    v_ten_v_g[m] = -k1_ten_k2[m + 2] * vpot_g_1 * vpot_g_2;
  }
  double vpot_b_1 = fo1[SONG2_FO_V_B], vpot_b_2 = fo2[SONG2_FO_V_B];
  double vpot_b_1_prime = fo1[SONG2_FO_V_B_P], vpot_b_2_prime = fo2[SONG2_FO_V_B_P];
  double delta_b_1 = fo1[SONG2_FO_DELTA_B], delta_b_2 = fo2[SONG2_FO_DELTA_B];
  double delta_b_1_prime = fo1[SONG2_FO_DELTA_B_P], delta_b_2_prime = fo2[SONG2_FO_DELTA_B_P];
  double u_b_1[3] = {0}, u_b_2[3] = {0}, u_b_1_prime[3] = {0}, u_b_2_prime[3] = {0}, u_b[3] = {0};
  double v_ten_v_b[3] = {0}, v_ten_v_b_prime[3] = {0};
  for (int im = 0; im <= c->index_m_max[1]; ++im) {
    int m = c->m[im];
    u_b_1[m] = -k1_m[m + 1] * vpot_b_1;
    u_b_2[m] = -k2_m[m + 1] * vpot_b_2;
    u_b_1_prime[m] = -k1_m[m + 1] * vpot_b_1_prime;
    u_b_2_prime[m] = -k2_m[m + 1] * vpot_b_2_prime;
    u_b[m] = b(1, 1, m) / 3 - delta_b_1 * u_b_2[m] - delta_b_2 * u_b_1[m];
  }
  for (int im = 0; im <= c->index_m_max[2]; ++im) {
    int m = c->m[im];
    v_ten_v_b[m] = -k1_ten_k2[m + 2] * vpot_b_1 * vpot_b_2;
    v_ten_v_b_prime[m] = -k1_ten_k2[m + 2] * (vpot_b_1 * vpot_b_2_prime + vpot_b_2 * vpot_b_1_prime);
  }
  /* quadratic collision term: already computed together with the total sources */
  for (int im = 0; im <= c->index_m_max[1]; ++im) {
    int m = c->m[im];
    double quadC_I_1M = (w->linear_only ? 0 : dI_qc2(1, m)) / kappa_dot;
    double quadC_u_g_m = quadC_I_1M / 4 + (u_b_1[m] * delta_b_2 + u_b_2[m] * delta_b_1) -
                         (u_g_1[m] * delta_g_2 + u_g_2[m] * delta_g_1);
    double delta_u_prime_b_m = delta_b_1_prime * u_b_2[m] + delta_b_2_prime * u_b_1[m] + delta_b_1 * u_b_2_prime[m] +
                               delta_b_2 * u_b_1_prime[m];
    double delta_u_prime_g_m = FOUR_THIRDS * delta_u_prime_b_m;
    double quadL_b_11M = -(db_qs2(1, 1, m) - db_qc2(1, 1, m));
    double quadL_I_1M = -(dI_qs2(1, m) - dI_qc2(1, m));
    double quadL_diff = quadL_b_11M / 3 - quadL_I_1M / 4 - delta_u_prime_g_m / 4 +
                        Hc * (u_b_1[m] * delta_b_2 + u_b_2[m] * delta_b_1);
    double R = 3 / (4 * r);
    double omega_m1 = (m == 1 ? y[PV->idx_omega] : 0);
    double U_slip = -quadC_u_g_m - R / (1 + R) * tau_c * (Hc * (u_b[m] + (m == 1 ? omega_m1 : 0)) + k / 4 * (m == 0 ? delta_g : 0) + quadL_diff);
    w->C_1m_tca1[m] = -dI_qc2(1, m) - 4 * R / (1 + R) * (Hc * (u_b[m] + (m == 1 ? omega_m1 : 0)) + k / 4 * (m == 0 ? delta_g : 0) + quadL_diff);
    double u_g_tca1 = u_b[m] - U_slip;
    w->I_1m_tca1[m] = 4 * (u_g_tca1 + delta_g_1 * u_g_2[m] + delta_g_2 * u_g_1[m]);
  }
  for (int im = 0; im <= c->index_m_max[2]; ++im) {
    int m = c->m[im];
    double gamma_m2_prime = (m == 2 ? y[PV->idx_gamma_p] : 0);
    double shear = 8 / 45. * tau_c * (-k * w->I_1m_tca1[m] * c_minus(2, m, m) - 4 * (m == 2 ? gamma_m2_prime : 0));
    double quadC_I_2M = dI_qc2(2, m) / kappa_dot;
    double quadC_E_2M = 0, quadC_B_2M = 0;
    if (s->has_polarization2) {
      quadC_E_2M = dE_qc2(2, m) / kappa_dot;
      quadC_B_2M = (m != 0 ? dB_qc2(2, m) : 0) / kappa_dot;
    }
    double quadL_I_2M = -(dI_qs2(2, m) - dI_qc2(2, m));
    double quadL_E_2M = 0;
    if (s->has_polarization2) quadL_E_2M = -(dE_qs2(2, m) - dE_qc2(2, m));
    shear += 8 / 45. * (-quadC_I_2M + SQRT_6 / 4 * quadC_E_2M - 15 * v_ten_v_g[m]);
    shear += 8 / 45. * tau_c * (quadL_I_2M - SQRT_6 / 4 * quadL_E_2M - 20 * v_ten_v_b_prime[m]);
    if (!s->has_polarization2)
      shear = -4 / 27. * (quadC_I_2M + 18 * v_ten_v_g[m] -
                          tau_c * (-20 * v_ten_v_b_prime[m] - k * w->I_1m[m] * c_minus(2, m, m) - 4 * (m == 2 ? gamma_m2_prime : 0) + quadL_I_2M));
    w->I_2m_tca1[m] = -15 / 2. * shear - 20 * v_ten_v_g[m];
    if (s->has_polarization2) {
      w->Pi_tca1[m] = (w->I_2m_tca1[m] - SQRT_6 * (quadC_E_2M - tau_c * quadL_E_2M)) / 4;
      w->E_2m_tca1[m] = -sqrt(6) * w->Pi_tca1[m] + quadC_E_2M - tau_c * quadL_E_2M;
      w->B_2m_tca1[m] = (m != 0 ? quadC_B_2M : 0);
    } else {
      w->Pi_tca1[m] = 0.1 * w->I_2m_tca1[m];
      w->E_2m_tca1[m] = w->B_2m_tca1[m] = 0;
    }
    (void)v_ten_v_b;
  }
}

static void workspace_at_tau(ws_t *w, const double *y) {
  cfg_t *c = w->c;
  const song2_spec *s = c->s;
  if (c->compute_m[0]) {
    w->I_00 = I(0, 0);
    w->N_00 = N(0, 0);
    w->b_200 = b(2, 0, 0);
    w->cdm_200 = cdm(2, 0, 0);
  }
  for (int im = 0; im <= c->index_m_max[1]; ++im) {
    int m = c->m[im];
    w->I_1m[m] = I(1, m);
    w->N_1m[m] = N(1, m);
    w->C_1m[m] = w->kappa_dot * (FOUR_THIRDS * b(1, 1, m) - I(1, m));
  }
  for (int im = 0; im <= c->index_m_max[2]; ++im) {
    int m = c->m[im];
    w->I_2m[m] = I(2, m);
    if (s->has_polarization2) { w->E_2m[m] = E(2, m); w->B_2m[m] = B(2, m); }
    w->b_22m[m] = 0; w->cdm_22m[m] = 0;
  }
  /* perfect fluids (perturbations2.c:8935-8972) */
  double vv_b = w->qs[w->iq_vv_b], vv_cdm = w->qs[w->iq_vv_cdm];
  w->b_200 = -2 * w->k1_dot_k2 * vv_b;
  w->cdm_200 = -2 * w->k1_dot_k2 * vv_cdm;
  for (int im = 0; im <= c->index_m_max[2]; ++im) {
    int m = c->m[im];
    w->b_22m[m] = 15 * w->k1_ten_k2[m + 2] * vv_b;
    w->cdm_22m[m] = 15 * w->k1_ten_k2[m + 2] * vv_cdm;
  }
  if (PV->tca) {
    tca_variables(w, y);
    for (int im = 0; im <= c->index_m_max[1]; ++im) w->I_1m[c->m[im]] = w->I_1m_tca1[c->m[im]];
    for (int im = 0; im <= c->index_m_max[2]; ++im) {
      int m = c->m[im];
      w->I_2m[m] = w->I_2m_tca1[m];
      if (s->has_polarization2) {
        w->E_2m[m] = w->E_2m_tca1[m];
        w->B_2m[m] = (m != 0 ? w->B_2m_tca1[m] : 0);
      }
    }
    for (int im = 0; im <= c->index_m_max[1]; ++im) w->C_1m[c->m[im]] = w->C_1m_tca1[c->m[im]];
  }
}

/* perturb2_rsa_variables (perturbations2.c:9773-10164) for rsa2_MD and
   rsa2_MD_with_reio with compute_quadsources_derivatives = no (input2.c
   defaults), and its use at the
   end of perturb2_einstein (:8777-8809): the photon and neutrino monopoles and
   dipoles from the RSA solution, the photon collision dipole from the RSA dipole.
   The m = 1 dipoles are zero (:10094-10098, a documented limitation). */
static void rsa_variables(ws_t *w, const double *y, double tau) {
  cfg_t *c = w->c;
  const song2_tables *tab = c->t;
  const double *fo1 = w->fo1, *fo2 = w->fo2;
  double k = w->k, Hc = w->Hc, kappa_dot = w->kappa_dot;
  /* rsa2_MD_with_reio (:9929-9953, 10064-10084): tau_c = 1/kappa' and its
     derivative tau_c' = -kappa'' tau_c^2, kappa'' from the background spline of
     ln kappa' (CLASS's pth->ddkappa is the derivative of its own table) */
  int reio = c->s->radiation_streaming_approximation == SONG2_RSA_MD_WITH_REIO;
  double tau_c = 1 / kappa_dot, tau_c_dot = 0;
  if (reio) {
    double dlnkd = spl_dx(tab->bg_size, SONG2_BG_SIZE, tab->bg_lntau0, tab->bg_dlntau, tab->bg, tab->bg_dd,
                          SONG2_BG_LN_KAPPA_DOT, log(tau));
    double kappa_dot_dot = kappa_dot * dlnkd / tau;
    tau_c_dot = -kappa_dot_dot * tau_c * tau_c;
  }
  double *k1_m = w->k1_m, *k2_m = w->k2_m;
  /* perturb2_fluid_variables (:9108-9338) */
  double vpot_g_1 = fo1[SONG2_FO_V_G], vpot_g_2 = fo2[SONG2_FO_V_G];
  double delta_g_1 = fo1[SONG2_FO_DELTA_G], delta_g_2 = fo2[SONG2_FO_DELTA_G];
  double v_dot_v_g = -w->k1_dot_k2 * vpot_g_1 * vpot_g_2;
  double vpot_ur_1 = fo1[SONG2_FO_V_UR], vpot_ur_2 = fo2[SONG2_FO_V_UR];
  double delta_ur_1 = fo1[SONG2_FO_DELTA_UR], delta_ur_2 = fo2[SONG2_FO_DELTA_UR];
  double v_dot_v_ur = -w->k1_dot_k2 * vpot_ur_1 * vpot_ur_2;
  if (c->compute_m[0]) {
    double psi = w->psi;
    double quadL_I_10 = -(dI_qs2(1, 0) - dI_qc2(1, 0));
    double delta_g_rsa = -4 * psi + quadL_I_10 / k;
    if (reio) {
      delta_g_rsa += -FOUR_THIRDS * b(1, 1, 0) / (k * tau_c);
      double quadC_I_10 = dI_qc2(1, 0) / kappa_dot;
      delta_g_rsa += -quadC_I_10 / (k * tau_c);
    }
    w->I_00 = delta_g_rsa + 8 * v_dot_v_g / 3;
    double quadL_N_10 = -dN_qs2(1, 0);
    double delta_ur_rsa = -4 * psi + quadL_N_10 / k;
    w->N_00 = delta_ur_rsa + 8 * v_dot_v_ur / 3;
  }
  for (int im = 0; im <= c->index_m_max[1]; ++im) {
    int m = c->m[im];
    double I_1m_rsa = 0, N_1m_rsa = 0;
    if (m == 0) {
      double phi_prime = w->phi_prime;
      double psi_prime_quad = w->qs[w->iq_psi_prime] - 2 * Hc * w->qs[w->iq_psi];
      double psi_prime = phi_prime + psi_prime_quad;
      double u_g_1 = -k1_m[1] * vpot_g_1, u_g_2 = -k2_m[1] * vpot_g_2;
      double u_g_rsa = 3 / k * (phi_prime + psi_prime);
      double quadL_I_00 = -(dI_qs2(0, 0) - dI_qc2(0, 0));
      double u_delta_g = u_g_1 * delta_g_2 + u_g_2 * delta_g_1;
      u_g_rsa += -u_delta_g - 3 / (4 * k) * quadL_I_00;
      if (reio) {
        double quadC_I_00 = dI_qc2(0, 0) / kappa_dot, quadC_I_10 = dI_qc2(1, 0) / kappa_dot;
        u_g_rsa += 1 / (k * tau_c) * (-(3 * Hc + tau_c_dot / tau_c) / k * b(1, 1, m) + 9 * w->psi +
                                      3 / 4. * quadC_I_00 - 3 * tau_c_dot * quadC_I_10 / (4 * k * tau_c));
      }
      I_1m_rsa = 4 * (u_g_rsa + delta_g_1 * u_g_2 + delta_g_2 * u_g_1);
      double u_ur_1 = -k1_m[1] * vpot_ur_1, u_ur_2 = -k2_m[1] * vpot_ur_2;
      double u_ur_rsa = 3 / k * (phi_prime + psi_prime);
      double quadL_N_00 = -dN_qs2(0, 0);
      double u_delta_ur = u_ur_1 * delta_ur_2 + u_ur_2 * delta_ur_1;
      u_ur_rsa += -u_delta_ur - 3 / (4 * k) * quadL_N_00;
      N_1m_rsa = 4 * (u_ur_rsa + delta_ur_1 * u_ur_2 + delta_ur_2 * u_ur_1);
    }
    w->I_1m[m] = I_1m_rsa;
    w->C_1m[m] = kappa_dot * (FOUR_THIRDS * b(1, 1, m) - I_1m_rsa);
    w->N_1m[m] = N_1m_rsa;
  }
}

static void einstein(ws_t *w, const double *y) {
  cfg_t *c = w->c;
  double rho_monopole = 0, rho_quadrupole = 0, rho_quadrupole_m1 = 0, rho_quadrupole_m2 = 0, rho_dipole = 0;
  double rho_monopole_b = 0, rho_monopole_cdm = 0;
  double k_sq = w->k_sq, k = w->k, a_sq = w->a_sq, Hc = w->Hc, Hc_prime = w->Hc_prime;
  double rho_g = w->rho_g, rho_b = w->rho_b, rho_cdm = w->rho_cdm, rho_ur = w->rho_ur;
  if (c->compute_m[0]) {
    rho_monopole = rho_g * w->I_00;
    rho_dipole = rho_g * w->I_1m[0];
    rho_quadrupole = rho_g * w->I_2m[0];
    rho_monopole_b = rho_b * b(0, 0, 0);
    rho_monopole += rho_monopole_b;
    rho_dipole += rho_b * b(1, 1, 0);
    rho_quadrupole += rho_b * w->b_22m[0];
    rho_monopole_cdm = rho_cdm * cdm(0, 0, 0);
    rho_monopole += rho_monopole_cdm;
    rho_dipole += rho_cdm * cdm(1, 1, 0);
    rho_quadrupole += rho_cdm * w->cdm_22m[0];
    rho_monopole += rho_ur * w->N_00;
    rho_dipole += rho_ur * w->N_1m[0];
    rho_quadrupole += rho_ur * N(2, 0);
  }
  if (c->compute_m[1]) rho_quadrupole_m1 = rho_g * w->I_2m[1] + rho_b * w->b_22m[1] + rho_cdm * w->cdm_22m[1] + rho_ur * N(2, 1);
  if (c->compute_m[2]) rho_quadrupole_m2 = rho_g * w->I_2m[2] + rho_b * w->b_22m[2] + rho_cdm * w->cdm_22m[2] + rho_ur * N(2, 2);
  if (c->compute_m[0]) {
    w->psi = y[PV->idx_phi] - 3 / 5. * (a_sq / k_sq) * rho_quadrupole + w->qs[w->iq_psi];
    w->phi_prime_poisson = -Hc * w->psi - k_sq / (3 * Hc) * y[PV->idx_phi] - a_sq * rho_monopole / (2 * Hc) +
                           w->qs[w->iq_phi_prime_poisson];
    w->phi_prime_longitudinal = -Hc * w->psi + 0.5 * (a_sq / k) * rho_dipole + w->qs[w->iq_phi_prime_longitudinal];
    w->phi_prime = y[PV->idx_phi_p];
    double psi = w->psi, phi = y[PV->idx_phi], phi_prime = w->phi_prime;
    w->phi_prime_prime = +k_sq / 3 * (psi - 2 * phi) - Hc * (0 + 3 * phi_prime) - 2 * psi * (Hc * Hc + Hc_prime) -
                         a_sq / 2 * (rho_monopole_b + rho_monopole_cdm) + w->qs[w->iq_phi_prime_prime];
  }
  if (c->compute_m[1])
    w->omega_m1_prime = -2 * Hc * y[PV->idx_omega] + 2 * SQRT_3 / (5. * k) * a_sq * rho_quadrupole_m1 + w->qs[w->iq_omega_m1_prime];
  if (c->compute_m[2])
    w->gamma_m2_prime_prime = -2 * Hc * y[PV->idx_gamma_p] - k_sq * y[PV->idx_gamma] - 2 / 5. * a_sq * rho_quadrupole_m2 +
                              w->qs[w->iq_gamma_m2_prime_prime];
  if (PV->rsa) rsa_variables(w, y, w->tau);
}

static double compute_psi_prime(ws_t *w, const double *y, const double *dy) {
  cfg_t *c = w->c;
  double *fo1 = w->fo1, *fo2 = w->fo2;
  double k = w->k, k_sq = k * k, a_sq = w->a_sq, Hc = w->Hc;
  double rho_g = w->rho_g, rho_b = w->rho_b, rho_cdm = w->rho_cdm, rho_ur = w->rho_ur;
  double rho_plus_3p_quadrupole = 2 * rho_g * w->I_2m[0];
  double rho_quadrupole_prime;
  if (!PV->tca) {
    rho_quadrupole_prime = rho_g * dI(2, 0);
  } else {
    double dI_20 = 2 / 3. * k * w->I_1m_tca1[0] - w->kappa_dot * (w->I_2m_tca1[0] - w->Pi_tca1[0]) + dI_qs2(2, 0);
    rho_quadrupole_prime = rho_g * dI_20;
  }
  rho_plus_3p_quadrupole += rho_b * w->b_22m[0];
  double db_220 = 15 * w->k1_ten_k2[2] * w->qs[w->iq_vvp_b];
  rho_quadrupole_prime += rho_b * db_220;
  rho_plus_3p_quadrupole += rho_cdm * w->cdm_22m[0];
  double dcdm_220 = 15 * w->k1_ten_k2[2] * w->qs[w->iq_vvp_cdm];
  rho_quadrupole_prime += rho_cdm * dcdm_220;
  rho_plus_3p_quadrupole += 2 * rho_ur * N(2, 0);
  rho_quadrupole_prime += rho_ur * dN(2, 0);
  (void)rho_plus_3p_quadrupole;
  double phi_prime = w->phi_prime, psi = w->psi, phi = y[PV->idx_phi];
  return phi_prime - 2 * Hc * (psi - phi) -
         3 / 5. * (a_sq / k_sq) * (rho_quadrupole_prime + Hc * rho_b * w->b_22m[0] + Hc * rho_cdm * w->cdm_22m[0]) +
         w->qs[w->iq_psi_prime];
}

/* ======================================================= derivs */

/* Evaluate the interpolated quantities at tau (background, first order,
   quadratic sources); shared by derivs and the Jacobian probes. */
static void prepare_tau(ws_t *w, double tau) {
  background_at_tau(w, tau);
  first_order_at_tau(w, tau);
  quadratic_sources(w, QS_WHAT_TOTAL);
}

/* The reference's derivs path (perturb2_quadratic_sources_at_tau,
   perturbations2.c:14366-14688): quadratic sources by cubic-spline interpolation
   of the triplet's table; during tight coupling the collision terms are computed
   directly from the interpolated first-order quantities, as perturb2_tca_variables
   does (perturbations2.c:9440-9456). */
static void prepare_tau_table(ws_t *w, double tau) {
  cfg_t *c = w->c;
  const song2_tables *t = c->t;
  background_at_tau(w, tau);
  if (w->linear_only || c->first_order_mode || !c->s->has_quadratic_sources || !w->qt_ready) {
    memset(w->qs, 0, sizeof(double) * w->qs2_size);
    memset(w->qc, 0, sizeof(double) * w->qs2_size);
    memset(w->fo1, 0, sizeof(double) * c->nfo);
    memset(w->fo2, 0, sizeof(double) * c->nfo);
    return;
  }
  double x = log(tau), dx = t->fo_dlntau;
  double u = (x - t->fo_lntau0) / dx;
  int i = (int)floor(u);
  if (i < w->qt_j0) i = w->qt_j0;
  if (i > w->qt_j0 + w->qt_n - 2) i = w->qt_j0 + w->qt_n - 2;
  double b = u - i, a = 1.0 - b;
  double ca = (a * a * a - a) * (dx * dx) / 6.0, cb = (b * b * b - b) * (dx * dx) / 6.0;
  int nq = w->qs2_size;
  const double *r0 = w->qtab + (size_t)(i - w->qt_j0) * 2 * nq, *r1 = r0 + 2 * nq;
  for (int q = 0; q < nq; ++q) w->qs[q] = a * r0[q] + b * r1[q] + ca * r0[nq + q] + cb * r1[nq + q];
  if (w->pv.tca || w->pv.rsa) {
    first_order_at_tau(w, tau);
    quadratic_sources(w, QS_WHAT_COLLISION);
  } else {
    memset(w->qc, 0, sizeof(double) * w->qs2_size);
  }
}

/* Quadratic sources of the triplet at the first-order nodes covering
   [tau_ini, tau_end] (exact first-order values at the nodes, background by
   spline), then natural cubic splines in ln tau (perturbations2.c:10407-10606). */
static void build_qs_table(ws_t *w, double tau_ini, double tau_end) {
  cfg_t *c = w->c;
  const song2_tables *t = c->t;
  w->qt_ready = 0;
  if (c->first_order_mode || !c->s->has_quadratic_sources) return;
  int N = t->fo_tau_size;
  double x0 = t->fo_lntau0, dx = t->fo_dlntau;
  int j0 = (int)floor((log(tau_ini) - x0) / dx);
  int j1 = (int)ceil((log(tau_end) - x0) / dx);
  if (j0 < 0) j0 = 0;
  if (j0 > N - 2) j0 = N - 2;
  if (j1 > N - 1) j1 = N - 1;
  if (j1 < j0 + 1) j1 = j0 + 1;
  int M = j1 - j0 + 1, nq = w->qs2_size;
  w->qt_j0 = j0;
  w->qt_n = M;
  size_t stride = (size_t)t->fo_tau_size * t->fo_size;
  const double *v1 = t->fo + stride * w->index_k1, *v2 = t->fo + stride * w->index_k2;
  for (int j = 0; j < M; ++j) {
    double x = x0 + (j0 + j) * dx;
    /* background at the node */
    double tau = exp(x);
#define BGX(qq) spl(t->bg_size, SONG2_BG_SIZE, t->bg_lntau0, t->bg_dlntau, t->bg, t->bg_dd, (qq), x)
    w->a = exp(BGX(SONG2_BG_LN_A));
    w->a_sq = w->a * w->a;
    w->Hc = exp(BGX(SONG2_BG_LN_HC));
    w->Hc_prime = BGX(SONG2_BG_HC_PRIME_TAU2) / (tau * tau);
    w->rho_g = exp(BGX(SONG2_BG_LN_RHO_G));
    w->rho_b = exp(BGX(SONG2_BG_LN_RHO_B));
    w->rho_cdm = exp(BGX(SONG2_BG_LN_RHO_CDM));
    w->rho_ur = exp(BGX(SONG2_BG_LN_RHO_UR));
    w->kappa_dot = exp(BGX(SONG2_BG_LN_KAPPA_DOT));
    w->exp_m_kappa = exp(-BGX(SONG2_BG_KAPPA));
#undef BGX
    w->g = w->kappa_dot * w->exp_m_kappa;
    w->r = w->rho_g / w->rho_b;
    memcpy(w->fo1, v1 + (size_t)(j0 + j) * t->fo_size, sizeof(double) * c->nfo);
    memcpy(w->fo2, v2 + (size_t)(j0 + j) * t->fo_size, sizeof(double) * c->nfo);
    quadratic_sources(w, QS_WHAT_TOTAL);
    memcpy(w->qtab + (size_t)j * 2 * nq, w->qs, sizeof(double) * nq);
  }
  /* natural spline, column by column (same recurrence as song2_spline_uniform) */
  for (int q = 0; q < nq; ++q) {
    double prev = 0.0, cprev = 0.0;
    w->qtab[nq + q] = 0.0;
    for (int j = 1; j < M - 1; ++j) {
      double ym = w->qtab[(size_t)(j - 1) * 2 * nq + q], y0 = w->qtab[(size_t)j * 2 * nq + q];
      double yp = w->qtab[(size_t)(j + 1) * 2 * nq + q];
      double r = 6.0 * (yp - 2.0 * y0 + ym) / (dx * dx);
      double bb = 4.0 - cprev;
      double ci = 1.0 / bb;
      prev = (r - prev) / bb;
      w->qtab[(size_t)j * 2 * nq + nq + q] = prev;
      w->qt_c[j] = ci;
      cprev = ci;
    }
    w->qtab[(size_t)(M - 1) * 2 * nq + nq + q] = 0.0;
    for (int j = M - 2; j >= 1; --j)
      w->qtab[(size_t)j * 2 * nq + nq + q] -= w->qt_c[j] * w->qtab[(size_t)(j + 1) * 2 * nq + nq + q];
  }
  w->qt_ready = 1;
}

static void derivs_prepared(ws_t *w, double tau, const double *y, double *dy) {
  cfg_t *c = w->c;
  const song2_spec *s = c->s;
  double k = w->k, Hc = w->Hc, kappa_dot = w->kappa_dot, r = w->r;
  w->st.n_rhs++;
  for (int i = 0; i < PV->n; ++i) dy[i] = 0.0;
  workspace_at_tau(w, y);
  einstein(w, y);
  double psi = 0, phi_prime = 0, omega_m1 = 0, omega_m1_prime = 0, gamma_m2_prime = 0;
  if (c->compute_m[0]) { phi_prime = w->phi_prime; psi = w->psi; }
  if (c->compute_m[1]) { omega_m1 = y[PV->idx_omega]; omega_m1_prime = w->omega_m1_prime; }
  if (c->compute_m[2]) gamma_m2_prime = y[PV->idx_gamma_p];
  double metric_continuity = 0, metric_euler = 0;
  if (c->compute_m[0]) { metric_continuity = -3 * phi_prime; metric_euler = k * psi; }
  int l_max_g = PV->l_max_g, l_max_pol_g = PV->l_max_pol_g, l_max_ur = PV->l_max_ur;
  double I_00 = w->I_00, N_00 = w->N_00, *N_1m = w->N_1m, *I_1m = w->I_1m, *I_2m = w->I_2m, *E_2m = w->E_2m;
  double *B_2m = w->B_2m, *b_22m = w->b_22m, b_200 = w->b_200;
  /* photon temperature */
  if (l_max_g > -1 && c->compute_m[0]) dI(0, 0) = -FOUR_THIRDS * (k * I_1m[0] / 4 + metric_continuity);
  if (l_max_g > 0)
    for (int im = 0; im <= c->index_m_max[1]; ++im) {
      int m = c->m[im];
      dI(1, m) = k * (c_minus(1, m, m) * I_00 - c_plus(1, m, m) * I_2m[m]) + w->C_1m[m];
      if (m == 0) dI(1, m) += 4 * metric_euler;
      if (m == 1) dI(1, m) += -4 * omega_m1_prime;
    }
  if (l_max_g > 1)
    for (int im = 0; im <= c->index_m_max[2]; ++im) {
      int m = c->m[im];
      double Pi = 0.1 * (I_2m[m] - SQRT_6 * E_2m[m]);
      dI(2, m) = k * (c_minus(2, m, m) * I_1m[m] - c_plus(2, m, m) * I(3, m)) - kappa_dot * (I_2m[m] - Pi);
      if (m == 2) dI(2, m) += 4 * gamma_m2_prime;
    }
  for (int l = 3; l <= l_max_g; ++l)
    for (int im = 0; im <= c->index_m_max[l]; ++im) {
      int m = c->m[im];
      dI(l, m) = k * (c_minus(l, m, m) * I(l - 1, m) - c_plus(l, m, m) * I(l + 1, m)) - kappa_dot * I(l, m);
    }
  if (PV->use_closure_g) {
    int l = l_max_g;
    for (int im = 0; im <= c->index_m_max[l]; ++im) {
      int m = c->m[im];
      double c_pre = (m == 0 ? (2 * l + 1) / (2 * l - 1.) : sqrt((double)(l + abs(m)) / (l - abs(m))) * (2 * l + 1) / (2 * l - 1.));
      double c_ = (l + 1 + abs(m)) / (k * tau);
      dI(l, m) = k * (c_pre * I(l - 1, m) - c_ * I(l, m)) - kappa_dot * I(l, m);
    }
  }
  if (s->has_quadratic_sources)
    for (int l = 0; l <= (l_max_g < w->l_max_g ? l_max_g : w->l_max_g); ++l)
      for (int im = 0; im <= c->index_m_max[l]; ++im) dI(l, c->m[im]) += dI_qs2(l, c->m[im]);
  /* polarisation */
  if (s->has_polarization2) {
    if (l_max_pol_g > 1)
      for (int im = 0; im <= c->index_m_max[2]; ++im) {
        int m = c->m[im];
        double Pi = 0.1 * (I_2m[m] - SQRT_6 * E_2m[m]);
        dE(2, m) = k * (-d_plus(2, m, m) * E(3, m) - d_zero(2, m, m) * B_2m[m]) - kappa_dot * (E_2m[m] + SQRT_6 * Pi);
      }
    for (int l = 3; l <= l_max_pol_g; ++l)
      for (int im = 0; im <= c->index_m_max[l]; ++im) {
        int m = c->m[im];
        dE(l, m) = k * (d_minus(l, m, m) * E(l - 1, m) - d_plus(l, m, m) * E(l + 1, m) - d_zero(l, m, m) * B(l, m)) -
                   kappa_dot * E(l, m);
      }
    for (int l = 2; l <= l_max_pol_g; ++l)
      for (int im = 0; im <= c->index_m_max[l]; ++im) {
        int m = c->m[im];
        dB(l, m) = k * (d_minus(l, m, m) * B(l - 1, m) - d_plus(l, m, m) * B(l + 1, m) + d_zero(l, m, m) * E(l, m)) -
                   kappa_dot * B(l, m);
      }
    if (PV->use_closure_pol_g) {
      int l = l_max_pol_g;
      for (int im = 0; im <= c->index_m_max[l]; ++im) {
        int m = c->m[im];
        double c_pre = sqrt(1 - (((double)m) * m) / (l * l) * (l + 2) / (l - 2.)) * (2 * l + 1) / (2 * l - 1.);
        double cc = (l + 3) / (k * tau);
        double c_mix = ((double)m) / ((double)l);
        dE(l, m) = k * (c_pre * E(l - 1, m) - cc * E(l, m) - c_mix * B(l, m)) - kappa_dot * E(l, m);
        dB(l, m) = k * (c_pre * B(l - 1, m) - cc * B(l, m) + c_mix * E(l, m)) - kappa_dot * B(l, m);
      }
    }
    if (s->has_quadratic_sources)
      for (int l = 2; l <= (l_max_pol_g < w->l_max_pol_g ? l_max_pol_g : w->l_max_pol_g); ++l)
        for (int im = 0; im <= c->index_m_max[l]; ++im) {
          int m = c->m[im];
          dE(l, m) += dE_qs2(l, m);
          dB(l, m) += dB_qs2(l, m);
        }
  }
  /* neutrinos */
  if (l_max_ur > -1 && c->compute_m[0]) dN(0, 0) = -FOUR_THIRDS * (k * N_1m[0] * 0.25 + metric_continuity);
  if (l_max_ur > 0)
    for (int im = 0; im <= c->index_m_max[1]; ++im) {
      int m = c->m[im];
      dN(1, m) = k * (c_minus(1, m, m) * N_00 - c_plus(1, m, m) * N(2, m));
      if (m == 0) dN(1, m) += 4 * metric_euler;
      if (m == 1) dN(1, m) += -4 * omega_m1_prime;
    }
  for (int l = 2; l <= l_max_ur; ++l)
    for (int im = 0; im <= c->index_m_max[l]; ++im) {
      int m = c->m[im];
      dN(l, m) = k * (c_minus(l, m, m) * N(l - 1, m) - c_plus(l, m, m) * N(l + 1, m));
    }
  if (l_max_ur > 1 && c->compute_m[2]) dN(2, 2) += 4 * gamma_m2_prime;
  if (PV->use_closure_ur) {
    int l = l_max_ur;
    for (int im = 0; im <= c->index_m_max[l]; ++im) {
      int m = c->m[im];
      double c_pre = (m == 0 ? (2 * l + 1) / (2 * l - 1.) : sqrt((double)(l + abs(m)) / (l - abs(m))) * (2 * l + 1) / (2 * l - 1.));
      double cc = (l + 1 + abs(m)) / (k * tau);
      dN(l, m) = k * (c_pre * N(l - 1, m) - cc * N(l, m));
    }
  }
  if (s->has_quadratic_sources)
    for (int l = 0; l <= (l_max_ur < w->l_max_ur ? l_max_ur : w->l_max_ur); ++l)
      for (int im = 0; im <= c->index_m_max[l]; ++im) dN(l, c->m[im]) += dN_qs2(l, c->m[im]);
  /* baryons */
  if (c->compute_m[0]) db(0, 0, 0) = -(k * b(1, 1, 0) * ONE_THIRD + metric_continuity) - Hc * b_200;
  for (int im = 0; im <= c->index_m_max[1]; ++im) {
    int m = c->m[im];
    db(1, 1, m) = -Hc * b(1, 1, m) + k * (c_minus(1, m, m) * b_200 - c_plus(1, m, m) * b_22m[m]) - r * w->C_1m[m];
    if (m == 0) db(1, 1, m) += 3 * metric_euler;
    if (m == 1) db(1, 1, m) += -3 * (omega_m1_prime + Hc * omega_m1);
  }
  if (s->has_quadratic_sources) {
    if (c->compute_m[0]) db(0, 0, 0) += db_qs2(0, 0, 0);
    for (int im = 0; im <= c->index_m_max[1]; ++im) db(1, 1, c->m[im]) += db_qs2(1, 1, c->m[im]);
  }
  /* CDM */
  if (c->compute_m[0]) dcdm(0, 0, 0) = -(k * cdm(1, 1, 0) * ONE_THIRD + metric_continuity) - Hc * w->cdm_200;
  for (int im = 0; im <= c->index_m_max[1]; ++im) {
    int m = c->m[im];
    dcdm(1, 1, m) = -Hc * cdm(1, 1, m) + k * (c_minus(1, m, m) * w->cdm_200 - c_plus(1, m, m) * w->cdm_22m[m]);
    if (m == 0) dcdm(1, 1, m) += 3 * metric_euler;
    if (m == 1) dcdm(1, 1, m) += -3 * (omega_m1_prime + Hc * omega_m1);
  }
  if (s->has_quadratic_sources) {
    if (c->compute_m[0]) dcdm(0, 0, 0) += dcdm_qs2(0, 0, 0);
    for (int im = 0; im <= c->index_m_max[1]; ++im) dcdm(1, 1, c->m[im]) += dcdm_qs2(1, 1, c->m[im]);
  }
  /* metric */
  if (c->compute_m[0]) {
    dy[PV->idx_phi] = w->phi_prime;
    double psi_prime = compute_psi_prime(w, y, dy);
    w->phi_prime_prime += -Hc * psi_prime;
    dy[PV->idx_phi_p] = w->phi_prime_prime;
  }
  if (c->compute_m[1]) dy[PV->idx_omega] = w->omega_m1_prime;
  if (c->compute_m[2]) {
    dy[PV->idx_gamma] = y[PV->idx_gamma_p];
    dy[PV->idx_gamma_p] = w->gamma_m2_prime_prime;
  }
  (void)psi;
}

static void derivs(ws_t *w, double tau, const double *y, double *dy) {
  prepare_tau_table(w, tau);
  derivs_prepared(w, tau, y, dy);
}

/* Exact Jacobian of the affine system: J e_j = (linear part of derivs)(e_j). */
static void jacobian(ws_t *w, double tau) {
  int n = PV->n;
  w->st.n_jac++;
  int saved_rhs = w->st.n_rhs;
  w->linear_only = 1;
  prepare_tau(w, tau);
  for (int j = 0; j < n; ++j) {
    memset(w->ylin, 0, sizeof(double) * n);
    w->ylin[j] = 1.0;
    derivs_prepared(w, tau, w->ylin, w->dylin);
    for (int i = 0; i < n; ++i) w->J[(size_t)i * n + j] = w->dylin[i];
  }
  w->linear_only = 0;
  w->st.n_rhs = saved_rhs;
}

/* ======================================================= vector layout */

/* approximation: 0 none, 1 tight coupling, 2 radiation streaming */
static void vector_layout(ws_t *w, int approx) {
  cfg_t *c = w->c;
  const song2_spec *s = c->s;
  pv_t *p = PV;
  p->tca = approx == 1;
  p->rsa = approx == 2;
  p->use_closure_g = p->use_closure_pol_g = p->use_closure_ur = 1;
  p->l_max_g = s->l_max_g;
  p->l_max_pol_g = s->has_polarization2 ? s->l_max_pol_g : -1;
  p->l_max_ur = s->l_max_ur;
  if (p->tca) {
    p->l_max_g = 0; p->use_closure_g = 0;
    p->l_max_pol_g = -1; p->use_closure_pol_g = 0;
  }
  if (p->rsa) {
    /* perturbations2.c:6778-6796: no massless hierarchies; their start indices
       all fall on the baryon block, as in the reference */
    p->l_max_g = p->l_max_pol_g = p->l_max_ur = -1;
    p->use_closure_g = p->use_closure_pol_g = p->use_closure_ur = 0;
  }
  if (!s->has_polarization2) p->use_closure_pol_g = 0;
  p->n_max_b = p->l_max_b = p->n_max_cdm = p->l_max_cdm = 1;
  int n = 0;
  p->idx_g = n; n += size_l_indexm(c, p->l_max_g);
  p->idx_E = n; if (s->has_polarization2) n += size_l_indexm(c, p->l_max_pol_g);
  p->idx_B = n; if (s->has_polarization2) n += size_l_indexm(c, p->l_max_pol_g);
  p->idx_ur = n; n += size_l_indexm(c, p->l_max_ur);
  p->idx_b = n; n += nlm_hier_b(c);
  p->idx_cdm = n; n += nlm_hier_b(c);
  p->idx_phi = p->idx_phi_p = p->idx_omega = p->idx_gamma = p->idx_gamma_p = -1;
  if (c->compute_m[0]) { p->idx_phi = n++; p->idx_phi_p = n++; }
  if (c->compute_m[1]) p->idx_omega = n++;
  if (c->compute_m[2]) { p->idx_gamma = n++; p->idx_gamma_p = n++; }
  p->n = n;
}

/* ======================================================= initial conditions */

static void initial_conditions(ws_t *w, double tau, double *y) {
  cfg_t *c = w->c;
  const song2_spec *s = c->s;
  double *fo1 = w->fo1, *fo2 = w->fo2;
  memset(y, 0, sizeof(double) * PV->n);
  prepare_tau(w, tau);
  double k = w->k, k_sq = w->k_sq, Hc = w->Hc, Hc_sq = Hc * Hc, a_sq = w->a_sq;
  double k1_0 = w->k1_m[1], k2_0 = w->k2_m[1];
  double rho_g = w->rho_g, rho_ur = w->rho_ur, rho_r = rho_g + rho_ur;
  double frac_ur = rho_ur / rho_r, frac_g = 1 - frac_ur;
  double rho_tot = Hc_sq / a_sq;
  double Omega_m = (w->rho_b + w->rho_cdm) / rho_tot, Omega_r = rho_r / rho_tot;
  if (s->ic == SONG2_IC_ZERO) return;
  if (s->ic == SONG2_IC_AD) {
    if (!c->compute_m[0]) return;
    double delta_g_1 = fo1[SONG2_FO_DELTA_G], delta_g_2 = fo2[SONG2_FO_DELTA_G];
    double vpot_g_1 = fo1[SONG2_FO_V_G], vpot_g_2 = fo2[SONG2_FO_V_G];
    double delta_b_1 = fo1[SONG2_FO_DELTA_B], delta_b_2 = fo2[SONG2_FO_DELTA_B];
    double vpot_b_1 = fo1[SONG2_FO_V_B], vpot_b_2 = fo2[SONG2_FO_V_B];
    double delta_cdm_1 = fo1[SONG2_FO_DELTA_CDM], delta_cdm_2 = fo2[SONG2_FO_DELTA_CDM];
    double vpot_cdm_1 = fo1[SONG2_FO_V_CDM], vpot_cdm_2 = fo2[SONG2_FO_V_CDM];
    double delta_ur_1 = fo1[SONG2_FO_DELTA_UR], delta_ur_2 = fo2[SONG2_FO_DELTA_UR];
    double vpot_ur_1 = fo1[SONG2_FO_V_UR], vpot_ur_2 = fo2[SONG2_FO_V_UR];
    double phi_1 = fo1[SONG2_FO_PHI], phi_2 = fo2[SONG2_FO_PHI];
    double psi_1 = fo1[SONG2_FO_PSI], psi_2 = fo2[SONG2_FO_PSI];
    double zeta = 2 * (3 / 5. * s->primordial_local_fnl_phi);
    double A_quad = w->qs[w->iq_psi];
    double I_2_0_quad = 5 / 8. * (c_minus_12(2, 0) * I_1_raw(1) * I_2_raw(1) + c_minus_21(2, 0) * I_2_raw(1) * I_1_raw(1));
    double N_2_0_quad = 1 / 3. * (k / Hc_sq) * dN_qs2(1, 0) + 1 / (2 * Hc) * dN_qs2(2, 0) + 8 / 3. * (k_sq / Hc_sq) * psi_1 * psi_2;
    double quadrupole_quad = (frac_g * I_2_0_quad + frac_ur * N_2_0_quad) * 3 / 5. * (Hc_sq / k_sq);
    double B_quad = A_quad - quadrupole_quad;
    double frac_g_factor = 1 + 4 / 15. * (1 - frac_g);
    double psi = 1. / frac_g_factor * 2 / 3. * (-zeta + psi_1 * psi_2 - 2 * phi_1 * phi_2 + B_quad);
    double I_2_0 = I_2_0_quad;
    double N_2_0 = 2 / 3. * (k_sq / Hc_sq) * psi + N_2_0_quad;
    double phi = (1 + 2 / 5. * frac_ur) * psi - B_quad;
    double L_quad = w->qs[w->iq_phi_prime_longitudinal];
    double u_0_adiabatic = 2 * (k / Hc) * (psi - L_quad / Hc) - (-k1_0 * vpot_cdm_1) * (3 * Omega_m * delta_cdm_2 + 4 * Omega_r * delta_g_2) -
                           (-k2_0 * vpot_cdm_2) * (3 * Omega_m * delta_cdm_1 + 4 * Omega_r * delta_g_1);
    u_0_adiabatic *= 1 / (3 * Omega_m + 4 * Omega_r);
    double I_1_0 = 4 * (u_0_adiabatic + delta_g_1 * (-k2_0 * vpot_g_2) + delta_g_2 * (-k1_0 * vpot_g_1));
    double N_1_0 = 4 * (u_0_adiabatic + delta_ur_1 * (-k2_0 * vpot_ur_2) + delta_ur_2 * (-k1_0 * vpot_ur_1));
    double b_1_1_0 = 3 * (u_0_adiabatic + delta_b_1 * (-k2_0 * vpot_b_2) + delta_b_2 * (-k1_0 * vpot_b_1));
    double cdm_1_1_0 = 3 * (u_0_adiabatic + delta_cdm_1 * (-k2_0 * vpot_cdm_2) + delta_cdm_2 * (-k1_0 * vpot_cdm_1));
    double I_0_0 = -2 * psi + 8 * psi_1 * psi_2;
    double N_0_0 = I_0_0;
    double b_0_0_0 = 3 * (I_0_0 / 4 - delta_g_1 * delta_g_2 / 16);
    double cdm_0_0_0 = b_0_0_0;
    y[PV->idx_phi] = phi;
    y[PV->idx_g] = I_0_0;
    if (!PV->tca) {
      y[PV->idx_g + LM(1, 0)] = I_1_0;
      y[PV->idx_g + LM(2, 0)] = I_2_0;
    }
    y[PV->idx_b + NLM(0, 0, 0)] = b_0_0_0;
    y[PV->idx_b + NLM(1, 1, 0)] = b_1_1_0;
    y[PV->idx_cdm + NLM(0, 0, 0)] = cdm_0_0_0;
    y[PV->idx_cdm + NLM(1, 1, 0)] = cdm_1_1_0;
    y[PV->idx_ur + LM(0, 0)] = N_0_0;
    y[PV->idx_ur + LM(1, 0)] = N_1_0;
    y[PV->idx_ur + LM(2, 0)] = N_2_0;
    double rho_monopole = w->rho_g * I_0_0 + w->rho_b * b_0_0_0 + w->rho_cdm * cdm_0_0_0 + w->rho_ur * N_0_0;
    y[PV->idx_phi_p] = -Hc * psi - k_sq / (3 * Hc) * phi - a_sq * rho_monopole / (2 * Hc) + w->qs[w->iq_phi_prime_poisson];
    (void)rho_monopole;
  } else if (s->ic == SONG2_IC_AD_FIRST_ORDER) {
    double fnl_zeta = 3 / 5. * s->primordial_local_fnl_phi;
    double R = 2 * (-fnl_zeta);
    double C = 0.5 * R;
    if (!c->compute_m[0]) return;
    double psi = 20 * C / (15 + 4 * frac_ur);
    y[PV->idx_phi] = (1 + 2 / 5. * frac_ur) * psi;
    double u_0 = 1 / 2. * k * tau * psi;
    double I_0_0 = -2 * psi;
    y[PV->idx_g] = I_0_0;
    if (!PV->tca) y[PV->idx_g + LM(1, 0)] = 4 * u_0;
    y[PV->idx_b + NLM(0, 0, 0)] = 3 / 4. * I_0_0;
    y[PV->idx_b + NLM(1, 1, 0)] = 3 * u_0;
    y[PV->idx_cdm + NLM(0, 0, 0)] = 3 / 4. * I_0_0;
    y[PV->idx_cdm + NLM(1, 1, 0)] = 3 * u_0;
    y[PV->idx_ur] = I_0_0;
    y[PV->idx_ur + LM(1, 0)] = 4 * u_0;
    double shear_ur = 1 / 15. * k * k * tau * tau * psi;
    /* I_20 = 10 shear (the normalisation of the second-order initial conditions,
       perturbations2.c:3901); the reference's debug-only first-order branch divides
       by 10 instead (perturbations2.c:4176), which leaves phi - psi wrong by 100x */
    y[PV->idx_ur + LM(2, 0)] = 10 * shear_ur;
    /* phi' of the Huang equation: the first-order potentials are constant at early times */
    y[PV->idx_phi_p] = 0.0;
  }
}

/* ======================================================= outputs */

/* First-order collision terms over kappa' (ppt->index_qs_monopole_collision_g and
   _E of the first-order module): the photon one is a column of the first-order
   table; the E one is the linear E collision term, -E_l - sqrt6/10 Pi delta_l2. */
static double coll_g_raw(const cfg_t *c, const double *fo, int l) { return (l < 0) ? 0.0 : fo[c->fo_CG + l]; }
static double coll_E_raw(const cfg_t *c, const double *fo, int l) {
  if (l < 2) return 0.0;
  double v = -fo[c->fo_E + l];
  if (l == 2) v += -SQRT_6 * 0.1 * (fo[SONG2_FO_I + 2] - SQRT_6 * fo[c->fo_E + 2]);
  return v;
}

/* delta-tilde terms of the (l,m) source of field 0/1/2 = T/E/B
   (perturbations2.c:12339-12398, 12509-12561, 12658-12710) */
static double delta_tilde_source(ws_t *w, int field, int l, int m) {
  cfg_t *c = w->c;
  const song2_spec *s = c->s;
  const double *fo1 = w->fo1, *fo2 = w->fo2;
  double delta_delta_lm = 0, delta_collision_lm = 0;
  int lq = (field == 0) ? s->l_max_los_quadratic_t : s->l_max_los_quadratic_p;
  for (int l1 = 0; l1 <= lq; ++l1)
    for (int l2 = abs(l1 - l); l2 <= (l1 + l < lq ? l1 + l : lq); ++l2) {
      if (field != 2 && (l1 + l2 + l) % 2 != 0) continue;
      if (field == 2 && (l1 + l2 + l) % 2 == 0) continue;
      for (int m1 = -l1; m1 <= l1; ++m1) {
        int m2 = m - m1;
        double coupling = (abs(m2) > l2) ? 0.0 : DTC(c, field, l, m, l1, m1, l2);
        if (field == 0) {
          double c_1 = rot_1(l2, m2) * coll_g_raw(c, fo1, l2);
          double c_2 = rot_2(l2, m2) * coll_g_raw(c, fo2, l2);
          delta_delta_lm += coupling * 2 * I_1(l1, m1) * I_2(l2, m2);
          delta_collision_lm += coupling * 2 * 0.5 * (I_1(l1, m1) * c_2 + I_2(l1, m1) * c_1);
        } else {
          double c_I_k1_l1 = rot_1(l1, m1) * coll_g_raw(c, fo1, l1);
          double c_I_k2_l1 = rot_2(l1, m1) * coll_g_raw(c, fo2, l1);
          double c_E_k1_l2 = rot_1(l2, m2) * coll_E_raw(c, fo1, l2);
          double c_E_k2_l2 = rot_2(l2, m2) * coll_E_raw(c, fo2, l2);
          delta_delta_lm += coupling * 2 * 0.5 * (I_1(l1, m1) * E_2(l2, m2) + I_2(l1, m1) * E_1(l2, m2));
          delta_collision_lm += coupling * 0.5 *
                                (I_1(l1, m1) * c_E_k2_l2 + c_I_k1_l1 * E_2(l2, m2) + I_2(l1, m1) * c_E_k1_l2 +
                                 c_I_k2_l1 * E_1(l2, m2));
        }
      }
    }
  return -QUAD_COEFF * w->kappa_dot * 0.5 * delta_delta_lm - QUAD_COEFF * w->kappa_dot * delta_collision_lm;
}

static void store_sources(ws_t *w, int index_tau, double tau, const double *y, const double *dy) {
  cfg_t *c = w->c;
  const song2_spec *s = c->s;
  double *fo1 = w->fo1, *fo2 = w->fo2;
  double k1 = w->k1, k2 = w->k2, k = w->k, *k1_m = w->k1_m, *k2_m = w->k2_m;
  w->st.sources_calls++;
  /* the reference recomputes the quadratic sources and the workspace here */
  prepare_tau(w, tau);
  workspace_at_tau(w, y);
  einstein(w, y);
  double kappa_dot = w->kappa_dot, exp_m_kappa = w->exp_m_kappa;
  double psi_1 = fo1[SONG2_FO_PSI], psi_2 = fo2[SONG2_FO_PSI], phi_1 = fo1[SONG2_FO_PHI], phi_2 = fo2[SONG2_FO_PHI];
  double phi_prime_1 = fo1[SONG2_FO_PHI_P], phi_prime_2 = fo2[SONG2_FO_PHI_P];
  double psi_prime_1 = fo1[SONG2_FO_PSI_P], psi_prime_2 = fo2[SONG2_FO_PSI_P];
  double psi = 0, phi_prime = 0, psi_prime = 0, omega_m1_prime = 0, gamma_m2_prime = 0;
  if (c->compute_m[0]) {
    double phi = y[PV->idx_phi];
    psi = w->psi;
    phi_prime = w->phi_prime;
    psi_prime = compute_psi_prime(w, y, dy);
    if (s->use_exponential_potentials) {
      double phi_exp = phi + 2 * phi_1 * phi_2;
      double psi_exp = psi - 2 * psi_1 * psi_2;
      double phi_exp_prime = phi_prime + 2 * (phi_1 * phi_prime_2 + phi_prime_1 * phi_2);
      double psi_exp_prime = psi_prime - 2 * (psi_1 * psi_prime_2 + psi_prime_1 * psi_2);
      phi = phi_exp; psi = psi_exp; phi_prime = phi_exp_prime; psi_prime = psi_exp_prime;
    }
    (void)phi;
  }
  if (c->compute_m[1]) omega_m1_prime = w->omega_m1_prime;
  if (c->compute_m[2]) gamma_m2_prime = y[PV->idx_gamma_p];
  int64_t col = (int64_t)index_tau * w->k3_size + w->index_k3;
  double *base = w->src_flat + w->pair_off + col;
  int dtilde = s->use_delta_tilde_in_los && s->has_quadratic_sources;
  if (s->has_source_T) {
    int switch_sw = s->has_sw ? 1 : 0, switch_isw = s->has_isw ? 1 : 0;
    for (int l = 0; l <= s->l_max_los_t; ++l)
      for (int im = 0; im <= c->index_m_max[l]; ++im) {
        int m = c->m[im];
        double src = 0;
        if (l == 0) {
          src += kappa_dot * w->I_00;
          if (s->has_pure_metric_in_los) src += 4 * phi_prime;
          else {
            src += switch_sw * (4 * kappa_dot * psi);
            src += switch_isw * (4 * (phi_prime + psi_prime));
          }
          if (s->has_quad_metric_in_los && !s->use_exponential_potentials) src += 8 * (phi_1 * phi_prime_2 + phi_2 * phi_prime_1);
        } else if (l == 1) {
          if (s->has_pure_scattering_in_los) src += FOUR_THIRDS * kappa_dot * b(1, 1, m);
          if (s->has_pure_metric_in_los) {
            if (m == 0) src += 4 * k * psi;
            if (m == 1) src += -4 * omega_m1_prime;
          } else if (m == 1)
            src += switch_isw * (-4 * omega_m1_prime);
          if (s->has_quad_metric_in_los) {
            if (!s->use_exponential_potentials)
              src += -4 * (k1_m[m + 1] * psi_1 * (psi_2 - phi_2) + k2_m[m + 1] * psi_2 * (psi_1 - phi_1));
            else
              src += -4 * (k1_m[m + 1] * psi_1 * (-psi_2 - phi_2) + k2_m[m + 1] * psi_2 * (-psi_1 - phi_1));
          }
        } else if (l == 2) {
          if (s->has_pure_scattering_in_los) src += kappa_dot * 0.1 * (w->I_2m[m] - SQRT_6 * w->E_2m[m]);
          /* the reference's tensor metric term sits in a dangling else (perturbations2.c:12298-12302):
             it is added only when has_pure_metric_in_los, for m == 2 */
          if (s->has_pure_metric_in_los && m == 2) src += 4 * gamma_m2_prime;
        }
        if (s->has_quad_scattering_in_los) src += dI_qc2(l, m);
        if (s->has_time_delay_in_los)
          src -= I_2_raw(l + 1) * c_plus_22(l, m) * k2 * (phi_1 + psi_1) - I_2_raw(l - 1) * c_minus_22(l, m) * k2 * (phi_1 + psi_1) +
                 I_1_raw(l + 1) * c_plus_11(l, m) * k1 * (phi_2 + psi_2) - I_1_raw(l - 1) * c_minus_11(l, m) * k1 * (phi_2 + psi_2);
        if (s->has_redshift_in_los)
          src -= -4 * phi_prime_1 * I_2(l, m) + I_2_raw(l + 1) * 4 * c_plus_12(l, m) * k1 * psi_1 -
                 I_2_raw(l - 1) * 4 * c_minus_12(l, m) * k1 * psi_1 - 4 * phi_prime_2 * I_1(l, m) +
                 I_1_raw(l + 1) * 4 * c_plus_21(l, m) * k2 * psi_2 - I_1_raw(l - 1) * 4 * c_minus_21(l, m) * k2 * psi_2;
        if (s->has_lensing_in_los)
          src -= I_2_raw(l + 1) * r_plus_12(l, m) * k1 * (phi_1 + psi_1) - I_2_raw(l - 1) * r_minus_12(l, m) * k1 * (phi_1 + psi_1) +
                 I_1_raw(l + 1) * r_plus_21(l, m) * k2 * (phi_2 + psi_2) - I_1_raw(l - 1) * r_minus_21(l, m) * k2 * (phi_2 + psi_2);
        if (dtilde) src += delta_tilde_source(w, 0, l, m);
        src *= exp_m_kappa;
        base[(int64_t)(c->run->index_tp2_T + RLM(l, m)) * w->per_type] = src;
      }
  }
  if (s->has_source_E) {
    for (int l = 2; l <= s->l_max_los_p; ++l)
      for (int im = 0; im <= c->index_m_max[l]; ++im) {
        int m = c->m[im];
        double src = 0;
        if (l == 2 && s->has_pure_scattering_in_los) src += -SQRT_6 * kappa_dot * 0.1 * (w->I_2m[m] - SQRT_6 * w->E_2m[m]);
        if (s->has_quad_scattering_in_los) src += dE_qc2(l, m);
        if (s->has_time_delay_in_los)
          src -= E_2_raw(l + 1) * d_plus_22(l, m) * k2 * (phi_1 + psi_1) - E_2_raw(l - 1) * d_minus_22(l, m) * k2 * (phi_1 + psi_1) +
                 E_1_raw(l + 1) * d_plus_11(l, m) * k1 * (phi_2 + psi_2) - E_1_raw(l - 1) * d_minus_11(l, m) * k1 * (phi_2 + psi_2);
        if (s->has_redshift_in_los)
          src -= -4 * phi_prime_1 * E_2(l, m) + E_2_raw(l + 1) * 4 * d_plus_12(l, m) * k1 * psi_1 -
                 E_2_raw(l - 1) * 4 * d_minus_12(l, m) * k1 * psi_1 - 4 * phi_prime_2 * E_1(l, m) +
                 E_1_raw(l + 1) * 4 * d_plus_21(l, m) * k2 * psi_2 - E_1_raw(l - 1) * 4 * d_minus_21(l, m) * k2 * psi_2;
        if (s->has_lensing_in_los)
          src -= E_2_raw(l + 1) * k_plus_12(l, m) * k1 * (phi_1 + psi_1) - E_2_raw(l - 1) * k_minus_12(l, m) * k1 * (phi_1 + psi_1) +
                 E_1_raw(l + 1) * k_plus_21(l, m) * k2 * (phi_2 + psi_2) - E_1_raw(l - 1) * k_minus_21(l, m) * k2 * (phi_2 + psi_2);
        if (dtilde) src += delta_tilde_source(w, 1, l, m);
        src *= exp_m_kappa;
        base[(int64_t)(c->run->index_tp2_E + RLM(l, m)) * w->per_type] = src;
      }
  }
  if (s->has_source_B) {
    for (int l = 2; l <= s->l_max_los_p; ++l)
      for (int im = 0; im <= c->index_m_max[l]; ++im) {
        int m = c->m[im];
        if (m == 0) continue;
        double src = 0;
        if (s->has_quad_scattering_in_los) src += dB_qc2(l, m);
        if (s->has_time_delay_in_los) src -= -k2 * E_2_raw(l) * d_zero_22(l, m) * (phi_1 + psi_1) - k1 * E_1_raw(l) * d_zero_11(l, m) * (phi_2 + psi_2);
        if (s->has_redshift_in_los) src -= -E_2_raw(l) * 4 * d_zero_12(l, m) * k1 * psi_1 - E_1_raw(l) * 4 * d_zero_21(l, m) * k2 * psi_2;
        if (s->has_lensing_in_los) src -= -E_2_raw(l) * k_zero_12(l, m) * k1 * (phi_1 + psi_1) - E_1_raw(l) * k_zero_21(l, m) * k2 * (phi_2 + psi_2);
        if (dtilde) src += delta_tilde_source(w, 2, l, m);
        src *= exp_m_kappa;
        base[(int64_t)(c->run->index_tp2_B + RLM(l, m)) * w->per_type] = src;
      }
  }
  if (s->has_source_delta_cdm && c->compute_m[0]) {
    double v_dot_v_cdm = -w->k1_dot_k2 * fo1[SONG2_FO_V_CDM] * fo2[SONG2_FO_V_CDM];
    base[(int64_t)c->run->index_tp2_delta_cdm * w->per_type] = 0.5 * (cdm(0, 0, 0) - 2 * v_dot_v_cdm);
  }
}

/* First-order quantities of one k at tau (the replacement for CLASS's
   ppt->quadsources rows): SONG variables at m = 0 with k along the z axis. */
static void store_first_order(ws_t *w, int index_tau, double tau, const double *y, const double *dy) {
  cfg_t *c = w->c;
  w->st.sources_calls++;
  prepare_tau(w, tau);
  workspace_at_tau(w, y);
  einstein(w, y);
  double k = w->k;
  double *o = w->fo_out + ((size_t)w->index_k1 * w->fo_tau_size + index_tau) * c->nfo;
  memset(o, 0, sizeof(double) * c->nfo);
  double psi_prime = compute_psi_prime(w, y, dy);
  o[SONG2_FO_PHI] = y[PV->idx_phi];
  o[SONG2_FO_PSI] = w->psi;
  o[SONG2_FO_PHI_P] = y[PV->idx_phi_p];
  o[SONG2_FO_PSI_P] = psi_prime;
  o[SONG2_FO_PHI_PP] = dy[PV->idx_phi_p];
  o[SONG2_FO_DELTA_G] = w->I_00;
  o[SONG2_FO_V_G] = -w->I_1m[0] / (4 * k);
  o[SONG2_FO_DELTA_B] = b(0, 0, 0);
  o[SONG2_FO_V_B] = -b(1, 1, 0) / (3 * k);
  o[SONG2_FO_DELTA_B_P] = dy[PV->idx_b + NLM(0, 0, 0)];
  o[SONG2_FO_V_B_P] = -dy[PV->idx_b + NLM(1, 1, 0)] / (3 * k);
  o[SONG2_FO_DELTA_CDM] = cdm(0, 0, 0);
  o[SONG2_FO_V_CDM] = -cdm(1, 1, 0) / (3 * k);
  o[SONG2_FO_V_CDM_P] = -dy[PV->idx_cdm + NLM(1, 1, 0)] / (3 * k);
  o[SONG2_FO_DELTA_UR] = w->N_00;
  o[SONG2_FO_V_UR] = -w->N_1m[0] / (4 * k);
  o[SONG2_FO_DIPOLE_B] = b(1, 1, 0);
  o[SONG2_FO_DIPOLE_CDM] = cdm(1, 1, 0);
  for (int l = 0; l <= c->fo_l_max; ++l) {
    double Il = (l == 0) ? w->I_00 : (l == 1) ? w->I_1m[0] : (l == 2) ? w->I_2m[0] : I(l, 0);
    double El = (l < 2) ? 0.0 : (l == 2) ? w->E_2m[0] : E(l, 0);
    double Nl = (l == 0) ? w->N_00 : (l == 1) ? w->N_1m[0] : N(l, 0);
    double Cl = (l == 0) ? 0.0 : (l == 1) ? w->C_1m[0] / w->kappa_dot
              : (l == 2) ? -w->I_2m[0] + 0.1 * (w->I_2m[0] - SQRT_6 * w->E_2m[0]) : -I(l, 0);
    o[SONG2_FO_I + l] = Il;
    o[c->fo_E + l] = El;
    o[c->fo_N + l] = Nl;
    o[c->fo_CG + l] = Cl;
  }
}

/* ======================================================= NDF15 */

static const double ndf_G[5] = {1.0, 1.5, 11.0 / 6.0, 25.0 / 12.0, 137.0 / 60.0};
static const double ndf_alpha[5] = {-0.1850, -1.0 / 9.0, -0.0823, -0.0415, 0.0};

static double norm_inf_w(int n, const double *x, const double *invwt) {
  double r = 0;
  for (int i = 0; i < n; ++i) {
    double v = fabs(x[i] * invwt[i]);
    if (v > r || v != v) r = (v != v) ? INFINITY : v;
  }
  return r;
}

/* LU with partial pivoting, in place (row major).  Returns 0 or 1 (singular). */
static int lu_factor(int n, double *A, int *piv) {
  for (int kk = 0; kk < n; ++kk) {
    int p = kk;
    double mx = fabs(A[(size_t)kk * n + kk]);
    for (int i = kk + 1; i < n; ++i) {
      double v = fabs(A[(size_t)i * n + kk]);
      if (v > mx) { mx = v; p = i; }
    }
    piv[kk] = p;
    if (mx == 0.0) return 1;
    if (p != kk)
      for (int j = 0; j < n; ++j) {
        double t = A[(size_t)kk * n + j];
        A[(size_t)kk * n + j] = A[(size_t)p * n + j];
        A[(size_t)p * n + j] = t;
      }
    double inv = 1.0 / A[(size_t)kk * n + kk];
    for (int i = kk + 1; i < n; ++i) {
      double f = A[(size_t)i * n + kk] * inv;
      A[(size_t)i * n + kk] = f;
      if (f != 0.0)
        for (int j = kk + 1; j < n; ++j) A[(size_t)i * n + j] -= f * A[(size_t)kk * n + j];
    }
  }
  return 0;
}

static void lu_solve(int n, const double *A, const int *piv, double *b) {
  for (int kk = 0; kk < n; ++kk) {
    int p = piv[kk];
    if (p != kk) { double t = b[kk]; b[kk] = b[p]; b[p] = t; }
  }
  for (int i = 0; i < n; ++i) {
    double s = b[i];
    for (int j = 0; j < i; ++j) s -= A[(size_t)i * n + j] * b[j];
    b[i] = s;
  }
  for (int i = n - 1; i >= 0; --i) {
    double s = b[i];
    for (int j = i + 1; j < n; ++j) s -= A[(size_t)i * n + j] * b[j];
    b[i] = s / A[(size_t)i * n + i];
  }
}

static int form_and_factor(ws_t *w, double hinvGak) {
  int n = PV->n;
  w->st.n_lu++;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) w->M[(size_t)i * n + j] = (i == j ? 1.0 : 0.0) - hinvGak * w->J[(size_t)i * n + j];
  return lu_factor(n, w->M, w->piv);
}

/* dif[:,0..k-1] <- dif[:,0..k-1] * (R(r) U), the backward-difference change of step size */
static void rescale_dif(int n, double *dif, int k, double r) {
  double Rm[5][5], U[5][5], RU[5][5];
  for (int i = 0; i < k; ++i)
    for (int j = 0; j < k; ++j) {
      double prod = 1.0;
      for (int p = 1; p <= i + 1; ++p) prod *= ((p - 1) - (j + 1) * r) / p;
      Rm[i][j] = prod;
      /* U(i,j) = (-1)^(i+1) C(j+1, i+1) (1-based) */
      double binom = 0.0;
      if (j >= i) {
        binom = 1.0;
        for (int p = 1; p <= i + 1; ++p) binom = binom * (j + 1 - (i + 1) + p) / p;
      }
      U[i][j] = ((i + 1) % 2 ? -binom : binom);
    }
  for (int i = 0; i < k; ++i)
    for (int j = 0; j < k; ++j) {
      double s = 0;
      for (int p = 0; p < k; ++p) s += Rm[i][p] * U[p][j];
      RU[i][j] = s;
    }
  double tmp[5];
  for (int e = 0; e < n; ++e) {
    for (int j = 0; j < k; ++j) {
      double s = 0;
      for (int i = 0; i < k; ++i) s += dif[(size_t)e * 7 + i] * RU[i][j];
      tmp[j] = s;
    }
    for (int j = 0; j < k; ++j) dif[(size_t)e * 7 + j] = tmp[j];
  }
}

typedef void (*output_fn)(ws_t *, int, double, const double *, const double *);

/* Integrate y from t0 to t1 and call out() at every tout[j] in (t0, t1]
   (or [t0, t1] when include_t0).  Returns a song2_status_code. */
static int ndf15(ws_t *w, double t0, double t1, double *y, const double *tout, int nout, int *jout,
                 int include_t0, output_fn out) {
  int n = PV->n;
  const song2_spec *s = w->c->s;
  double rtol = s->rtol, threshold = s->threshold;
  const double eps = 2.220446049250313e-16;
  const int maxk = 5, maxit = 4;
  double invGa[5], erconst[5];
  for (int i = 0; i < 5; ++i) {
    invGa[i] = 1.0 / (ndf_G[i] * (1.0 - ndf_alpha[i]));
    erconst[i] = ndf_alpha[i] * ndf_G[i] + 1.0 / (i + 2);
  }
  double *dif = w->dif, *yp = w->dytmp, *ynew = w->ynew, *difkp1 = w->difkp1, *psiv = w->psiv;
  double *rhs = w->rhs, *del = w->del, *invwt = w->invwt, *ftmp = w->ytmp;
  double t = t0, hmax = 0.1 * fabs(t1 - t0);
  /* outputs at t0 */
  while (*jout < nout && tout[*jout] <= t0 && include_t0) {
    if (tout[*jout] == t0) {
      derivs(w, t0, y, yp);
      out(w, *jout, t0, y, yp);
    }
    ++(*jout);
  }
  derivs(w, t, y, yp);
  jacobian(w, t);
  int Jcurrent = 1;
  double htspan = fabs(t1 - t0);
  double hmin = 16 * eps * fabs(t);
  double absh = fmin(hmax, htspan);
  for (int i = 0; i < n; ++i) invwt[i] = 1.0 / fmax(fabs(y[i]), threshold);
  double rh = 1.25 * norm_inf_w(n, yp, invwt) / sqrt(rtol);
  if (absh * rh > 1) absh = 1.0 / rh;
  absh = fmax(absh, hmin);
  double h = absh;
  int k = 1;
  memset(dif, 0, sizeof(double) * (size_t)n * 7);
  for (int i = 0; i < n; ++i) dif[(size_t)i * 7 + 0] = h * yp[i];
  double hinvGak = h * invGa[k - 1];
  int nconhk = 0;
  if (form_and_factor(w, hinvGak)) return SONG2_E_SINGULAR;
  int havrate = 0;
  double rate = 0;
  double abshlast = absh;
  int klast = k;
  int done = 0;
  int nsteps_total = 0;
  while (!done) {
    hmin = 16 * eps * fabs(t);
    absh = fmin(hmax, fmax(hmin, absh));
    h = absh;
    if (1.1 * absh >= fabs(t1 - t)) {
      h = t1 - t;
      absh = fabs(h);
      done = 1;
    }
    if (absh != abshlast || k != klast) {
      rescale_dif(n, dif, k, absh / abshlast);
      hinvGak = h * invGa[k - 1];
      nconhk = 0;
      if (form_and_factor(w, hinvGak)) return SONG2_E_SINGULAR;
      havrate = 0;
    }
    int nofailed = 1;
    double err = 0, tnew = t;
    for (;;) {
      int gotynew = 0;
      while (!gotynew) {
        if (++nsteps_total > s->max_steps) return SONG2_E_MAXSTEPS;
        for (int i = 0; i < n; ++i) {
          double ps = 0, pr = y[i];
          for (int j = 0; j < k; ++j) {
            ps += dif[(size_t)i * 7 + j] * ndf_G[j];
            pr += dif[(size_t)i * 7 + j];
          }
          psiv[i] = ps * invGa[k - 1];
          ynew[i] = pr;
          difkp1[i] = 0.0;
        }
        tnew = t + h;
        if (done) tnew = t1;
        h = tnew - t;
        for (int i = 0; i < n; ++i) invwt[i] = 1.0 / fmax(fmax(fabs(y[i]), fabs(ynew[i])), threshold);
        double minnrm = 100 * eps * norm_inf_w(n, ynew, invwt);
        double oldnrm = 0;
        for (int iter = 1; iter <= maxit; ++iter) {
          derivs(w, tnew, ynew, ftmp);
          for (int i = 0; i < n; ++i) rhs[i] = hinvGak * ftmp[i] - (psiv[i] + difkp1[i]);
          memcpy(del, rhs, sizeof(double) * n);
          lu_solve(n, w->M, w->piv, del);
          double newnrm = norm_inf_w(n, del, invwt);
          for (int i = 0; i < n; ++i) { difkp1[i] += del[i]; ynew[i] += del[i]; }
          if (!(newnrm == newnrm)) break;
          if (newnrm <= minnrm) { gotynew = 1; break; }
          else if (iter == 1) {
            if (havrate) {
              double errit = newnrm * rate / (1 - rate);
              if (errit <= 0.05 * rtol) { gotynew = 1; break; }
            } else rate = 0;
          } else if (newnrm > 0.9 * oldnrm) break;
          else {
            rate = fmax(0.9 * rate, newnrm / oldnrm);
            havrate = 1;
            double errit = newnrm * rate / (1 - rate);
            if (errit <= 0.5 * rtol) { gotynew = 1; break; }
            else if (iter == maxit) break;
            else {
              double rp = 1.0;
              for (int q = 0; q < maxit - iter; ++q) rp *= rate;
              if (0.5 * rtol < errit * rp) break;
            }
          }
          oldnrm = newnrm;
        }
        if (!gotynew) {
          w->st.n_newton_fail++;
          if (absh <= hmin) return SONG2_E_NEWTON;
          if (Jcurrent) {
            double abshold = absh;
            absh = fmax(0.3 * absh, hmin);
            h = absh;
            done = 0;
            rescale_dif(n, dif, k, absh / abshold);
            abshlast = absh; /* dif now corresponds to absh */
            hinvGak = h * invGa[k - 1];
            nconhk = 0;
          } else {
            jacobian(w, t);
            Jcurrent = 1;
          }
          if (form_and_factor(w, hinvGak)) return SONG2_E_SINGULAR;
          havrate = 0;
        }
      }
      for (int i = 0; i < n; ++i)
        if (!(ynew[i] == ynew[i]) || fabs(ynew[i]) > 1e300) return SONG2_E_NAN;
      err = norm_inf_w(n, difkp1, invwt) * erconst[k - 1];
      if (err > rtol) {
        w->st.n_rejected++;
        if (absh <= hmin) return SONG2_E_HMIN;
        double abshl = absh;
        if (nofailed) {
          nofailed = 0;
          double hopt = absh * fmax(0.1, 0.833 * pow(rtol / err, 1.0 / (k + 1)));
          if (k > 1) {
            double errkm1 = 0;
            for (int i = 0; i < n; ++i) {
              double v = fabs((dif[(size_t)i * 7 + k - 1] + difkp1[i]) * invwt[i]);
              if (v > errkm1) errkm1 = v;
            }
            errkm1 *= erconst[k - 2];
            double hkm1 = absh * fmax(0.1, 0.769 * pow(rtol / errkm1, 1.0 / k));
            if (hkm1 > hopt) {
              hopt = fmin(absh, hkm1);
              k = k - 1;
            }
          }
          absh = fmax(hmin, hopt);
        } else {
          absh = fmax(hmin, 0.5 * absh);
        }
        h = absh;
        if (absh < abshl) done = 0;
        rescale_dif(n, dif, k, absh / abshl);
        abshlast = absh;
        klast = k;
        hinvGak = h * invGa[k - 1];
        nconhk = 0;
        if (form_and_factor(w, hinvGak)) return SONG2_E_SINGULAR;
        havrate = 0;
      } else
        break;
    }
    /* accepted */
    w->st.n_steps++;
    for (int i = 0; i < n; ++i) {
      double *d = dif + (size_t)i * 7;
      d[k + 1] = difkp1[i] - d[k];
      d[k] = difkp1[i];
      for (int j = k - 1; j >= 0; --j) d[j] += d[j + 1];
    }
    /* dense output on (t, tnew] */
    while (*jout < nout && tout[*jout] <= tnew) {
      double to = tout[*jout];
      if (to > t || (include_t0 && to == t)) {
        double sv = (to - tnew) / h;
        for (int i = 0; i < n; ++i) {
          double acc = ynew[i], term = 1.0;
          for (int j = 0; j < k; ++j) {
            term *= (sv + j) / (j + 1);
            acc += dif[(size_t)i * 7 + j] * term;
          }
          w->ylin[i] = acc;
        }
        if (to == tnew) memcpy(w->ylin, ynew, sizeof(double) * n);
        derivs(w, to, w->ylin, w->dylin);
        out(w, *jout, to, w->ylin, w->dylin);
      }
      ++(*jout);
    }
    klast = k;
    abshlast = absh;
    nconhk = (nconhk + 1 < maxk + 2) ? nconhk + 1 : maxk + 2;
    if (nconhk >= k + 2) {
      double temp = 1.2 * pow(err / rtol, 1.0 / (k + 1));
      double hopt = (temp > 0.1) ? absh / temp : 10 * absh;
      int kopt = k;
      if (k > 1) {
        double errkm1 = 0;
        for (int i = 0; i < n; ++i) {
          double v = fabs(dif[(size_t)i * 7 + k - 1] * invwt[i]);
          if (v > errkm1) errkm1 = v;
        }
        errkm1 *= erconst[k - 2];
        temp = 1.3 * pow(errkm1 / rtol, 1.0 / k);
        double hkm1 = (temp > 0.1) ? absh / temp : 10 * absh;
        if (hkm1 > hopt) { hopt = hkm1; kopt = k - 1; }
      }
      if (k < maxk) {
        double errkp1 = 0;
        for (int i = 0; i < n; ++i) {
          double v = fabs(dif[(size_t)i * 7 + k + 1] * invwt[i]);
          if (v > errkp1) errkp1 = v;
        }
        errkp1 *= erconst[k];
        temp = 1.4 * pow(errkp1 / rtol, 1.0 / (k + 2));
        double hkp1 = (temp > 0.1) ? absh / temp : 10 * absh;
        if (hkp1 > hopt) { hopt = hkp1; kopt = k + 1; }
      }
      if (hopt > absh) {
        absh = hopt;
        if (k != kopt) k = kopt;
      }
    }
    t = tnew;
    memcpy(y, ynew, sizeof(double) * n);
    Jcurrent = 0;
  }
  return SONG2_OK;
}

/* ======================================================= per-triplet solve */

/* RSA trigger (perturbations2.c:5309-5321) */
static int rsa_is_on(ws_t *w, double tau) {
  const song2_spec *s = w->c->s;
  if (s->radiation_streaming_approximation == SONG2_RSA_NONE || w->c->first_order_mode) return 0;
  return (tau * w->k > s->radiation_streaming_trigger_tau_over_tau_k) && (tau > w->c->t->tau_free_streaming);
}

static int tca_is_on(ws_t *w, double tau) {
  const song2_spec *s = w->c->s;
  if (!s->tight_coupling) return 0;
  background_at_tau(w, tau);
  double tau_c = 1 / w->kappa_dot, tau_h = 1 / w->Hc;
  double kmax = w->k;
  if (w->k1 > kmax) kmax = w->k1;
  if (w->k2 > kmax) kmax = w->k2;
  double tau_k = 1 / kmax;
  return (tau_c / tau_h < s->tca_trigger_tau_c_over_tau_h) && (tau_c / tau_k < s->tca_trigger_tau_c_over_tau_k);
}

static int solve_triplet(ws_t *w, const double *tout, int nout, output_fn out, double *ybuf, char *err) {
  cfg_t *c = w->c;
  const song2_spec *s = c->s;
  double kmax = w->k;
  if (w->k1 > kmax) kmax = w->k1;
  if (w->k2 > kmax) kmax = w->k2;
  double tau_ini;
  if (o_start_time(s, c->t, kmax, tout[0], &tau_ini, err)) return SONG2_E_CONFIG;
  double tau_end = tout[nout - 1];
  /* approximation intervals (perturb2_find_approximation_switches,
     perturbations2.c:4854-5209): TCA from the start until it switches off, then
     the full system, then the RSA once it switches on */
  int tca0 = tca_is_on(w, tau_ini);
  double t_tca = tau_ini;
  if (tca0) {
    if (tca_is_on(w, tau_end)) t_tca = tau_end;
    else {
      double lo = tau_ini, hi = tau_end;
      while ((hi - lo) / lo > s->tol_tau_approx) {
        double mid = 0.5 * (lo + hi);
        if (tca_is_on(w, mid)) lo = mid; else hi = mid;
      }
      t_tca = 0.5 * (lo + hi);
    }
  }
  double t_rsa = tau_end;
  if (t_tca < tau_end && rsa_is_on(w, tau_end)) {
    if (rsa_is_on(w, t_tca)) t_rsa = t_tca;
    else {
      double lo = t_tca, hi = tau_end;
      while ((hi - lo) / lo > s->tol_tau_approx) {
        double mid = 0.5 * (lo + hi);
        if (rsa_is_on(w, mid)) hi = mid; else lo = mid;
      }
      t_rsa = 0.5 * (lo + hi);
    }
  }
  double lim[4];
  int ap[3], nint = 0;
  lim[0] = tau_ini;
  if (tca0) { ap[nint] = 1; lim[++nint] = t_tca; }
  if (lim[nint] < t_rsa) { ap[nint] = 0; lim[++nint] = t_rsa; }
  if (t_rsa < tau_end) { ap[nint] = 2; lim[++nint] = tau_end; }
  build_qs_table(w, tau_ini, tau_end);
  int jout = 0;
  for (int iv = 0; iv < nint; ++iv) {
    if (iv == 0) {
      vector_layout(w, ap[0]);
      initial_conditions(w, lim[0], ybuf);
    } else if (ap[iv] == 2) {
      /* RSA on: the massless hierarchies are dropped, matter and metric carry
         over (perturbations2.c:7105-7300) */
      pv_t old = w->pv;
      double *yold = w->ytmp;
      memcpy(yold, ybuf, sizeof(double) * old.n);
      vector_layout(w, 2);
      pv_t *p = PV;
      memset(ybuf, 0, sizeof(double) * p->n);
      for (int i = 0; i < nlm_hier_b(c); ++i) {
        ybuf[p->idx_b + i] = yold[old.idx_b + i];
        ybuf[p->idx_cdm + i] = yold[old.idx_cdm + i];
      }
      if (c->compute_m[0]) { ybuf[p->idx_phi] = yold[old.idx_phi]; ybuf[p->idx_phi_p] = yold[old.idx_phi_p]; }
      if (c->compute_m[1]) ybuf[p->idx_omega] = yold[old.idx_omega];
      if (c->compute_m[2]) { ybuf[p->idx_gamma] = yold[old.idx_gamma]; ybuf[p->idx_gamma_p] = yold[old.idx_gamma_p]; }
    } else {
      /* TCA -> full remap (perturbations2.c:7233-7285) */
      pv_t old = w->pv;
      double *yold = w->ytmp;
      memcpy(yold, ybuf, sizeof(double) * old.n);
      /* TCA quantities at the switching time, from the old vector, evaluated as in
         derivs (the reference takes them from the last derivs call) */
      prepare_tau_table(w, lim[iv]);
      workspace_at_tau(w, yold);
      double I1[3], I2[3], E2[3], B2[3];
      memcpy(I1, w->I_1m_tca1, sizeof(I1));
      memcpy(I2, w->I_2m_tca1, sizeof(I2));
      memcpy(E2, w->E_2m_tca1, sizeof(E2));
      memcpy(B2, w->B_2m_tca1, sizeof(B2));
      vector_layout(w, 0);
      pv_t *p = PV;
      memset(ybuf, 0, sizeof(double) * p->n);
      for (int i = 0; i < nlm_hier_b(c); ++i) {
        ybuf[p->idx_b + i] = yold[old.idx_b + i];
        ybuf[p->idx_cdm + i] = yold[old.idx_cdm + i];
      }
      if (c->compute_m[0]) { ybuf[p->idx_phi] = yold[old.idx_phi]; ybuf[p->idx_phi_p] = yold[old.idx_phi_p]; }
      if (c->compute_m[1]) ybuf[p->idx_omega] = yold[old.idx_omega];
      if (c->compute_m[2]) { ybuf[p->idx_gamma] = yold[old.idx_gamma]; ybuf[p->idx_gamma_p] = yold[old.idx_gamma_p]; }
      for (int im = 0; im <= c->index_m_max[1]; ++im) ybuf[p->idx_g + LM(1, c->m[im])] = I1[c->m[im]];
      for (int im = 0; im <= c->index_m_max[2]; ++im) {
        int m = c->m[im];
        ybuf[p->idx_g + LM(2, m)] = I2[m];
        if (s->has_polarization2) {
          ybuf[p->idx_E + LM(2, m)] = E2[m];
          ybuf[p->idx_B + LM(2, m)] = B2[m];
        }
      }
      for (int l = 0; l <= old.l_max_g; ++l)
        for (int im = 0; im <= c->index_m_max[l]; ++im)
          ybuf[p->idx_g + LM(l, c->m[im])] = yold[old.idx_g + LM(l, c->m[im])];
      for (int l = 0; l <= s->l_max_ur; ++l)
        for (int im = 0; im <= c->index_m_max[l]; ++im)
          ybuf[p->idx_ur + LM(l, c->m[im])] = yold[old.idx_ur + LM(l, c->m[im])];
    }
    int st = ndf15(w, lim[iv], lim[iv + 1], ybuf, tout, nout, &jout, iv == 0, out);
    if (st != SONG2_OK) return st;
  }
  if (w->st.sources_calls != nout) return SONG2_E_CONFIG;
  return SONG2_OK;
}

/* ======================================================= drivers */

typedef struct { int i1, i2, i3; double *k3row; int k3_size; int64_t pair_off, porder; } trip_t;

static int64_t build_work(const song2_spec *s, trip_t *list) {
  /* k3 grids are concatenated in pair order (i1 ascending, i2 <= i1 ascending) */
  int64_t n = 0, *k3off = (int64_t *)malloc(sizeof(int64_t) * s->k_size * s->k_size);
  int64_t off = 0;
  for (int i1 = 0; i1 < s->k_size; ++i1)
    for (int i2 = 0; i2 <= i1; ++i2) {
      k3off[i1 * s->k_size + i2] = off;
      off += s->k3_size[i1 * s->k_size + i2];
    }
  for (int i1 = s->k_size - 1; i1 >= 0; --i1)
    for (int i2 = 0; i2 <= i1; ++i2) {
      int nk3 = s->k3_size[i1 * s->k_size + i2];
      int64_t po = o_pair_offset(s, i1, i2);
      for (int i3 = 0; i3 < nk3; ++i3) {
        if (list) {
          list[n].i1 = i1; list[n].i2 = i2; list[n].i3 = i3;
          list[n].k3row = (double *)(s->k3 + k3off[i1 * s->k_size + i2]);
          list[n].k3_size = nk3;
          list[n].pair_off = po;
          list[n].porder = k3off[i1 * s->k_size + i2] + i3;
        }
        ++n;
      }
    }
  free(k3off);
  return n;
}

static int evolve_impl(const song2_spec *s, const song2_tables *t, double *src, song2_triplet_stats *stats,
                       const int64_t *sel, int64_t first, int64_t count, int nthreads, char *err);

int song2_oracle_evolve_range(const song2_spec *s, const song2_tables *t, double *src, song2_triplet_stats *stats,
                              int64_t first, int64_t count, int nthreads, char *err) {
  return evolve_impl(s, t, src, stats, NULL, first, count, nthreads, err);
}

int song2_oracle_evolve_list(const song2_spec *s, const song2_tables *t, double *src, song2_triplet_stats *stats,
                             const int64_t *items, int64_t count, int nthreads, char *err) {
  return evolve_impl(s, t, src, stats, items, 0, count, nthreads, err);
}

static int evolve_impl(const song2_spec *s, const song2_tables *t, double *src, song2_triplet_stats *stats,
                       const int64_t *sel, int64_t first, int64_t count, int nthreads, char *err) {
  cfg_t c;
  if (cfg_init(&c, s, t, t->fo_l_max, err)) return 1;
  if (t->fo_l_max < c.L_big + 1) { snprintf(err, SONG2_ERRLEN, "first-order table l_max too small"); cfg_free(&c); return 1; }
  /* hierarchy classes of an uneven batch: the run-wide spec with the class's l_max
     and modes 0..m_max; the source types stay the run-wide ones */
  int ncls = s->n_classes > 0 ? s->n_classes : 0;
  song2_spec *cspec = NULL;
  cfg_t *ccfg = NULL;
  if (ncls) {
    if (!s->class_l_max || !s->class_m_max || !s->triplet_class) {
      snprintf(err, SONG2_ERRLEN, "n_classes > 0 needs class_l_max, class_m_max and triplet_class");
      cfg_free(&c);
      return 1;
    }
    cspec = (song2_spec *)calloc(ncls, sizeof(song2_spec));
    ccfg = (cfg_t *)calloc(ncls, sizeof(cfg_t));
    for (int k = 0; k < ncls; ++k) {
      int L = s->class_l_max[k], mm = s->class_m_max[k];
      int bad = L < 2 || L > s->l_max_g || L > s->l_max_ur || (s->has_polarization2 && L > s->l_max_pol_g) || mm < 0 ||
                mm >= SONG2_MAX_M;
      for (int m = 0; !bad && m <= mm; ++m) bad = !c.compute_m[m];
      cspec[k] = *s;
      cspec[k].n_classes = 0;
      cspec[k].l_max_g = cspec[k].l_max_ur = L;
      if (s->has_polarization2) cspec[k].l_max_pol_g = L;
      cspec[k].m_size = mm + 1;
      for (int m = 0; m <= mm; ++m) cspec[k].m[m] = m;
      if (bad || cfg_init(&ccfg[k], &cspec[k], t, t->fo_l_max, err)) {
        if (bad) snprintf(err, SONG2_ERRLEN, "class %d: l_max or m_max not covered by the run-wide spec", k);
        for (int q = 0; q < k; ++q) cfg_free(&ccfg[q]);
        free(ccfg); free(cspec); cfg_free(&c);
        return 1;
      }
      ccfg[k].run = &c;
    }
  }
  int64_t n = build_work(s, NULL);
  trip_t *list = (trip_t *)malloc(sizeof(trip_t) * (n > 0 ? n : 1));
  build_work(s, list);
  int failed = 0;
  if (first < 0) first = 0;
  if (!sel && first + count > n) count = n - first;
  if (sel)
    for (int64_t i = 0; i < count; ++i)
      if (sel[i] < 0 || sel[i] >= n) { snprintf(err, SONG2_ERRLEN, "bad item"); failed = -1; }
  if (ncls)
    for (int64_t i = 0; i < n; ++i) {
      int k = s->triplet_class[list[i].porder];
      if (k < 0 || k >= ncls) { snprintf(err, SONG2_ERRLEN, "triplet_class entry out of range"); failed = -1; }
    }
  int64_t per_type = (int64_t)s->tau_size * o_n_triplets(s);
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel if (failed == 0)
  {
    ws_t *w = NULL;
    cfg_t *wc = NULL;
    double *ybuf = NULL;
    char lerr[SONG2_ERRLEN];
#pragma omp for schedule(dynamic)
    for (int64_t jt = first; jt < first + count; ++jt) {
      if (failed < 0) continue;
      int64_t it = sel ? sel[jt] : jt;
      trip_t *tr = &list[it];
      cfg_t *tc = ncls ? &ccfg[s->triplet_class[tr->porder]] : &c;
      if (tc != wc) {
        if (w) { ws_free(w); free(ybuf); }
        w = ws_alloc(tc);
        ybuf = (double *)calloc(w->nmax, sizeof(double));
        wc = tc;
      }
      memset(&w->st, 0, sizeof(w->st));
      w->src_flat = src;
      w->per_type = per_type;
      w->pair_off = tr->pair_off;
      w->k3_size = tr->k3_size;
      int stc;
      if (geometrical_corner(w, tr->i1, tr->i2, tr->i3, tr->k3row)) stc = SONG2_E_CONFIG;
      else stc = solve_triplet(w, s->tau, s->tau_size, store_sources, ybuf, lerr);
      w->st.status = stc;
      if (stats) stats[it] = w->st;
      if (stc != SONG2_OK) {
#pragma omp atomic
        failed++;
      }
    }
    if (w) { ws_free(w); free(ybuf); }
  }
  free(list);
  for (int k = 0; k < ncls; ++k) cfg_free(&ccfg[k]);
  free(ccfg);
  free(cspec);
  cfg_free(&c);
  if (failed < 0) return 1;
  if (failed) { snprintf(err, SONG2_ERRLEN, "%d triplets failed", failed); return 1; }
  return 0;
}

int song2_oracle_evolve(const song2_spec *s, const song2_tables *t, double *src, song2_triplet_stats *stats,
                        int nthreads, char *err) {
  return song2_oracle_evolve_range(s, t, src, stats, 0, o_n_triplets(s), nthreads, err);
}

int song2_oracle_first_order(const song2_spec *s2, const song2_tables *t, int fo_l_max, int fo_tau_size,
                             double fo_lntau0, double fo_dlntau, double *fo_out, int nthreads, char *err) {
  song2_spec s = *s2;
  s.ic = SONG2_IC_AD_FIRST_ORDER;
  /* first-order normalisation: primordial curvature zeta = 1, i.e. C = -1/2 in
     the has_ad_first_order initial conditions (fnl_phi = 5/6 there) */
  s.primordial_local_fnl_phi = 5.0 / 6.0;
  s.m_size = 1; s.m[0] = 0;
  s.has_quadratic_sources = 0;
  s.has_source_T = s.has_source_E = s.has_source_B = s.has_source_delta_cdm = 0;
  /* evolve more multipoles than stored, so the truncation stays away from the table */
  s.l_max_g = s.l_max_pol_g = s.l_max_ur = fo_l_max + 5;
  s.l_max_los_t = s.l_max_los_p = 0;
  cfg_t c;
  if (cfg_init(&c, &s, t, fo_l_max, err)) return 1;
  double *tq = (double *)malloc(sizeof(double) * fo_tau_size);
  for (int i = 0; i < fo_tau_size; ++i) tq[i] = exp(fo_lntau0 + i * fo_dlntau);
  int failed = 0;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel
  {
    ws_t *w = ws_alloc(&c);
    double *ybuf = (double *)calloc(w->nmax, sizeof(double));
    char lerr[SONG2_ERRLEN];
#pragma omp for schedule(dynamic)
    for (int ik = 0; ik < s.k_size; ++ik) {
      memset(&w->st, 0, sizeof(w->st));
      double kk = s.k[ik];
      double krow[1] = {kk};
      w->fo_out = fo_out;
      w->fo_tau_size = fo_tau_size;
      /* equilateral (k,k,k): with no quadratic sources the result depends on k only */
      int stc;
      {
        /* geometrical_corner reads s->k[index]; use the triplet (ik, ik, 0) with k3 = k */
        stc = geometrical_corner(w, ik, ik, 0, krow) ? SONG2_E_CONFIG : SONG2_OK;
      }
      if (stc == SONG2_OK) stc = solve_triplet(w, tq, fo_tau_size, store_first_order, ybuf, lerr);
      if (stc != SONG2_OK) {
#pragma omp atomic
        failed++;
      }
    }
    free(ybuf);
    ws_free(w);
  }
  free(tq);
  cfg_free(&c);
  if (failed) { snprintf(err, SONG2_ERRLEN, "%d first-order modes failed", failed); return 1; }
  return 0;
}

int song2_oracle_rhs(const song2_spec *s, const song2_tables *t, int i1, int i2, int i3, int tca, double tau,
                     const double *y, double *dy, char *err) {
  cfg_t c;
  if (cfg_init(&c, s, t, t->fo_l_max, err)) return -1;
  int64_t n = build_work(s, NULL);
  trip_t *list = (trip_t *)malloc(sizeof(trip_t) * n);
  build_work(s, list);
  double *k3row = NULL;
  for (int64_t i = 0; i < n; ++i)
    if (list[i].i1 == i1 && list[i].i2 == i2) { k3row = list[i].k3row; break; }
  ws_t *w = ws_alloc(&c);
  int nn = -1;
  if (k3row && !geometrical_corner(w, i1, i2, i3, k3row)) {
    vector_layout(w, tca);
    derivs(w, tau, y, dy);
    nn = w->pv.n;
  }
  ws_free(w);
  free(list);
  cfg_free(&c);
  return nn;
}

int song2_oracle_geometry_checks(const song2_spec *s, int i1, int i2, int i3, double *max_dev) {
  song2_tables dummy;
  memset(&dummy, 0, sizeof(dummy));
  cfg_t c;
  char err[SONG2_ERRLEN];
  if (cfg_init(&c, s, &dummy, 0, err)) return 99;
  int64_t n = build_work(s, NULL);
  trip_t *list = (trip_t *)malloc(sizeof(trip_t) * n);
  build_work(s, list);
  double *k3row = NULL;
  for (int64_t i = 0; i < n; ++i)
    if (list[i].i1 == i1 && list[i].i2 == i2) { k3row = list[i].k3row; break; }
  ws_t *w = ws_alloc(&c);
  int fails = 0;
  double dev = 0;
  if (!k3row || geometrical_corner(w, i1, i2, i3, k3row)) fails = 100;
  else {
    cfg_t *cc = &c;
    double k1 = w->k1, k2 = w->k2, k = w->k;
    double sink1k = sqrt(1 - w->cosk1k * w->cosk1k), sink2k = sqrt(1 - w->cosk2k * w->cosk2k);
    double kz1 = k1 * w->cosk1k, kz2 = k2 * w->cosk2k, kx1 = k1 * sink1k, kx2 = -k2 * sink2k;
#define CHK(x, tol) do { double _d = fabs(x); if (_d > dev) dev = _d; if (_d > (tol)) ++fails; } while (0)
    CHK((k1 * sink1k - k2 * sink2k) / k1, 1e-8);  /* 1e4 * _SMALL_ in the reference */
    CHK((k - (kz1 + kz2)) / k, 1e-12);
    CHK((kx1 + kx2) / k, 1e-8);
    CHK(1 - kz1 / w->k1_m[1], 1e-12);
    CHK(1 - kz2 / w->k2_m[1], 1e-12);
    /* the l = 1 rotation coefficients are the spherical components of the unit
       vectors, divided by sin(theta_k1) when rescaled (:5953-5970) */
    int resc = s->rescale_cmb_sources;
    double k1_P1_cart = -kx1 / SQRT_2, k2_P1_cart = -kx2 / SQRT_2;
    if (resc) { k1_P1_cart /= sink1k; k2_P1_cart = k2_P1_cart / sink2k * k1 / k2; }
    /* sin(theta) from 1 - cos^2 loses digits as 1/sin^2: near-collinear triangles
       are checked to that conditioning */
    double cond = 1.0 / fmin(1.0, 1e4 * sink1k * sink1k);
    if (fabs(kx1) > 1e-6 * k1) {
      CHK(1 - k1_P1_cart / w->k1_m[2], 1e-8 * cond);
      CHK(1 - k2_P1_cart / w->k2_m[2], 1e-8 * cond);
    }
    if (resc && fabs(kx1) > 1e-6 * k1) {
      /* rescaled k1 (x) k2 times sin^m equals the Cartesian, unrescaled one (:6025-6064) */
      double u1M = kx1 / SQRT_2, u1P = -u1M, u2M = kx2 / SQRT_2, u2P = -u2M;
      double t[3] = {kz1 * kz2 - w->k1_dot_k2 / 3., (u1P * kz2 + u2P * kz1) / SQRT_3, SQRT_2 / SQRT_3 * u1P * u2P};
      (void)u1M; (void)u2M;
      for (int m = 0; m <= 2; ++m) {
        double un = w->k1_ten_k2[m + 2] * pow(sink1k, m);
        if (fabs(un) > 1e-30) CHK((t[m] - un) / (k1 * k2), 1e-8 * cond);
      }
    }
    double k1k2s = w->k1_m[1] * w->k2_m[1] - w->k1_m[0] * w->k2_m[2] - w->k1_m[2] * w->k2_m[0];
    CHK((k1k2s - w->k1_dot_k2) / (k1 * k2), 1e-8);
    CHK(w->rot1[0] - 1.0, 1e-14);
    if (cc->compute_m[0]) {
      CHK(w->cm12[cc->lm_array[0][cc->index_m[0]]], 1e-14);
      double r12 = w->rot1[cc->lm_quad[1][0]] * w->rot2[0];
      if (fabs(r12) > 1e-12) CHK(1 - w->cm12[cc->lm_array[1][cc->index_m[0]]] / r12, 1e-12);
      for (int l = 0; l <= cc->L_big; ++l) CHK(w->dz12[cc->lm_array[l][cc->index_m[0]]], 1e-12);
    }
    for (int im = 0; im <= cc->index_m_max[2]; ++im) {
      int m = cc->m[im];
      int lm = cc->lm_array[2][im];
      CHK((k1 * k2 * w->cm12[lm] - w->k1_ten_k2[m + 2]) / (k1 * k2), 1e-8);
      CHK((k1 * k1 * w->cm11[lm] - w->k1_ten_k1[m + 2]) / (k1 * k1), 1e-8);
      CHK((k2 * k2 * w->cm22[lm] - w->k2_ten_k2[m + 2]) / (k2 * k2), 1e-8);
    }
#undef CHK
  }
  if (max_dev) *max_dev = dev;
  ws_free(w);
  free(list);
  cfg_free(&c);
  return fails;
}
