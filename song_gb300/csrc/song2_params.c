/* song2_params.c - reader of the reference's ini/pre parameter files for the
 * keys of the hot path: the problem (song2_spec), its grids and the
 * line-of-sight settings (input2.c:137-2016 parses them into ppt2/ppr2/ptr2/pbs2).
 *
 * File format (CLASS's parser): one `name = value` per line, '#' starts a
 * comment, blank lines and lines without '=' are ignored, names and values are
 * trimmed; the ini and pre files form one list and a name may appear only once.
 */
#include <ctype.h>
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "song2.h"

#define P_MAXN 512
#define P_KEY 128
#define P_VAL 512

typedef struct {
  int n;
  char key[P_MAXN][P_KEY];
  char val[P_MAXN][P_VAL];
  char src[P_MAXN][16];
} plist;

static char *trim(char *s) {
  while (*s && isspace((unsigned char)*s)) ++s;
  char *e = s + strlen(s);
  while (e > s && isspace((unsigned char)e[-1])) *--e = 0;
  return s;
}

static int read_file(const char *path, const char *tag, plist *pl, char *err) {
  if (!path) return 0;
  FILE *f = fopen(path, "r");
  if (!f) {
    snprintf(err, SONG2_ERRLEN, "cannot open %.900s", path);
    return 1;
  }
  char line[2048];
  int ln = 0;
  while (fgets(line, sizeof line, f)) {
    ++ln;
    char *h = strchr(line, '#');
    if (h) *h = 0;
    char *eq = strchr(line, '=');
    if (!eq) continue;
    *eq = 0;
    char *k = trim(line), *v = trim(eq + 1);
    if (!*k) continue;
    for (int i = 0; i < pl->n; ++i)
      if (!strcmp(pl->key[i], k)) {
        snprintf(err, SONG2_ERRLEN, "multiple entries of '%.100s' (%s and %s:%d)", k, pl->src[i], tag, ln);
        fclose(f);
        return 1;
      }
    if (pl->n >= P_MAXN || strlen(k) >= P_KEY || strlen(v) >= P_VAL) {
      snprintf(err, SONG2_ERRLEN, "parameter list too long at %s:%d", tag, ln);
      fclose(f);
      return 1;
    }
    strcpy(pl->key[pl->n], k);
    strcpy(pl->val[pl->n], v);
    snprintf(pl->src[pl->n], sizeof pl->src[0], "%s:%d", tag, ln);
    pl->n++;
  }
  fclose(f);
  return 0;
}

static const char *get(const plist *pl, const char *k) {
  for (int i = 0; i < pl->n; ++i)
    if (!strcmp(pl->key[i], k)) return pl->val[i];
  return NULL;
}

/* the newer name wins over its obsolete alias (input2.c reads the alias first) */
static const char *get2(const plist *pl, const char *old_name, const char *new_name) {
  const char *v = get(pl, new_name);
  return v ? v : get(pl, old_name);
}

static int yes(const char *v) { return v && (strchr(v, 'y') || strchr(v, 'Y')); }

static int num(const char *v, const char *k, double *out, char *err) {
  char *end;
  double d = strtod(v, &end);
  if (end == v || *trim(end)) {
    snprintf(err, SONG2_ERRLEN, "'%s = %.200s' is not a number", k, v);
    return 1;
  }
  *out = d;
  return 0;
}

#define RD_D(name, dst)                                  \
  do {                                                   \
    const char *v_ = get(pl, name);                      \
    if (v_ && num(v_, name, &(dst), err)) return 1;      \
  } while (0)
#define RD_D2(old, name, dst)                            \
  do {                                                   \
    const char *v_ = get2(pl, old, name);                \
    if (v_ && num(v_, name, &(dst), err)) return 1;      \
  } while (0)
#define RD_I2(old, name, dst)                            \
  do {                                                   \
    const char *v_ = get2(pl, old, name);                \
    double d_;                                           \
    if (v_) {                                            \
      if (num(v_, name, &d_, err)) return 1;             \
      (dst) = (int)d_;                                   \
    }                                                    \
  } while (0)

void song2_params_defaults(song2_params *g) {
  memset(g, 0, sizeof(*g));
  /* input2.c:2071-2075, 2316-2325: smart samplings, custom grids as below */
  g->k_sampling = SONG2_SAMPLING_SMART;
  g->k_min = 1e-4;
  g->k_max = 0.1;
  g->k_size = 10;
  g->k3_sampling = SONG2_SAMPLING_SMART;
  g->k3_size = 100;
  g->custom_tau = 0;
  g->tau_sampling = SONG2_SAMPLING_LIN;
  g->tau_ini = 1;
  g->tau_end = 0;
  g->tau_size = 2000;
  /* CLASS's l sampling of the Bessel module */
  g->l_max_scalars = 2500;
  g->l_logstep = 1.12;
  g->l_linstep = 40;
  /* smart sampling (input2.c:2290-2299, 2175, 2316) */
  g->k_min_tau0 = 0.1;
  g->k_max_tau0_over_l_max = 2;
  g->k_step_sub = 0.1;
  g->k_step_super = 0.025;
  g->k_logstep_super = 1.8;
  g->k_step_transition = 0.2;
  g->k_per_decade_for_pk = 10;
  g->k_per_decade_for_bao = 70;
  g->k_bao_center = 3;
  g->k_bao_width = 4;
  g->k_max_for_pk = 0.1;
  g->h = 0.67556;
  g->k3_size_min = 5;
  g->has_cmb = 0;
  g->has_lss = 0;
  /* input2.c:2278-2279; CLASS's precision default for the start */
  g->tau_stepsize = 0.4;
  g->tau_late_boost = 1;
  g->tau_start_c_over_h = 0.008;
}

static int sampling(const char *v, const char *k, int *out, char *err) {
  if (!strcmp(v, "lin") || !strcmp(v, "linear")) *out = SONG2_SAMPLING_LIN;
  else if (!strcmp(v, "log") || !strcmp(v, "logarithmic")) *out = SONG2_SAMPLING_LOG;
  else if (!strcmp(v, "smart") || !strcmp(v, "class")) *out = SONG2_SAMPLING_SMART;
  else if (!strcmp(v, "sym") || !strcmp(v, "symmetric")) *out = SONG2_SAMPLING_SYM;
  else if (!strcmp(v, "theta_12")) *out = SONG2_SAMPLING_THETA12;
  else {
    snprintf(err, SONG2_ERRLEN, "%s = %.200s is not a sampling the reference knows", k, v);
    return 1;
  }
  return 0;
}

int song2_read_params(const char *ini_path, const char *pre_path, song2_spec *s, song2_params *g,
                      song2_los_spec *los, char *err) {
  static plist list;  /* large; the reader is not reentrant */
  plist *pl = &list;
  pl->n = 0;
  if (read_file(ini_path, "ini", pl, err) || read_file(pre_path, "pre", pl, err)) return 1;
  song2_spec_defaults(s);
  s->radiation_streaming_approximation = SONG2_RSA_MD; /* the reference's default (input2.c:2139) */
  song2_params_defaults(g);

  /* output: which line-of-sight sources (input2.c:209-277, perturbations2.c:843-945) */
  int has_t = 0, has_e = 0, has_b = 0, has_cdm = 0, stop_p2 = 0, stop_t2 = 0;
  const char *v = get(pl, "output");
  if (v) {
    if (strstr(v, "tBisp") || strstr(v, "TBISP") || strstr(v, "tCl2") || strstr(v, "TCL2")) has_t = 1;
    if (strstr(v, "pBisp") || strstr(v, "PBISP") || strstr(v, "eBisp") || strstr(v, "EBISP") || strstr(v, "pCl2") ||
        strstr(v, "PCL2") || strstr(v, "eCl2") || strstr(v, "ECL2"))
      has_e = 1;
    if (strstr(v, "bBisp") || strstr(v, "BBISP") || strstr(v, "bCl2") || strstr(v, "BCL2")) has_b = 1;
    if (strstr(v, "delta_cdm_pk") || strstr(v, "pk_delta_cdm") || strstr(v, "mPk") || strstr(v, "delta_cdm_bk") ||
        strstr(v, "bk_delta_cdm") || strstr(v, "mBisp"))
      has_cdm = 1;
    if (strstr(v, "stop_at_perturbations2") || strstr(v, "P2")) stop_p2 = 1;
    if (strstr(v, "stop_at_transfers2") || strstr(v, "T2")) stop_t2 = 1;
  }

  /* physics switches (input2.c:534-760) */
  if ((v = get(pl, "quadratic_sources")) && !yes(v)) s->has_quadratic_sources = 0;
  if ((v = get(pl, "quadratic_liouville")) && !yes(v)) s->has_quadratic_liouville = 0;
  if ((v = get(pl, "quadratic_collision")) && !yes(v)) s->has_quadratic_collision = 0;
  if (!s->has_quadratic_sources) s->has_quadratic_liouville = s->has_quadratic_collision = 0;
  if ((v = get(pl, "polarization_second_order")) && !yes(v)) s->has_polarization2 = 0;
  if ((v = get(pl, "perfect_baryons")) && !yes(v)) {
    snprintf(err, SONG2_ERRLEN, "perfect_baryons = no (imperfect baryons) is not supported");
    return 1;
  }
  if ((v = get(pl, "perfect_cdm")) && !yes(v)) {
    snprintf(err, SONG2_ERRLEN, "perfect_cdm = no (imperfect CDM) is not supported");
    return 1;
  }
  RD_D2("tol_perturb_integration_2nd_order", "tol_perturb_integration_song", s->rtol);
  if ((v = get(pl, "perturbed_recombination_song")) && yes(v)) {
    snprintf(err, SONG2_ERRLEN, "perturbed_recombination_song = yes is not supported");
    return 1;
  }
  s->has_pure_scattering_in_los = yes(get2(pl, "include_pure_scattering_in_los_2nd_order", "include_pure_scattering_song"));
  s->has_quad_scattering_in_los = yes(get2(pl, "include_quad_scattering_in_los_2nd_order", "include_quad_scattering_song"));
  {
    const char *m1 = get(pl, "include_metric_in_los_2nd_order"), *m2 = get(pl, "include_metric_song"),
               *m3 = get(pl, "include_pure_metric_song");
    s->has_pure_metric_in_los = yes(m3 ? m3 : (m2 ? m2 : m1));
  }
  s->has_quad_metric_in_los = yes(get2(pl, "include_quad_metric_in_los_2nd_order", "include_quad_metric_song"));
  s->has_time_delay_in_los = yes(get2(pl, "include_time_delay_in_los_2nd_order", "include_time_delay_song"));
  s->has_redshift_in_los = yes(get2(pl, "include_redshift_in_los_2nd_order", "include_redshift_song"));
  s->has_lensing_in_los = yes(get2(pl, "include_lensing_in_los_2nd_order", "include_lensing_song"));
  s->has_sw = yes(get2(pl, "include_sachs_wolfe_in_los_2nd_order", "include_sachs_wolfe_song"));
  s->has_isw = yes(get2(pl, "include_integrated_sachs_wolfe_in_los_2nd_order", "include_integrated_sachs_wolfe_song"));
  if (s->has_sw || s->has_isw) s->has_pure_metric_in_los = 0;
  s->use_delta_tilde_in_los = yes(get(pl, "use_delta_tilde_in_los"));
  s->use_exponential_potentials = yes(get(pl, "use_exponential_potentials"));
  if (s->has_isw && yes(get(pl, "only_early_isw"))) {
    snprintf(err, SONG2_ERRLEN, "only_early_isw = yes is not supported");
    return 1;
  }
  if (s->use_delta_tilde_in_los && s->has_redshift_in_los) {
    snprintf(err, SONG2_ERRLEN, "the delta_tilde options are not compatible with the redshift term");
    return 1;
  }
  if ((v = get2(pl, "phi_prime_equation", "phi_equation_song")) && !strstr(v, "huang")) {
    snprintf(err, SONG2_ERRLEN, "phi_equation_song = %.200s: only the Huang equation is supported", v);
    return 1;
  }
  if ((v = get2(pl, "ic_2nd_order", "ic_song"))) {
    if (!strcmp(v, "ad") || !strcmp(v, "AD")) s->ic = SONG2_IC_AD;
    else if (strstr(v, "ad_first_order") || strstr(v, "AD_1ST") || strstr(v, "ad1")) s->ic = SONG2_IC_AD_FIRST_ORDER;
    else if (strstr(v, "zero") || strstr(v, "ZERO")) s->ic = SONG2_IC_ZERO;
    else {
      snprintf(err, SONG2_ERRLEN, "ic_song = %.200s not supported (ad, ad_first_order, zero)", v);
      return 1;
    }
  }
  RD_D("primordial_local_fnl_phi", s->primordial_local_fnl_phi);
  RD_I2("tight_coupling_approximation_2nd_order", "tight_coupling_approximation_song", s->tight_coupling);
  RD_D2("tight_coupling_trigger_tau_c_over_tau_h_2nd_order", "tight_coupling_trigger_tau_c_over_tau_h_song",
        s->tca_trigger_tau_c_over_tau_h);
  RD_D2("tight_coupling_trigger_tau_c_over_tau_k_2nd_order", "tight_coupling_trigger_tau_c_over_tau_k_song",
        s->tca_trigger_tau_c_over_tau_k);
  RD_I2("radiation_streaming_approximation_2nd_order", "radiation_streaming_approximation_song",
        s->radiation_streaming_approximation);
  RD_D2("radiation_streaming_trigger_tau_over_tau_k_2nd_order", "radiation_streaming_trigger_tau_over_tau_k_song",
        s->radiation_streaming_trigger_tau_over_tau_k);
  if (s->tight_coupling < 0 || s->tight_coupling > 1 || s->radiation_streaming_approximation < 0 ||
      s->radiation_streaming_approximation > 2) {
    snprintf(err, SONG2_ERRLEN, "unknown tight-coupling (%d) or radiation-streaming (%d) method", s->tight_coupling,
             s->radiation_streaming_approximation);
    return 1;
  }
  RD_D2("start_small_k_at_tau_c_over_tau_h_2nd_order", "start_small_k_at_tau_c_over_tau_h_song",
        s->start_small_k_at_tau_c_over_tau_h);
  RD_D2("start_large_k_at_tau_h_over_tau_k_2nd_order", "start_large_k_at_tau_h_over_tau_k_song",
        s->start_large_k_at_tau_h_over_tau_k);

  /* hierarchies and line of sight (input2.c:1748-1880) */
  RD_I2("l_max_g_2nd_order", "l_max_g_song", s->l_max_g);
  RD_I2("l_max_pol_g_2nd_order", "l_max_pol_g_song", s->l_max_pol_g);
  RD_I2("l_max_ur_2nd_order", "l_max_ur_song", s->l_max_ur);
  {
    const char *vt = get2(pl, "l_max_T_los", "l_max_los_t");
    const char *vp = get(pl, "l_max_los_p");
    if (!vp) vp = get(pl, "l_max_B_los");
    if (!vp) vp = get(pl, "l_max_E_los");
    double d;
    if (vt) {
      if (num(vt, "l_max_los_t", &d, err)) return 1;
      s->l_max_los_t = (int)d;
    }
    if (vp) {
      if (num(vp, "l_max_los_p", &d, err)) return 1;
      s->l_max_los_p = (int)d;
    }
    vt = get2(pl, "l_max_T_quadratic_los", "l_max_los_quadratic_t");
    vp = get(pl, "l_max_los_quadratic_p");
    if (!vp) vp = get(pl, "l_max_B_quadratic_los");
    if (!vp) vp = get(pl, "l_max_E_quadratic_los");
    if (vt) {
      if (num(vt, "l_max_los_quadratic_t", &d, err)) return 1;
      s->l_max_los_quadratic_t = (int)d;
    }
    if (vp) {
      if (num(vp, "l_max_los_quadratic_p", &d, err)) return 1;
      s->l_max_los_quadratic_p = (int)d;
    }
  }
  if ((v = get2(pl, "modes_2nd_order", "modes_song"))) {
    char buf[P_VAL];
    strcpy(buf, v);
    int n = 0;
    for (char *tok = strtok(buf, ","); tok; tok = strtok(NULL, ",")) {
      double d;
      if (num(trim(tok), "modes_song", &d, err)) return 1;
      if (n >= SONG2_MAX_M) {
        snprintf(err, SONG2_ERRLEN, "modes_song holds more than %d values", SONG2_MAX_M);
        return 1;
      }
      s->m[n++] = (int)d;
    }
    s->m_size = n;
    for (int i = 0; i + 1 < n; ++i)
      if (s->m[i] >= s->m[i + 1]) {
        snprintf(err, SONG2_ERRLEN, "the m-list provided in modes_song is not strictly ascending");
        return 1;
      }
    if (n < 1 || s->m[0] < 0 || s->m[n - 1] >= SONG2_MAX_M) {
      snprintf(err, SONG2_ERRLEN, "modes_song must hold values in 0..%d", SONG2_MAX_M - 1);
      return 1;
    }
  }
  int m_max = s->m[s->m_size - 1];
  s->has_source_T = has_t;
  s->has_source_E = has_e || has_b;
  s->has_source_B = (has_e || has_b) && m_max != 0;
  s->has_source_delta_cdm = has_cdm;
  if (!s->has_polarization2 && (has_e || has_b)) {
    snprintf(err, SONG2_ERRLEN, "polarization_second_order must be yes for E or B outputs");
    return 1;
  }
  /* rescaling of the CMB sources (input2.c:1955-1971) */
  s->rescale_cmb_sources = !(stop_p2 || stop_t2) && m_max != 0;
  g->has_cmb = has_t || has_e || has_b;
  g->has_lss = has_cdm;

  /* grids (input2.c:320-530) */
  if ((v = get(pl, "sources2_k_sampling")) && sampling(v, "sources2_k_sampling", &g->k_sampling, err)) return 1;
  RD_D2("k_min_scalars", "k_min_custom_song", g->k_min);
  RD_D2("k_max_scalars", "k_max_custom_song", g->k_max);
  RD_I2("k_size_scalars", "k_size_custom_song", g->k_size);
  if ((v = get(pl, "sources2_k3_sampling")) && sampling(v, "sources2_k3_sampling", &g->k3_sampling, err)) return 1;
  {
    double d;
    if ((v = get(pl, "k3_size"))) {
      if (num(v, "k3_size", &d, err)) return 1;
      g->k3_size = (int)d;
    }
  }
  v = get2(pl, "custom_time_sampling_for_2nd_order_sources", "custom_time_sampling_song_sources");
  g->custom_tau = yes(v);
  RD_D2("custom_tau_ini_2nd_order_sources", "custom_tau_ini_song_sources", g->tau_ini);
  RD_D2("custom_tau_end_2nd_order_sources", "custom_tau_end_song_sources", g->tau_end);
  RD_I2("custom_tau_size_2nd_order_sources", "custom_tau_size_song_sources", g->tau_size);
  if ((v = get2(pl, "custom_tau_mode_2nd_order_sources", "custom_tau_mode_song_sources"))) {
    if (strstr(v, "lin") || strstr(v, "LIN")) g->tau_sampling = SONG2_SAMPLING_LIN;
    else if (strstr(v, "log") || strstr(v, "LOG")) g->tau_sampling = SONG2_SAMPLING_LOG;
    else {
      snprintf(err, SONG2_ERRLEN, "custom_tau_mode_song_sources = %.200s (lin or log)", v);
      return 1;
    }
  }
  /* the intrinsic bispectrum's interpolation in k1, k2 and its r sampling size */
  if ((v = get(pl, "transfers_k1_interpolation")))
    g->bi_k1_interpolation = strstr(v, "cubic") ? SONG2_INTERP_CUBIC : SONG2_INTERP_LINEAR;
  if ((v = get(pl, "transfers_k2_interpolation")))
    g->bi_k2_interpolation = strstr(v, "cubic") ? SONG2_INTERP_CUBIC : SONG2_INTERP_LINEAR;
  {
    double d;
    if ((v = get(pl, "r_size"))) {
      if (num(v, "r_size", &d, err)) return 1;
      if (d < 2) {
        snprintf(err, SONG2_ERRLEN, "r_size = %g must be at least 2", d);
        return 1;
      }
      g->bi_r_size = (int)d;
    }
  }
  /* input2.c:362-377 (the first key is the obsolete spelling) */
  RD_D2("perturb_sampling_stepsize_for_2nd_order", "perturb_sampling_stepsize_song", g->tau_stepsize);
  RD_D("perturb_sampling_late_time_boost", g->tau_late_boost);
  RD_D("start_sources_at_tau_c_over_tau_h", g->tau_start_c_over_h);
  if (g->tau_stepsize <= 0) {
    snprintf(err, SONG2_ERRLEN, "perturb_sampling_stepsize_song = %g must be positive", g->tau_stepsize);
    return 1;
  }
  if (g->custom_tau && g->tau_ini <= 0) {
    snprintf(err, SONG2_ERRLEN, "please choose 'tau_ini' greater than zero");
    return 1;
  }
  /* smart k sampling (input2.c:405-470) */
  RD_D2("k_scalar_min_tau0_2nd_order", "k_min_tau0_song", g->k_min_tau0);
  RD_D2("k_scalar_max_tau0_over_l_max_2nd_order", "k_max_tau0_over_l_max_song", g->k_max_tau0_over_l_max);
  RD_D2("k_scalar_step_sub_2nd_order", "k_step_sub_song", g->k_step_sub);
  {
    const char *a = get(pl, "k_scalar_linstep_super_2nd_order"), *b = get(pl, "k_linstep_super_2nd_order"),
               *c = get(pl, "k_step_super_song");
    const char *w = c ? c : (b ? b : a);
    if (w && num(w, "k_step_super_song", &g->k_step_super, err)) return 1;
  }
  RD_D2("k_scalar_logstep_super_2nd_order", "k_logstep_super_song", g->k_logstep_super);
  RD_D2("k_scalar_step_transition_2nd_order", "k_step_transition_song", g->k_step_transition);
  RD_D("k_per_decade_for_pk_song", g->k_per_decade_for_pk);
  RD_D("k_per_decade_for_bao_song", g->k_per_decade_for_bao);
  RD_D("k_bao_center", g->k_bao_center);
  RD_D("k_bao_width", g->k_bao_width);
  RD_D("h", g->h);
  if (g->k_logstep_super <= 1) {
    snprintf(err, SONG2_ERRLEN, "logarithmic step must be larger than 1");
    return 1;
  }
  if (g->has_lss) {
    const char *ph = get(pl, "P_k_max_h/Mpc_song"), *p1 = get(pl, "P_k_max_1/Mpc_song");
    if (ph && p1) {
      snprintf(err, SONG2_ERRLEN, "you cannot enter both P_k_max_h/Mpc and P_k_max_1/Mpc, choose one");
      return 1;
    }
    double d;
    if (ph) {
      if (num(ph, "P_k_max_h/Mpc_song", &d, err)) return 1;
      g->k_max_for_pk = d * g->h;
    }
    if (p1) {
      if (num(p1, "P_k_max_1/Mpc_song", &d, err)) return 1;
      g->k_max_for_pk = d;
    }
    RD_D("k_max_for_pk", g->k_max_for_pk);
  }
  {
    double d;
    if ((v = get(pl, "k3_size_min"))) {
      if (num(v, "k3_size_min", &d, err)) return 1;
      g->k3_size_min = (int)d;
    }
  }
  /* CLASS's l sampling keys */
  {
    double d;
    if ((v = get(pl, "l_max_scalars"))) {
      if (num(v, "l_max_scalars", &d, err)) return 1;
      g->l_max_scalars = (int)d;
    }
    RD_D("l_logstep", g->l_logstep);
    if ((v = get(pl, "l_linstep"))) {
      if (num(v, "l_linstep", &d, err)) return 1;
      g->l_linstep = (int)d;
    }
  }

  /* line of sight (input2.c:1433-1543, 1699-1740) */
  if (los) {
    song2_los_spec keep = *los;
    song2_los_defaults(los, NULL, NULL);
    los->l_size = keep.l_size;
    los->l = keep.l;
    los->tau0 = keep.tau0;
    los->tau_rec = keep.tau_rec;
    if ((v = get2(pl, "transfer2_k_sampling", "transfer2_k3_sampling"))) {
      if (strstr(v, "bessel")) los->k3_sampling = SONG2_K3_SAMPLING_BESSEL;
      else if (strstr(v, "class") || strstr(v, "smart")) los->k3_sampling = SONG2_K3_SAMPLING_CLASS;
      else {
        snprintf(err, SONG2_ERRLEN, "transfer2_k3_sampling = %.200s (bessel, smart or class)", v);
        return 1;
      }
    }
    RD_D2("k_step_trans_scalars_2nd_order", "q_linstep_song", los->q_linstep);
    if (get(pl, "k_step_trans_scalars_2nd_order") && !get(pl, "q_linstep_song")) los->q_linstep *= 95; /* :1489-1503 */
    if ((v = get(pl, "transfer2_tau_sampling"))) {
      if (strstr(v, "sources") || strstr(v, "source")) los->tau_sampling = SONG2_TAU_SAMPLING_SOURCES;
      else if (strstr(v, "custom") || strstr(v, "smart")) los->tau_sampling = SONG2_TAU_SAMPLING_CUSTOM;
      else if (strstr(v, "bessel")) los->tau_sampling = SONG2_TAU_SAMPLING_BESSEL;
      else {
        snprintf(err, SONG2_ERRLEN, "transfer2_tau_sampling = %.200s (sources, custom or bessel)", v);
        return 1;
      }
    }
    {
      const char *a = get(pl, "tau_step_trans_2nd_order"), *b = get(pl, "tau_step_trans_song"),
                 *c = get(pl, "tau_linstep_song");
      double d;
      if (c) {
        if (num(c, "tau_linstep_song", &d, err)) return 1;
        los->tau_linstep = d;
      } else if (b || a) {
        if (num(b ? b : a, "tau_step_trans_song", &d, err)) return 1;
        los->tau_linstep = d / (2 * 3.141592653589793);
      }
      if (los->tau_linstep < 0) los->tau_linstep = 1e300; /* no points added (:1542-1543) */
    }
    if ((v = get(pl, "sources_time_interpolation")))
      los->time_interpolation = (strstr(v, "cubic") || strstr(v, "spline")) ? SONG2_INTERP_CUBIC : SONG2_INTERP_LINEAR;
    if ((v = get(pl, "sources_k3_interpolation")))
      los->k3_interpolation = (strstr(v, "cubic") || strstr(v, "spline")) ? SONG2_INTERP_CUBIC : SONG2_INTERP_LINEAR;
    if ((v = get(pl, "bessels_interpolation")))
      los->bessel_interpolation = strstr(v, "cubic") ? SONG2_INTERP_CUBIC : SONG2_INTERP_LINEAR;
    if ((v = get(pl, "bispectra_k3_extrapolation")))
      los->k3_extrapolation = strstr(v, "flat") ? SONG2_K3_EXTRAP_FLAT : SONG2_K3_EXTRAP_NONE;
    RD_D("extra_k3_oscillations_left", los->extra_k3_oscillations_left);
    RD_D("extra_k3_oscillations_right", los->extra_k3_oscillations_right);
    RD_D2("bessel_x_step_2nd_order", "bessel_x_step_song", los->x_step);
    RD_D2("bessel_j_cut_2nd_order", "bessel_j_cut_song", los->j_cut);
    RD_D2("bessel_J_cut_2nd_order", "bessel_J_cut_song", los->J_cut);
    /* pbs2->xx_max for the lin/log k samplings (input2.c:1982-2006) */
    los->x_max = (g->k_max * 18000.0 + los->x_step) * 1.05;
  }
  return 0;
}

/* ----------------------------------------------------------- smart grids */

static double bgc(const song2_tables *t, int col, double x) {
  double u = (x - t->bg_lntau0) / t->bg_dlntau;
  int i = (int)floor(u);
  if (i < 0) i = 0;
  if (i > t->bg_size - 2) i = t->bg_size - 2;
  double b = u - i, a = 1.0 - b, h = t->bg_dlntau;
  const double *y0 = t->bg + (size_t)i * SONG2_BG_SIZE, *y1 = y0 + SONG2_BG_SIZE;
  const double *d0 = t->bg_dd + (size_t)i * SONG2_BG_SIZE, *d1 = d0 + SONG2_BG_SIZE;
  return a * y0[col] + b * y1[col] + ((a * a * a - a) * d0[col] + (b * b * b - b) * d1[col]) * h * h / 6.0;
}

static double sound_speed(const song2_tables *t, double x) {
  double R = 0.75 * exp(bgc(t, SONG2_BG_LN_RHO_B, x) - bgc(t, SONG2_BG_LN_RHO_G, x));
  return 1.0 / sqrt(3.0 * (1.0 + R));
}

double song2_sound_horizon(const song2_tables *t, double tau) {
  /* before the table: radiation domination with R -> 0, c_s -> 1/sqrt(3) */
  double x0 = t->bg_lntau0, x1 = log(tau);
  double rs = exp(x0) * sound_speed(t, x0);
  if (x1 <= x0) return tau * sound_speed(t, x0);
  /* Simpson's rule in ln tau (dtau = tau dln tau) on the table's spacing, halved */
  int n = 2 * (int)ceil((x1 - x0) / t->bg_dlntau);
  if (n < 2) n = 2;
  double h = (x1 - x0) / n, sum = 0.0;
  for (int i = 0; i <= n; ++i) {
    double x = x0 + i * h;
    double f = exp(x) * sound_speed(t, x);
    sum += f * ((i == 0 || i == n) ? 1.0 : (i % 2 ? 4.0 : 2.0));
  }
  return rs + sum * h / 3.0;
}

#define S2_PI 3.141592653589793238462643383279502884
#define S2_K_SIZE_CAP 1000000

int song2_k_grid_smart(const song2_params *g, double tau0, double rs_rec, int l_scalar_max, double *k_out,
                       char *err) {
  if (g->k_step_transition == 0 || rs_rec == 0 || tau0 <= 0) {
    snprintf(err, SONG2_ERRLEN, "smart k sampling: k_step_transition, rs_rec and tau0 must be non-zero");
    return -1;
  }
  double k_min = g->k_min_tau0 / tau0;
  int n = 0;
  double prev = k_min, k = k_min;
  if (k_out) k_out[n] = k_min;
  ++n;
  double k_rec = 2 * S2_PI / rs_rec;
  double k_max_cmb = 0, k_max_lss = 0;
  if (g->has_cmb) {
    k_max_cmb = g->k_max_tau0_over_l_max * l_scalar_max / tau0;
    while (k < k_max_cmb) {
      double lin_step = g->k_step_super +
                        0.5 * (tanh((prev - k_rec) / k_rec / g->k_step_transition) + 1) * (g->k_step_sub - g->k_step_super);
      double log_step = prev * (g->k_logstep_super - 1.);
      double st = lin_step * k_rec < log_step ? lin_step * k_rec : log_step;
      if (st / k < 1e-16) {
        snprintf(err, SONG2_ERRLEN, "k step = %e < machine precision", st);
        return -1;
      }
      if ((log_step > (lin_step * k_rec)) || (prev > k_rec)) k = prev + lin_step * k_rec;
      else k = prev * g->k_logstep_super;
      if (k_out) k_out[n] = k;
      ++n;
      prev = k;
      if (n + 1 > S2_K_SIZE_CAP) {
        snprintf(err, SONG2_ERRLEN, "k size for CMB is too large; check k_step_sub, k_step_super and k_logstep_super");
        return -1;
      }
    }
  }
  if (g->has_lss) {
    k_max_lss = g->k_max_for_pk;
    while (k < k_max_lss) {
      k *= pow(10, 1 / (g->k_per_decade_for_pk +
                        (g->k_per_decade_for_bao - g->k_per_decade_for_pk) *
                            (1 - tanh(pow((log(k) - log(g->k_bao_center * k_rec)) / log(g->k_bao_width), 4)))));
      if (k_out) k_out[n] = k;
      ++n;
      if (n + 1 > S2_K_SIZE_CAP) {
        snprintf(err, SONG2_ERRLEN, "k size for LSS is too large; check k_per_decade_for_pk and k_per_decade_for_bao");
        return -1;
      }
    }
  }
  if (k_out) k_out[n - 1] = k_max_cmb > k_max_lss ? k_max_cmb : k_max_lss;
  return n;
}

static int cmp_d(const void *a, const void *b) {
  double x = *(const double *)a, y = *(const double *)b;
  return (x > y) - (x < y);
}

/* merge_arrays_double: the union of two arrays, sorted, exact duplicates removed */
static int merge_sorted(double *buf, int n) {
  qsort(buf, n, sizeof(double), cmp_d);
  int m = 0;
  for (int i = 0; i < n; ++i)
    if (m == 0 || buf[i] != buf[m - 1]) buf[m++] = buf[i];
  return m;
}

int song2_k3_grids_smart(const double *k, int k_size, int k3_size_min, int *k3_size_out, double *k3_out,
                         char *err) {
  int64_t off = 0;
  for (int i1 = 0; i1 < k_size; ++i1)
    for (int i2 = 0; i2 < k_size; ++i2) k3_size_out[i1 * k_size + i2] = 0;
  int cap = k_size + 2 + (k3_size_min > 0 ? k3_size_min + 2 : 0);
  double *buf = (double *)malloc(sizeof(double) * cap);
  if (!buf) {
    snprintf(err, SONG2_ERRLEN, "out of memory");
    return 1;
  }
  for (int i1 = 0; i1 < k_size; ++i1)
    for (int i2 = 0; i2 <= i1; ++i2) {
      double k1 = k[i1], k2 = k[i2];
      double k3_min = fabs(k1 - k2) + 1e-10, k3_max = k1 + k2 - 1e-10;
      if ((k1 + k2) / 100 > k3_min) k3_min = (k1 + k2) / 100;
      if (k[0] > k3_min) k3_min = k[0];
      if (k[k_size - 1] < k3_max) k3_max = k[k_size - 1];
      if (k3_min >= k3_max || k3_min < k[0] || k3_min > k[k_size - 1] || k3_max < k[0] || k3_max > k[k_size - 1]) {
        snprintf(err, SONG2_ERRLEN, "found k3_min=%g, k3_max=%g for k1(%d)=%g and k2(%d)=%g", k3_min, k3_max, i1, k1,
                 i2, k2);
        free(buf);
        return 1;
      }
      int lo = 0;
      while (k[lo] < k3_min) ++lo;
      int hi = k_size - 1;
      while (k[hi] > k3_max) --hi;
      int n = hi - lo + 1;
      if (n < 0) n = 0;
      for (int j = 0; j < n; ++j) buf[j] = k[lo + j];
      buf[n] = k3_min;
      buf[n + 1] = k3_max;
      n = merge_sorted(buf, n + 2);
      if (n < k3_size_min) {
        int extra = k3_size_min - n + 2;
        for (int j = 0; j < extra; ++j) buf[n + j] = k3_min + j * (k3_max - k3_min) / (extra - 1);
        n = merge_sorted(buf, n + extra);
      }
      k3_size_out[i1 * k_size + i2] = n;
      if (k3_out) memcpy(k3_out + off, buf, sizeof(double) * n);
      off += n;
    }
  free(buf);
  return 0;
}

/* ---------------------------------------------------- source time grid */

/* value and first two x-derivatives of a column's spline at x = ln tau */
static void bg_d2(const song2_tables *t, int col, double x, double *v, double *d1, double *d2) {
  double u = (x - t->bg_lntau0) / t->bg_dlntau;
  int i = (int)floor(u);
  if (i < 0) i = 0;
  if (i > t->bg_size - 2) i = t->bg_size - 2;
  double h = t->bg_dlntau, b = u - i, a = 1.0 - b;
  const double *y0 = t->bg + (size_t)i * SONG2_BG_SIZE, *y1 = y0 + SONG2_BG_SIZE;
  const double *q0 = t->bg_dd + (size_t)i * SONG2_BG_SIZE, *q1 = q0 + SONG2_BG_SIZE;
  *v = a * y0[col] + b * y1[col] + ((a * a * a - a) * q0[col] + (b * b * b - b) * q1[col]) * h * h / 6.0;
  *d1 = (y1[col] - y0[col]) / h - (3 * a * a - 1) / 6.0 * h * q0[col] + (3 * b * b - 1) / 6.0 * h * q1[col];
  *d2 = a * q0[col] + b * q1[col];
}

/* kappa', CLASS's variation rate of the thermodynamics
   sqrt(kappa1^2 + (kappa2 / kappa1)^2 + |kappa3 / kappa1|) with kappa1..3 the first
   three conformal-time derivatives of the optical depth, from the spline of
   s = ln kappa1 in x = ln tau; the conformal Hubble rate aH and a''/a */
static void thermo_rates(const song2_tables *t, double tau, double *kd, double *rate, double *hc, double *app_a) {
  double x = log(tau), s, sx, sxx;
  bg_d2(t, SONG2_BG_LN_KAPPA_DOT, x, &s, &sx, &sxx);
  /* d/dtau = (1/tau) d/dx: ds/dtau = sx / tau, d2s/dtau2 = (sxx - sx) / tau^2 */
  double s1 = sx / tau, s2 = (sxx - sx) / (tau * tau);
  double k1 = exp(s);
  double k2 = k1 * s1;
  double k3 = k1 * (s2 + s1 * s1);
  *kd = k1;
  *rate = sqrt(k1 * k1 + (k2 / k1) * (k2 / k1) + fabs(k3 / k1));
  double lh, lhx, lhxx;
  bg_d2(t, SONG2_BG_LN_HC, x, &lh, &lhx, &lhxx);
  double H = exp(lh);        /* aH */
  double Hp = H * lhx / tau; /* (aH)' */
  *hc = H;
  *app_a = Hp + H * H;       /* a''/a = (aH)' + (aH)^2 */
}

int song2_tau_grid_class(const song2_tables *t, double stepsize, double late_boost, double start_tau_c_over_tau_h,
                         double tol_tau, int has_cmb, double *out, char *err) {
  double tau_rec = song2_recombination_time(t);
  double tau_ini;
  if (has_cmb) {
    /* the thermodynamics table's start: z = 1e4 (CLASS recfast_z_initial) */
    double lo = t->bg_lntau0, hi = log(tau_rec), target = -log(1e4 + 1.0);
    for (int it = 0; it < 200 && hi - lo > 1e-14; ++it) {
      double mid = 0.5 * (lo + hi), v, d1, d2;
      bg_d2(t, SONG2_BG_LN_A, mid, &v, &d1, &d2);
      if (v < target) lo = mid;
      else hi = mid;
    }
    double tau_lower = exp(0.5 * (lo + hi)), tau_upper = tau_rec, kd, rate, hc, app;
    thermo_rates(t, tau_lower, &kd, &rate, &hc, &app);
    if (hc / kd > start_tau_c_over_tau_h) {
      snprintf(err, SONG2_ERRLEN, "start of the source sampling before the thermodynamics table (tau=%g)", tau_lower);
      return -1;
    }
    thermo_rates(t, tau_upper, &kd, &rate, &hc, &app);
    if (hc / kd < start_tau_c_over_tau_h) {
      snprintf(err, SONG2_ERRLEN,
               "start of the source sampling after recombination; decrease start_sources_at_tau_c_over_tau_h");
      return -1;
    }
    double tau_mid = 0.5 * (tau_lower + tau_upper);
    for (int it = 0; it < 400 && tau_upper - tau_lower > tol_tau; ++it) {
      thermo_rates(t, tau_mid, &kd, &rate, &hc, &app);
      if (hc / kd > start_tau_c_over_tau_h) tau_upper = tau_mid;
      else tau_lower = tau_mid;
      tau_mid = 0.5 * (tau_lower + tau_upper);
    }
    tau_ini = tau_mid;
  } else {
    tau_ini = tau_rec;
  }
  int n = 0;
  double tau = tau_ini;
  if (out) out[n] = tau;
  ++n;
  while (tau < t->tau0) {
    double kd, rate, hc, app, timescale;
    thermo_rates(t, tau, &kd, &rate, &hc, &app);
    if (has_cmb) {
      double isw2 = fabs(2 * app - hc * hc) * late_boost * late_boost;
      timescale = 1 / sqrt(rate * rate + isw2);
    } else {
      timescale = 1 / hc;
    }
    double step = stepsize * timescale;
    if (fabs(step / tau) < 10 * DBL_EPSILON) { /* CLASS's smallest_allowed_variation */
      snprintf(err, SONG2_ERRLEN, "integration step = %e < machine precision", step);
      return -1;
    }
    tau += step;
    if (out) out[n] = tau;
    ++n;
    if (n + 1 > 1000000) {
      snprintf(err, SONG2_ERRLEN, "source time sampling too large; check perturb_sampling_stepsize_song");
      return -1;
    }
  }
  if (out) out[n - 1] = t->tau0;
  return n;
}

/* ------------------------------------------------- theta_12 k3 sampling */

int song2_k3_grids_theta12(const double *k, int k_size, int k3_size, int *k3_size_out, double *k3_out, char *err) {
  if (k3_size < 2) {
    snprintf(err, SONG2_ERRLEN, "theta_12 sampling needs k3_size >= 2, got %d", k3_size);
    return 1;
  }
  int64_t off = 0;
  for (int i = 0; i < k_size * k_size; ++i) k3_size_out[i] = 0;
  for (int i1 = 0; i1 < k_size; ++i1)
    for (int i2 = 0; i2 <= i1; ++i2) {
      double k1 = k[i1], k2 = k[i2];
      /* the limits of the lin/log samplings (perturbations2.c:1973-1984) */
      double k3_min = fabs(k1 - k2) + 1e-10, k3_max = k1 + k2 - 1e-10;
      if ((k1 + k2) / 100 > k3_min) k3_min = (k1 + k2) / 100;
      if (k[0] > k3_min) k3_min = k[0];
      if (k[k_size - 1] < k3_max) k3_max = k[k_size - 1];
      if (k3_min >= k3_max) {
        snprintf(err, SONG2_ERRLEN, "found k3_min=%g>k3_max=%g for k1(%d)=%g and k2(%d)=%g", k3_min, k3_max, i1, k1,
                 i2, k2);
        return 1;
      }
      double cmin = (k3_min * k3_min - k1 * k1 - k2 * k2) / (2 * k1 * k2);
      double cmax = (k3_max * k3_max - k1 * k1 - k2 * k2) / (2 * k1 * k2);
      if (fabs(cmin) > 1 || fabs(cmax) > 1) {
        snprintf(err, SONG2_ERRLEN, "cos(theta_12) out of [-1, 1] for k1(%d)=%g and k2(%d)=%g", i1, k1, i2, k2);
        return 1;
      }
      /* linear in the angle between k1 and k2 (perturbations2.c:2029-2060) */
      double th_min = acos(cmin), th_max = acos(cmax);
      double step = (th_max - th_min) / (k3_size - 1);
      if (i1 == i2) {
        th_min += step / 5;
        step = (th_max - th_min) / (k3_size - 1);
      }
      k3_size_out[i1 * k_size + i2] = k3_size;
      if (k3_out)
        for (int i3 = 0; i3 < k3_size; ++i3) {
          double c = cos(th_min + i3 * step);
          k3_out[off + i3] = sqrt(k1 * k1 + k2 * k2 + 2 * c * k1 * k2);
        }
      off += k3_size;
    }
  return 0;
}

/* ------------------------------------------------- cosmology keys */

int song2_read_cosmo(const char *ini_path, const char *pre_path, song2_cosmo *c, char *err) {
  static plist list; /* large; the reader is not reentrant */
  plist *pl = &list;
  pl->n = 0;
  if (read_file(ini_path, "ini", pl, err) || read_file(pre_path, "pre", pl, err)) return 1;
  /* the benchmark cosmology where a key is absent */
  c->h = 0.678;
  c->omega_b = 0.0224;
  c->omega_cdm = 0.120;
  c->N_eff = 3.046;
  c->T_cmb = 2.7255;
  c->YHe = 0.24;
  c->z_reio = 0.0;
  const char *v;
  const char *h = get(pl, "h"), *H0 = get(pl, "H0");
  if (h && H0) {
    snprintf(err, SONG2_ERRLEN, "give one of h and H0");
    return 1;
  }
  if (h && num(h, "h", &c->h, err)) return 1;
  if (H0) {
    double d;
    if (num(H0, "H0", &d, err)) return 1;
    c->h = d / 100.0;
  }
  if (get(pl, "100*theta_s")) {
    snprintf(err, SONG2_ERRLEN, "100*theta_s is not supported: give h or H0");
    return 1;
  }
  RD_D("T_cmb", c->T_cmb);
  /* physical or relative densities */
  {
    const char *ob = get(pl, "omega_b"), *Ob = get(pl, "Omega_b");
    const char *oc = get(pl, "omega_cdm"), *Oc = get(pl, "Omega_cdm");
    if ((ob && Ob) || (oc && Oc)) {
      snprintf(err, SONG2_ERRLEN, "give one of omega_b and Omega_b (omega_cdm and Omega_cdm)");
      return 1;
    }
    double d;
    if (ob && num(ob, "omega_b", &c->omega_b, err)) return 1;
    if (Ob) {
      if (num(Ob, "Omega_b", &d, err)) return 1;
      c->omega_b = d * c->h * c->h;
    }
    if (oc && num(oc, "omega_cdm", &c->omega_cdm, err)) return 1;
    if (Oc) {
      if (num(Oc, "Omega_cdm", &d, err)) return 1;
      c->omega_cdm = d * c->h * c->h;
    }
  }
  {
    const char *n1 = get(pl, "N_ur"), *n2 = get(pl, "N_eff");
    if (n1 && n2) {
      snprintf(err, SONG2_ERRLEN, "give one of N_ur and N_eff");
      return 1;
    }
    const char *w = n1 ? n1 : n2;
    if (w && num(w, n1 ? "N_ur" : "N_eff", &c->N_eff, err)) return 1;
  }
  if ((v = get(pl, "N_ncdm"))) {
    double d;
    if (num(v, "N_ncdm", &d, err)) return 1;
    if (d != 0) {
      snprintf(err, SONG2_ERRLEN, "massive neutrinos (N_ncdm = %g) are not supported", d);
      return 1;
    }
  }
  if ((v = get(pl, "Omega_k"))) {
    double d;
    if (num(v, "Omega_k", &d, err)) return 1;
    if (d != 0) {
      snprintf(err, SONG2_ERRLEN, "curvature (Omega_k = %g) is not supported: the background is flat", d);
      return 1;
    }
  }
  if ((v = get(pl, "YHe"))) {
    if (strstr(v, "BBN") || strstr(v, "bbn")) {
      snprintf(err, SONG2_ERRLEN, "YHe = BBN needs CLASS's BBN table: give a number");
      return 1;
    }
    if (num(v, "YHe", &c->YHe, err)) return 1;
  }
  /* reionisation: none, or the tanh model at a given z_reio */
  {
    const char *p = get(pl, "reio_parametrization");
    int camb = 0;
    if (p) {
      if (strstr(p, "reio_none")) camb = 0;
      else if (strstr(p, "reio_camb")) camb = 1;
      else {
        snprintf(err, SONG2_ERRLEN, "reio_parametrization = %.200s (reio_none or reio_camb)", p);
        return 1;
      }
    }
    if (get(pl, "tau_reio")) {
      snprintf(err, SONG2_ERRLEN, "tau_reio is not supported: give z_reio");
      return 1;
    }
    const char *zr = get(pl, "z_reio");
    if (camb && !zr) {
      snprintf(err, SONG2_ERRLEN, "reio_camb needs z_reio");
      return 1;
    }
    if (camb && num(zr, "z_reio", &c->z_reio, err)) return 1;
  }
  if (!(c->h > 0) || !(c->omega_b > 0) || !(c->omega_cdm >= 0) || !(c->T_cmb > 0) || !(c->YHe >= 0 && c->YHe < 1) ||
      !(c->N_eff >= 0) || !(c->z_reio >= 0)) {
    snprintf(err, SONG2_ERRLEN, "cosmological parameters out of range");
    return 1;
  }
  return 0;
}
