/*
 * song2_capi.cu - host side of the C ABI declared in include/song2.h.
 *
 * Builds the device layout of a run (state vector grouped by azimuthal m,
 * quadratic-source vector, source types, coupling tables), uploads it once
 * with cudaMemcpyAsync into a device arena owned by a song2_ctx, launches the
 * persistent evolver and copies the sources back.
 */
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "song2_internal.h"

struct song2_ctx {
  DevSpec spec;
  DevPtrs ptrs;
  int precision;
  int block, grid;
  size_t smem;
  std::vector<void *> allocs;
  double *d_sources;
  size_t sources_len;
  song2_triplet_stats *d_stats;
  double *d_fo_out;
  size_t fo_out_len;
  int *d_queue;
  int n_items;
  int tp2_size;
  int64_t per_type;
  cudaEvent_t ev0, ev1;
  float last_ms;
  int last_launches;
  song2_launch launch;
  int kmode;    /* kernel of single-group runs (song2_launch_evolver's mode) */
  int n_teams;
  /* uneven batches: consecutive item ranges launched one after the other, the
     classes with large shared-memory plans first, so that the small ones run
     several CTAs per SM */
  struct Group {
    int first, count, grid;
    size_t smem;
    int mode;   /* kernel of the group (song2_launch_evolver's mode) */
  };
  std::vector<Group> groups;
  /* host copy of the device work list (launch-group order) and, after
     song2_ctx_run_part, its split into parts: part q of group g is the range
     part_first[g * parts + q], part_count[...] */
  std::vector<WorkItem> h_items;
  int parts = 0;
  std::vector<int> part_first, part_count;
  /* song2_ctx_run_graph: the run's memsets and launches captured once */
  cudaStream_t cap_stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
};

namespace {

#define CK(x)                                                                        \
  do {                                                                               \
    cudaError_t e_ = (x);                                                            \
    if (e_ != cudaSuccess) {                                                         \
      snprintf(err, SONG2_ERRLEN, "%s failed: %s", #x, cudaGetErrorString(e_));      \
      return 1;                                                                      \
    }                                                                                \
  } while (0)

int size_l_indexm(int l_max, const int *m, int m_size) {
  int n = 0;
  for (int l = 0; l <= l_max; ++l)
    for (int i = 0; i < m_size; ++i)
      if (m[i] <= l) ++n;
  return n;
}

struct HostLayout {
  DevSpec s;
  std::vector<short> eq_sp, eq_l, eq_m, idx_I, idx_E, idx_B, idx_N, qs_sp, qs_l, qs_m, row_slot, qs_slot, qo_slot, mx_idx,
      mx_pos;
  std::vector<double> cmin, cplu, dmin, dplu, dzer;
  std::vector<GenRow> gen;
};

/* Build everything that depends only on the spec. */
int build_layout(const song2_spec *sp, const song2_tables *tab, int first_order_mode, HostLayout &H, char *err) {
  DevSpec &s = H.s;
  memset(&s, 0, sizeof(s));
  s.l_max_g = sp->l_max_g;
  s.l_max_pol = sp->has_polarization2 ? sp->l_max_pol_g : -1;
  s.l_max_ur = sp->l_max_ur;
  s.l_los_t = sp->l_max_los_t;
  s.l_los_p = sp->l_max_los_p;
  s.m_size = sp->m_size;
  if (sp->m_size < 1 || sp->m_size > SONG2_MAX_M) { snprintf(err, SONG2_ERRLEN, "bad m_size"); return 1; }
  for (int i = 0; i < SONG2_MAX_M; ++i) s.index_m[i] = -1;
  int m_max = 0;
  for (int i = 0; i < sp->m_size; ++i) {
    int m = sp->m[i];
    if (m < 0 || m >= SONG2_MAX_M || (i > 0 && m <= sp->m[i - 1])) {
      snprintf(err, SONG2_ERRLEN, "modes must be ascending in 0..%d", SONG2_MAX_M - 1);
      return 1;
    }
    s.m[i] = m; s.compute_m[m] = 1; s.index_m[m] = i;
    m_max = std::max(m_max, m);
  }
  if (sp->l_max_g < 2 || sp->l_max_ur < 2 || (sp->has_polarization2 && sp->l_max_pol_g < 2)) {
    snprintf(err, SONG2_ERRLEN, "l_max_* must be at least 2");
    return 1;
  }
  /* the E/B closure of the reference (perturbations2.c:8033-8036) needs
     1 - m^2/l^2 (l+2)/(l-2) >= 0 at l = l_max_pol for every evolved m */
  if (sp->has_polarization2)
    for (int i = 0; i < sp->m_size; ++i) {
      double l = sp->l_max_pol_g, m = sp->m[i];
      if (l <= 2 || 1 - m * m / (l * l) * (l + 2) / (l - 2) < 0) {
        snprintf(err, SONG2_ERRLEN, "l_max_pol_g = %d is too small for m = %d (polarisation closure)",
                 sp->l_max_pol_g, sp->m[i]);
        return 1;
      }
    }
  int L = std::max(sp->l_max_g, sp->l_max_ur);
  if (sp->has_polarization2) L = std::max(L, sp->l_max_pol_g);
  L = std::max(L, std::max(sp->l_max_los_t, sp->l_max_los_p));
  if (L + 2 >= S2_LMAXP) { snprintf(err, SONG2_ERRLEN, "l_max too large (max %d)", SONG2_MAX_L); return 1; }
  s.L_big = L;
  s.Lq = L + 1;
  s.mq_max = std::min(m_max + 1, s.Lq);
  /* delta-tilde sources (perturb2_get_lm_lists, perturbations2.c:1285-1300; the
     flag check of input2.c:742-744): the couplings reach |m1|, |m2| <= the
     quadratic cut, so the rotation coefficients are needed up to that m */
  if (sp->use_delta_tilde_in_los && !first_order_mode) {
    if (sp->has_redshift_in_los) {
      snprintf(err, SONG2_ERRLEN, "use_delta_tilde_in_los excludes has_redshift_in_los");
      return 1;
    }
    int qt = sp->l_max_los_quadratic_t, qp = sp->l_max_los_quadratic_p;
    int Q = std::max(qt, qp);
    if (qt < 0 || qp < 0 || Q > L || Q > SONG2_MAX_M + 1) {
      snprintf(err, SONG2_ERRLEN, "l_max_los_quadratic_t/p must lie in 0..min(%d, l_max)", SONG2_MAX_M + 1);
      return 1;
    }
    s.dtilde = sp->has_quadratic_sources ? 1 : 0;
    s.dt_qt = qt; s.dt_qp = qp; s.dt_Q = Q;
    s.dt_L = std::max(sp->l_max_los_t, sp->l_max_los_p);
    s.mq_max = std::max(s.mq_max, Q);
  }
  s.rescale = sp->rescale_cmb_sources && !first_order_mode;
  /* radiation-streaming approximation (perturbations2.c:5309-5321) */
  if (sp->radiation_streaming_approximation != SONG2_RSA_NONE && !first_order_mode) {
    if (sp->radiation_streaming_approximation != SONG2_RSA_MD &&
        sp->radiation_streaming_approximation != SONG2_RSA_MD_WITH_REIO) {
      snprintf(err, SONG2_ERRLEN, "radiation_streaming_approximation %d: none (0), MD (1) or MD_with_reio (2)",
               sp->radiation_streaming_approximation);
      return 1;
    }
    if (!(tab && tab->tau_free_streaming > 0) || !(sp->radiation_streaming_trigger_tau_over_tau_k > 0)) {
      snprintf(err, SONG2_ERRLEN, "the RSA needs tables.tau_free_streaming > 0 and a positive k tau trigger");
      return 1;
    }
    s.rsa = sp->radiation_streaming_approximation;
    s.rsa_k = sp->radiation_streaming_trigger_tau_over_tau_k;
    s.tau_fs = tab->tau_free_streaming;
  }
  /* closure coefficients at l_max (the same expressions as the closure rows of
     perturb2_derivs, evaluated once per hierarchy class instead of per right-hand side) */
  for (int mm = 0; mm < SONG2_MAX_M; ++mm) {
    auto c_in = [&](int l) {
      return l <= mm ? 0.0 : (mm == 0 ? (2.0 * l + 1) / (2.0 * l - 1) : sqrt((double)(l + mm) / (l - mm)) * (2.0 * l + 1) / (2.0 * l - 1));
    };
    s.cl_I[mm] = c_in(s.l_max_g);
    s.cl_N[mm] = c_in(s.l_max_ur);
    int lp = s.l_max_pol;
    s.cl_P[mm] = lp > 2 ? sqrt(std::max(0.0, 1 - ((double)mm * mm) / ((double)lp * lp) * (lp + 2) / (lp - 2.0))) *
                              (2.0 * lp + 1) / (2.0 * lp - 1)
                        : 0.0;
    s.cmix_P[mm] = lp > 0 ? (double)mm / lp : 0.0;
  }
  for (int l = 0; l < S2_LMAXP; ++l) {
    s.index_m_max[l] = -1;
    for (int i = 0; i < s.m_size; ++i)
      if (s.m[i] <= l) s.index_m_max[l] = i;
  }
  int n = 0;
  for (int l = 0; l < S2_LMAXP; ++l)
    for (int i = 0; i < SONG2_MAX_M; ++i) s.lm_array[l][i] = -1;
  for (int l = 0; l <= s.Lq; ++l)
    for (int i = 0; i < s.m_size; ++i)
      if (s.m[i] <= l) s.lm_array[l][i] = (short)n++;
  s.n_lm = n;
  n = 0;
  for (int l = 0; l < S2_LMAXP; ++l)
    for (int m = 0; m < SONG2_MAX_M + 2; ++m) s.lmq[l][m] = -1;
  for (int l = 0; l <= s.Lq; ++l)
    for (int m = 0; m <= std::min(l, s.mq_max); ++m) s.lmq[l][m] = (short)n++;
  s.n_lmq = n;
  s.has_pol = sp->has_polarization2;
  s.has_qs = sp->has_quadratic_sources && !first_order_mode;
  s.has_liou = sp->has_quadratic_liouville;
  s.has_coll = sp->has_quadratic_collision;
  s.tca_on = sp->tight_coupling;
  s.tca_h = sp->tca_trigger_tau_c_over_tau_h;
  s.tca_k = sp->tca_trigger_tau_c_over_tau_k;
  s.ic = sp->ic;
  s.fnl = sp->primordial_local_fnl_phi;
  s.los_pure_scat = sp->has_pure_scattering_in_los;
  s.los_quad_scat = sp->has_quad_scattering_in_los;
  s.los_pure_metric = sp->has_pure_metric_in_los;
  s.los_quad_metric = sp->has_quad_metric_in_los;
  s.los_time_delay = sp->has_time_delay_in_los;
  s.los_redshift = sp->has_redshift_in_los;
  s.los_lensing = sp->has_lensing_in_los;
  s.los_sw = sp->has_sw;
  s.los_isw = sp->has_isw;
  s.los_exp_pot = sp->use_exponential_potentials;
  s.rtol = sp->rtol;
  s.threshold = sp->threshold;
  if (!(sp->threshold >= 1e-30 && sp->threshold <= 1e30) || !(sp->rtol > 0)) {
    snprintf(err, SONG2_ERRLEN, "rtol must be positive and threshold in [1e-30, 1e30]");
    return 1;
  }
  s.max_steps = sp->max_steps;
  s.start_h = sp->start_small_k_at_tau_c_over_tau_h;
  s.start_k = sp->start_large_k_at_tau_h_over_tau_k;
  s.tol_tau = sp->tol_tau_approx;
  auto LM = [&](int l, int m) { return (int)s.lm_array[l][s.index_m[m]]; };

  /* quadratic-source layout (same order as perturb2_workspace_init) */
  int q = 0;
  H.qs_sp.clear(); H.qs_l.clear(); H.qs_m.clear();
  auto push_q = [&](int sp_, int l, int m) { H.qs_sp.push_back((short)sp_); H.qs_l.push_back((short)l); H.qs_m.push_back((short)m); ++q; };
  auto push_hier = [&](int sp_, int lmax) {
    for (int l = 0; l <= lmax; ++l)
      for (int i = 0; i < s.m_size; ++i)
        if (s.m[i] <= l) push_q(sp_, l, s.m[i]);
  };
  s.iq_g = q; push_hier(SP_I, s.l_max_g);
  s.iq_E = q; if (s.has_pol) push_hier(SP_E, s.l_max_pol);
  s.iq_B = q; if (s.has_pol) push_hier(SP_B, s.l_max_pol);
  s.iq_ur = q; push_hier(SP_N, s.l_max_ur);
  s.iq_b = q;
  s.iq_b000 = s.iq_c000 = -1;
  s.iq_b11[0] = s.iq_b11[1] = s.iq_c11[0] = s.iq_c11[1] = -1;
  if (s.compute_m[0]) { s.iq_b000 = (short)q; push_q(SP_B000, 0, 0); }
  for (int i = 0; i < s.m_size; ++i) if (s.m[i] <= 1) { s.iq_b11[s.m[i]] = (short)q; push_q(SP_B11, 1, s.m[i]); }
  s.iq_cdm = q;
  if (s.compute_m[0]) { s.iq_c000 = (short)q; push_q(SP_C000, 0, 0); }
  for (int i = 0; i < s.m_size; ++i) if (s.m[i] <= 1) { s.iq_c11[s.m[i]] = (short)q; push_q(SP_C11, 1, s.m[i]); }
  s.iq_psi = q; push_q(SP_METRIC, 0, 0);
  s.iq_psi_prime = q; push_q(SP_METRIC, 0, 0);
  s.iq_phi_prime_poisson = q; push_q(SP_METRIC, 0, 0);
  s.iq_phi_prime_longitudinal = q; push_q(SP_METRIC, 0, 0);
  s.iq_phi_prime_prime = q; push_q(SP_METRIC, 0, 0);
  s.iq_omega_m1_prime = q; push_q(SP_METRIC, 0, 0);
  s.iq_gamma_m2_prime_prime = q; push_q(SP_METRIC, 0, 0);
  s.iq_vv_g = q; push_q(SP_METRIC, 0, 0);
  s.iq_vv_ur = q; push_q(SP_METRIC, 0, 0);
  s.iq_dd_b = q; push_q(SP_METRIC, 0, 0);
  s.iq_vv_b = q; push_q(SP_METRIC, 0, 0);
  s.iq_vv_cdm = q; push_q(SP_METRIC, 0, 0);
  s.iq_vvp_b = q; push_q(SP_METRIC, 0, 0);
  s.iq_vvp_cdm = q; push_q(SP_METRIC, 0, 0);
  s.qs2_size = q;

  /* state vector, grouped in m blocks */
  H.eq_sp.clear(); H.eq_l.clear(); H.eq_m.clear();
  H.idx_I.assign(s.n_lm, -1); H.idx_E.assign(s.n_lm, -1); H.idx_B.assign(s.n_lm, -1); H.idx_N.assign(s.n_lm, -1);
  int ni = 0;
  auto push_e = [&](int sp_, int l, int m) { H.eq_sp.push_back((short)sp_); H.eq_l.push_back((short)l); H.eq_m.push_back((short)m); return ni++; };
  s.idx_phi = s.idx_phip = s.idx_omega = s.idx_gamma = s.idx_gammap = s.idx_b000 = s.idx_c000 = -1;
  s.idx_b11[0] = s.idx_b11[1] = s.idx_c11[0] = s.idx_c11[1] = -1;
  s.nblk = s.m_size;
  for (int b = 0; b < s.m_size; ++b) {
    int m = s.m[b];
    s.blk_start[b] = ni;
    if (m == 0) {
      s.idx_phi = push_e(SP_PHI, 0, 0);
      s.idx_phip = push_e(SP_PHIP, 0, 0);
      s.idx_b000 = push_e(SP_B000, 0, 0);
      s.idx_b11[0] = push_e(SP_B11, 1, 0);
      s.idx_c000 = push_e(SP_C000, 0, 0);
      s.idx_c11[0] = push_e(SP_C11, 1, 0);
    } else if (m == 1) {
      s.idx_omega = push_e(SP_OMEGA, 0, 1);
      s.idx_b11[1] = push_e(SP_B11, 1, 1);
      s.idx_c11[1] = push_e(SP_C11, 1, 1);
    } else if (m == 2) {
      s.idx_gamma = push_e(SP_GAMMA, 0, 2);
      s.idx_gammap = push_e(SP_GAMMAP, 0, 2);
    }
    for (int l = m; l <= s.L_big; ++l) {
      int lm = LM(l, m);
      if (l <= s.l_max_g) H.idx_I[lm] = (short)push_e(SP_I, l, m);
      if (s.has_pol && l >= 2 && l <= s.l_max_pol) H.idx_E[lm] = (short)push_e(SP_E, l, m);
      if (s.has_pol && m >= 1 && l >= 2 && l <= s.l_max_pol) H.idx_B[lm] = (short)push_e(SP_B, l, m);
      if (l <= s.l_max_ur) H.idx_N[lm] = (short)push_e(SP_N, l, m);
    }
    s.blk_size[b] = ni - s.blk_start[b];
  }
  s.n = ni;
  if (s.n > 32767) { snprintf(err, SONG2_ERRLEN, "system too large"); return 1; }
  /* structured iteration matrix of every block: the core (every entry that is not
     a hierarchy moment with l >= 3) and the moment chains I, E (paired with B where
     the block has B) and N over l >= 3.  A moment with l >= 3 couples only to the
     same species at l - 1, l, l + 1 (and E to B at the same l), so each chain is
     block tridiagonal, and its first node couples to the core's l = 2 moments. */
  H.mx_idx.clear();
  H.mx_pos.assign(s.n, 0);
  int off = 0;
  for (int b = 0; b < s.nblk; ++b) {
    int b0 = s.blk_start[b], nb = s.blk_size[b];
    std::vector<int> core;
    /* chain 0: I, 1: E/B, 2: N; per chain the state indices of (l, component) */
    std::vector<std::vector<std::pair<int, int>>> chain(3);
    for (int i = b0; i < b0 + nb; ++i) {
      int sp_ = H.eq_sp[i], l = H.eq_l[i];
      int ch = sp_ == SP_I ? 0 : (sp_ == SP_E || sp_ == SP_B) ? 1 : sp_ == SP_N ? 2 : -1;
      if (ch < 0 || l <= 2) core.push_back(i);
      else chain[ch].push_back({l, i});
    }
    if ((int)core.size() > S2_MAXCORE) {
      snprintf(err, SONG2_ERRLEN, "core of block m=%d has %d entries (max %d)", s.m[b], (int)core.size(), S2_MAXCORE);
      return 1;
    }
    s.core_n[b] = (int)core.size();
    s.core_idx[b] = (int)H.mx_idx.size();
    for (size_t p = 0; p < core.size(); ++p) {
      H.mx_idx.push_back((short)core[p]);
      H.mx_pos[core[p]] = (short)p;
    }
    int nch = 0;
    for (int ch = 0; ch < 3; ++ch) {
      if (chain[ch].empty()) continue;
      auto &v = chain[ch];
      int lfirst = v.front().first, llast = v.back().first;
      int len = llast - lfirst + 1;
      int d = (int)v.size() / len;
      if ((d != 1 && d != 2) || (int)v.size() != d * len) {
        snprintf(err, SONG2_ERRLEN, "moment chain %d of block m=%d is not regular", ch, s.m[b]);
        return 1;
      }
      s.ch_d[b][nch] = d;
      s.ch_len[b][nch] = len;
      s.ch_idx[b][nch] = (int)H.mx_idx.size();
      /* node k holds l = lfirst + k; component 0 is I, E or N, component 1 is B */
      std::vector<short> nodes((size_t)len * d, -1);
      for (auto &e : v) {
        int k = e.first - lfirst, comp = H.eq_sp[e.second] == SP_B ? 1 : 0;
        nodes[(size_t)k * d + comp] = (short)e.second;
        H.mx_pos[e.second] = (short)(((nch + 1) << 8) | (comp << 7) | k);
      }
      for (short x : nodes) {
        if (x < 0) {
          snprintf(err, SONG2_ERRLEN, "moment chain %d of block m=%d has a gap", ch, s.m[b]);
          return 1;
        }
        H.mx_idx.push_back(x);
      }
      s.ch_off[b][nch] = off;
      off += 3 * d * d * len + 2 * d * s.core_n[b];
      ++nch;
    }
    s.ch_n[b] = nch;
    s.core_off[b] = off;
    off += s.core_n[b] * s.core_n[b];
  }
  if ((int)H.mx_idx.size() != s.n) {
    snprintf(err, SONG2_ERRLEN, "iteration-matrix structure does not cover the state");
    return 1;
  }
  s.n_ch1 = s.n_ch2 = 0;
  for (int b = 0; b < s.nblk; ++b)
    for (int ch = 0; ch < s.ch_n[b]; ++ch) {
      if (s.ch_d[b][ch] == 1) s.ch1[s.n_ch1++] = (short)(b << 4 | ch);
      else s.ch2[s.n_ch2++] = (short)(b << 4 | ch);
    }
  s.lu_elems = off;

  /* evaluation order of the rows and of the quadratic-source entries: the
     hierarchy entries grouped by species (I, E, B, N), each group padded to whole
     warps, so that the threads of a warp run one code path; the few other entries
     (metric, matter, and the seven entries that carry the metric parts of the
     quadratic sources, heaviest first) go one per warp into free slots, so that
     their different code paths run side by side on different warps */
  auto slots = [](const std::vector<short> &sp_of, const std::vector<int> &first, std::vector<short> &out) {
    const int cls_sp[4] = {SP_I, SP_E, SP_B, SP_N};
    out.clear();
    std::vector<int> rest;
    for (int f : first)
      if (f >= 0) rest.push_back(f);
    for (size_t i = 0; i < sp_of.size(); ++i) {
      int sp_ = sp_of[i];
      if (sp_ == SP_NONE) continue;
      bool hier = false;
      for (int u = 0; u < 4; ++u) hier |= sp_ == cls_sp[u];
      bool listed = false;
      for (int f : first) listed |= f == (int)i;
      if (!hier && !listed) rest.push_back((int)i);
    }
    for (int g = 0; g < 4; ++g) {
      size_t start = out.size();
      for (size_t i = 0; i < sp_of.size(); ++i)
        if (sp_of[i] == cls_sp[g]) out.push_back((short)i);
      while ((out.size() - start) % 32) out.push_back(-1);
    }
    int nw = (int)out.size() / 32;
    std::vector<int> used(nw, 0);
    for (int e : rest) {
      int best = -1, bestscore = 0;
      for (int w = 0; w < nw; ++w) {
        int fr = 0;
        for (int u = 0; u < 32; ++u) fr += out[w * 32 + u] < 0;
        int score = fr - 64 * used[w];
        if (fr > 0 && (best < 0 || score > bestscore)) { best = w; bestscore = score; }
      }
      if (best < 0) {
        out.resize(out.size() + 32, -1);
        used.push_back(0);
        best = nw++;
      }
      for (int u = 31; u >= 0; --u)
        if (out[best * 32 + u] < 0) { out[best * 32 + u] = (short)e; break; }
      used[best]++;
    }
  };
  /* the core rows (everything but the hierarchy moments with l >= 3, which run
     from the GenRow table built below) */
  {
    std::vector<short> sp_core(H.eq_sp);
    for (int i = 0; i < s.n; ++i) {
      int sp_ = sp_core[i];
      if ((sp_ == SP_I || sp_ == SP_E || sp_ == SP_B || sp_ == SP_N) && H.eq_l[i] >= 3) sp_core[i] = SP_NONE;
    }
    slots(sp_core, {s.idx_phip}, H.row_slot);
  }
  slots(H.qs_sp, {s.iq_psi, s.iq_phi_prime_prime, s.iq_phi_prime_longitudinal, s.iq_phi_prime_poisson,
                  s.iq_omega_m1_prime, s.iq_gamma_m2_prime_prime, s.iq_vv_g}, H.qs_slot);
  /* the entries the source functions and the workspace read at an output time:
     the hierarchy moments up to l = max(2, l_max_los_t, l_max_los_p), the matter and
     the metric entries (perturb2_sources recomputes only what it uses) */
  {
    int lo = std::max(2, std::max(sp->l_max_los_t, sp->l_max_los_p));
    std::vector<short> sp_out(H.qs_sp);
    for (size_t i = 0; i < sp_out.size(); ++i) {
      int sp_ = sp_out[i];
      if ((sp_ == SP_I || sp_ == SP_E || sp_ == SP_B || sp_ == SP_N) && H.qs_l[i] > lo) sp_out[i] = SP_NONE;
    }
    slots(sp_out, {s.iq_psi, s.iq_phi_prime_prime, s.iq_phi_prime_longitudinal, s.iq_phi_prime_poisson,
                   s.iq_omega_m1_prime, s.iq_gamma_m2_prime_prime, s.iq_vv_g}, H.qo_slot);
  }
  s.n_row_slots = (int)H.row_slot.size();
  s.n_qs_slots = (int)H.qs_slot.size();
  s.n_qo_slots = (int)H.qo_slot.size();

  /* coupling tables for l <= Lq */
  H.cmin.assign((size_t)s.n_lm * 3, 0.0); H.cplu = H.cmin; H.dmin = H.cmin; H.dplu = H.cmin; H.dzer = H.cmin;
  for (int l = 0; l <= s.Lq; ++l)
    for (int i = 0; i < s.m_size; ++i) {
      int m = s.m[i];
      if (m > l) continue;
      int lm = LM(l, m);
      for (int m1 = m - 1; m1 <= m + 1; ++m1) {
        H.cmin[lm * 3 + m - m1 + 1] = song2_coupling_c_minus(l, m1, m);
        H.cplu[lm * 3 + m - m1 + 1] = song2_coupling_c_plus(l, m1, m);
        H.dmin[lm * 3 + m - m1 + 1] = song2_coupling_d_minus(l, m1, m);
        H.dplu[lm * 3 + m - m1 + 1] = song2_coupling_d_plus(l, m1, m);
        H.dzer[lm * 3 + m - m1 + 1] = song2_coupling_d_zero(l, m1, m);
      }
    }

  /* the chain rows as table entries (the same couplings and closures as the row
     function of the evolver) */
  H.gen.clear();
  for (int i = 0; i < s.n; ++i) {
    int sp_ = H.eq_sp[i], l = H.eq_l[i], m = H.eq_m[i];
    if (!(sp_ == SP_I || sp_ == SP_E || sp_ == SP_B || sp_ == SP_N) || l < 3) continue;
    GenRow r;
    memset(&r, 0, sizeof(r));
    r.i = (short)i;
    r.j1 = r.j2 = r.j3 = -1;
    int lm = LM(l, m);
    auto at = [&](const std::vector<short> &idx, int ll) -> short {
      if (ll < 0 || ll > s.Lq || m > ll) return -1;
      return idx[LM(ll, m)];
    };
    if (sp_ == SP_I || sp_ == SP_N) {
      const std::vector<short> &idx = sp_ == SP_I ? H.idx_I : H.idx_N;
      int lmax = sp_ == SP_I ? s.l_max_g : s.l_max_ur;
      r.kind = sp_ == SP_I ? 0 : 3;
      r.q = (short)((sp_ == SP_I ? s.iq_g : s.iq_ur) + lm);
      r.j1 = at(idx, l - 1);
      if (l == lmax) {
        r.c1 = sp_ == SP_I ? s.cl_I[m] : s.cl_N[m];
        r.cd = l + 1 + m;
      } else {
        r.c1 = H.cmin[lm * 3 + 1];
        r.c2 = -H.cplu[lm * 3 + 1];
        r.j2 = at(idx, l + 1);
      }
    } else {
      int e = sp_ == SP_E;
      const std::vector<short> &idx = e ? H.idx_E : H.idx_B;
      r.kind = e ? 1 : 2;
      r.q = (short)((e ? s.iq_E : s.iq_B) + lm);
      r.j1 = l - 1 >= 2 ? at(idx, l - 1) : -1;
      r.j3 = (m >= 1) ? (e ? H.idx_B[lm] : H.idx_E[lm]) : -1;
      if (l == s.l_max_pol) {
        r.c1 = s.cl_P[m];
        r.c3 = e ? -s.cmix_P[m] : s.cmix_P[m];
        r.cd = l + 3;
      } else {
        r.c1 = H.dmin[lm * 3 + 1];
        r.c2 = -H.dplu[lm * 3 + 1];
        r.c3 = e ? -H.dzer[lm * 3 + 1] : H.dzer[lm * 3 + 1];
        r.j2 = at(idx, l + 1);
      }
    }
    H.gen.push_back(r);
  }
  s.n_gen = (int)H.gen.size();

  /* source types (perturb2_indices_of_perturbs, perturbations2.c:667-1075) */
  int tp = 0;
  auto add_tp = [&](int kind, int lmax) {
    int base = tp;
    for (int l = 0; l <= lmax; ++l)
      for (int i = 0; i < s.m_size; ++i)
        if (s.m[i] <= l) {
          int t = base + LM(l, s.m[i]);
          if (t >= S2_MAXTP) continue;
          s.tp_kind[t] = kind; s.tp_l[t] = l; s.tp_m[t] = s.m[i];
        }
    tp = base + size_l_indexm(lmax, s.m, s.m_size);
  };
  if (!first_order_mode) {
    if (sp->has_source_T) add_tp(TP_T, sp->l_max_los_t);
    if (sp->has_source_E) add_tp(TP_E, sp->l_max_los_p);
    if (sp->has_source_B) add_tp(TP_B, sp->l_max_los_p);
    if (sp->has_source_delta_cdm) { s.tp_kind[tp] = TP_D; s.tp_l[tp] = 0; s.tp_m[tp] = 0; ++tp; }
  }
  if (tp > S2_MAXTP) { snprintf(err, SONG2_ERRLEN, "too many source types"); return 1; }
  s.tp2_size = tp;
  s.mode_first_order = first_order_mode;
  s.tau_size = sp->tau_size;
  s.k_size = sp->k_size;
  /* tables */
  s.bg_size = tab->bg_size;
  s.bg_lntau0 = tab->bg_lntau0;
  s.bg_dlntau = tab->bg_dlntau;
  s.bg_inv_dx = 1.0 / tab->bg_dlntau;
  s.bg_dx2_6 = tab->bg_dlntau * tab->bg_dlntau / 6.0;
  if (!first_order_mode) {
    s.fo_l_max = tab->fo_l_max;
    s.nfo = song2_fo_size(tab->fo_l_max);
    if (tab->fo_size != s.nfo || tab->fo_k_size != sp->k_size || !tab->fo || !tab->fo_dd) {
      snprintf(err, SONG2_ERRLEN, "first-order table does not match the spec");
      return 1;
    }
    if (tab->fo_l_max < s.L_big + 1) {
      snprintf(err, SONG2_ERRLEN, "first-order table stores l <= %d, need %d", tab->fo_l_max, s.L_big + 1);
      return 1;
    }
    s.fo_tau_size = tab->fo_tau_size;
    s.fo_lntau0 = tab->fo_lntau0;
    s.fo_dlntau = tab->fo_dlntau;
    s.fo_inv_dx = 1.0 / tab->fo_dlntau;
    s.fo_dx2_6 = tab->fo_dlntau * tab->fo_dlntau / 6.0;
    s.fo_k_size = tab->fo_k_size;
  }
  s.fo_E = SONG2_FO_I + (s.fo_l_max + 1);
  s.fo_N = SONG2_FO_I + 2 * (s.fo_l_max + 1);
  s.fo_CG = SONG2_FO_I + 3 * (s.fo_l_max + 1);
  s.lu_stride = s.lu_elems;
  s.qtab_stride = (long)s.fo_tau_size * 2 * s.qs2_size;
  return 0;
}

/* Layouts of the hierarchy classes of an uneven batch: the run-wide spec with the
   class's l_max and modes 0..m_max; the source types stay the run-wide ones. */
int build_class_layouts(const song2_spec *sp, const song2_tables *tab, const DevSpec &run, std::vector<HostLayout> &HC,
                        char *err) {
  if (!sp->class_l_max || !sp->class_m_max || !sp->triplet_class) {
    snprintf(err, SONG2_ERRLEN, "n_classes > 0 needs class_l_max, class_m_max and triplet_class");
    return 1;
  }
  HC.resize(sp->n_classes);
  for (int k = 0; k < sp->n_classes; ++k) {
    int L = sp->class_l_max[k], mm = sp->class_m_max[k];
    if (L < 2 || L > sp->l_max_g || L > sp->l_max_ur || (sp->has_polarization2 && L > sp->l_max_pol_g)) {
      snprintf(err, SONG2_ERRLEN, "class %d: l_max %d outside 2..run-wide l_max", k, L);
      return 1;
    }
    if (mm < 0 || mm >= SONG2_MAX_M) {
      snprintf(err, SONG2_ERRLEN, "class %d: m_max %d outside 0..%d", k, mm, SONG2_MAX_M - 1);
      return 1;
    }
    for (int m = 0; m <= mm; ++m)
      if (!run.compute_m[m]) {
        snprintf(err, SONG2_ERRLEN, "class %d: mode %d is not in the run-wide mode list", k, m);
        return 1;
      }
    song2_spec sc = *sp;
    sc.n_classes = 0;
    sc.l_max_g = sc.l_max_ur = L;
    if (sp->has_polarization2) sc.l_max_pol_g = L;
    sc.m_size = mm + 1;
    for (int m = 0; m <= mm; ++m) sc.m[m] = m;
    if (build_layout(&sc, tab, 0, HC[k], err)) return 1;
    DevSpec &d = HC[k].s;
    d.tp2_size = run.tp2_size;
    memcpy(d.tp_kind, run.tp_kind, sizeof(d.tp_kind));
    memcpy(d.tp_l, run.tp_l, sizeof(d.tp_l));
    memcpy(d.tp_m, run.tp_m, sizeof(d.tp_m));
  }
  return 0;
}

/* ppt2->coupling_coefficients of the three fields in the dt_index() layout */
static std::vector<double> dt_table(const DevSpec &s) {
  std::vector<double> t;
  if (!s.dtilde) return t;
  t.assign(dt_table_size(s), 0.0);
  int Q = s.dt_Q;
  for (int f = 0; f < 3; ++f)
    for (int l = 0; l <= s.dt_L; ++l)
      for (int m = 0; m <= std::min(l, SONG2_MAX_M - 1); ++m)
        for (int l1 = 0; l1 <= Q; ++l1)
          for (int m1 = -l1; m1 <= l1; ++m1)
            for (int l2 = 0; l2 <= Q; ++l2)
              t[dt_index(s, f, l, m, l1, m1, l2)] = song2_delta_tilde_coupling(f, l, m, l1, m1, l2);
  return t;
}

template <typename V> int upload(song2_ctx *c, const V &v, const typename V::value_type **dst, cudaStream_t st, char *err) {
  void *p = nullptr;
  size_t bytes = std::max<size_t>(1, v.size() * sizeof(typename V::value_type));
  CK(cudaMalloc(&p, bytes));
  c->allocs.push_back(p);
  if (!v.empty()) CK(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(typename V::value_type), cudaMemcpyHostToDevice, st));
  *dst = (const typename V::value_type *)p;
  return 0;
}

int upload_raw(song2_ctx *c, const void *src, size_t bytes, void **dst, cudaStream_t st, char *err) {
  void *p = nullptr;
  CK(cudaMalloc(&p, std::max<size_t>(1, bytes)));
  c->allocs.push_back(p);
  if (bytes) CK(cudaMemcpyAsync(p, src, bytes, cudaMemcpyHostToDevice, st));
  *dst = p;
  return 0;
}

int alloc_dev(song2_ctx *c, size_t bytes, void **dst, char *err) {
  void *p = nullptr;
  CK(cudaMalloc(&p, std::max<size_t>(1, bytes)));
  c->allocs.push_back(p);
  *dst = p;
  return 0;
}

/* Shared set-up of a context: spec layout, tables, work items. */
int ctx_setup(song2_ctx *c, const song2_spec *sp, const song2_tables *tab, int precision, int first_order_mode,
              const std::vector<WorkItem> &items, const std::vector<double> &k3, const std::vector<int> &k3_off,
              const std::vector<int> &k3_size, const std::vector<int64_t> &pair_off, int fo_tau_size,
              double fo_lntau0, double fo_dlntau, int fo_l_max, char *err) {
  HostLayout H;
  if (first_order_mode) {
    /* the layout needs fo sizes for the output table */
    memset(&H.s, 0, sizeof(H.s));
  }
  if (build_layout(sp, tab, first_order_mode, H, err)) return 1;
  DevSpec &s = H.s;
  std::vector<HostLayout> HC;
  int classes = !first_order_mode && sp->n_classes > 0;
  if (classes && build_class_layouts(sp, tab, s, HC, err)) return 1;
  if (classes)
    for (const WorkItem &w : items)
      if (w.cls < 0 || w.cls >= sp->n_classes) {
        snprintf(err, SONG2_ERRLEN, "triplet_class entry %d outside 0..%d", w.cls, sp->n_classes - 1);
        return 1;
      }
  if (classes) {
    /* scratch strides of the largest class */
    for (auto &hc : HC) {
      s.lu_stride = std::max(s.lu_stride, hc.s.lu_elems);
      s.qtab_stride = std::max(s.qtab_stride, hc.s.qtab_stride);
    }
  }
  if (first_order_mode) {
    s.fo_l_max = fo_l_max;
    s.nfo = song2_fo_size(fo_l_max);
    s.fo_tau_size = fo_tau_size;
    s.fo_lntau0 = fo_lntau0;
    s.fo_dlntau = fo_dlntau;
    s.fo_inv_dx = 1.0 / fo_dlntau;
    s.fo_dx2_6 = fo_dlntau * fo_dlntau / 6.0;
    s.fo_k_size = sp->k_size;
    s.fo_E = SONG2_FO_I + (fo_l_max + 1);
    s.fo_N = SONG2_FO_I + 2 * (fo_l_max + 1);
    s.fo_CG = SONG2_FO_I + 3 * (fo_l_max + 1);
  }
  s.n_items = (int)items.size();
  c->precision = precision;
  c->n_items = s.n_items;
  c->tp2_size = s.tp2_size;
  int64_t per_type = 0;
  if (!first_order_mode) per_type = song2_sources_per_type(sp);
  s.per_type = per_type;
  c->per_type = per_type;

  int dev = 0, nsm = 0, smem_optin = 0;
  CK(cudaGetDevice(&dev));
  /* the evolver keeps its per-thread workspace copy (Jacobian probes) on the stack */
  size_t stack = 0;
  CK(cudaDeviceGetLimit(&stack, cudaLimitStackSize));
  if (stack < 4096) CK(cudaDeviceSetLimit(cudaLimitStackSize, 4096));
  CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  CK(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  /* launch configuration: explicit, or the default below */
  song2_launch L = c->launch;
  /* SONG2_LAUNCH="warp_team,teams_per_cta,threads_per_team,lu_in_smem" overrides the
     automatic choice (used to pin a configuration in profiling commands) */
  const char *env = getenv("SONG2_LAUNCH");
  if (env && L.teams_per_cta <= 0 && L.threads_per_team <= 0 && !L.warp_team) {
    int a = 0, b = 0, t = 0, d = 0;
    if (sscanf(env, "%d,%d,%d,%d", &a, &b, &t, &d) == 4) {
      L.warp_team = a; L.teams_per_cta = b; L.threads_per_team = t; L.lu_in_smem = d;
    }
  }
  if (classes) {
    /* uneven batches run one CTA per triplet; automatic: 256 threads, iteration
       matrices in shared memory where they fit */
    L.warp_team = 0;
    L.teams_per_cta = 1;
    if (L.threads_per_team <= 0) {
      L.threads_per_team = 256;
      L.lu_in_smem = 1;
    }
  }
  if (L.teams_per_cta <= 0 && L.threads_per_team <= 0 && !L.warp_team) {
    /* measured on config-2-sized problems: both forms are fastest with 256
       threads and their iteration matrices in shared memory (two CTAs per SM) */
    L.warp_team = 0;
    L.teams_per_cta = 1;
    L.threads_per_team = 256;
    L.lu_in_smem = 1;
  }
  if (L.warp_team == 2) {
    /* G lanes per triplet: G a power of two up to 32, whole warps per CTA, at most
       four warps per CTA */
    int G = 1;
    while (G < L.threads_per_team && G < 32) G <<= 1;
    L.threads_per_team = G;
    int per_warp = 32 / G;
    int warps = (L.teams_per_cta + per_warp - 1) / per_warp;
    warps = std::max(1, std::min(4, warps));
    L.teams_per_cta = warps * per_warp;
    L.lu_in_smem = 0;
    c->block = 32 * warps;
  } else if (L.warp_team) {
    if (L.teams_per_cta < 1) L.teams_per_cta = 4;
    if (L.teams_per_cta > 8) L.teams_per_cta = 8;
    L.threads_per_team = 32;
    c->block = 32 * L.teams_per_cta;
  } else {
    L.teams_per_cta = 1;
    if (L.threads_per_team < 32) L.threads_per_team = 256;
    L.threads_per_team = std::min(256, (L.threads_per_team / 32) * 32);
    c->block = L.threads_per_team;
  }
  /* shared memory of a CTA: the team plans (the largest class in uneven batches,
     after the copy of the class spec) */
  auto plan_bytes = [&](int lu) -> size_t {
    if (!classes) return song2_smem_bytes(s, precision, c->block, lu) * L.teams_per_cta;
    size_t mx = 0;
    for (auto &hc : HC) mx = std::max(mx, song2_smem_bytes(hc.s, precision, c->block, lu));
    return song2_class_spec_bytes() + mx;
  };
  /* uneven batches: per class, the iteration matrices go to shared memory when
     they fit the class's launch group (two CTAs per SM for the classes whose plan
     without them fits half an SM, one CTA per SM for the others) */
  int smem_sm = 0;
  CK(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
  size_t half = (size_t)smem_sm / 2 > 1024 ? (size_t)smem_sm / 2 - 1024 : 0;
  /* SONG2_CLASS_SPLIT_BYTES overrides the plan size that separates the groups */
  const char *split = getenv("SONG2_CLASS_SPLIT_BYTES");
  if (split && atol(split) > 0) half = (size_t)atol(split);
  std::vector<size_t> pb(HC.size());
  std::vector<int> small_cls(HC.size(), 0);
  int any_global_lu = 0;
  for (size_t k = 0; k < HC.size(); ++k) {
    size_t p0 = song2_class_spec_bytes() + song2_smem_bytes(HC[k].s, precision, c->block, 0);
    size_t p1 = song2_class_spec_bytes() + song2_smem_bytes(HC[k].s, precision, c->block, 1);
    small_cls[k] = p0 <= half;
    size_t room = small_cls[k] ? half : (size_t)smem_optin;
    HC[k].s.lu_in_smem = L.lu_in_smem && p1 <= room;
    pb[k] = HC[k].s.lu_in_smem ? p1 : p0;
    any_global_lu |= !HC[k].s.lu_in_smem;
  }
  if (classes) {
    s.lu_in_smem = !any_global_lu;
  } else {
    if (L.lu_in_smem && plan_bytes(1) > (size_t)smem_optin) L.lu_in_smem = 0;
    s.lu_in_smem = L.lu_in_smem;
  }
  s.team_lanes = L.warp_team == 2 ? L.threads_per_team : 0;
  if (L.warp_team == 2) c->smem = song2_team_smem_bytes(s, L.teams_per_cta);
  else if (classes) c->smem = *std::max_element(pb.begin(), pb.end());
  else c->smem = plan_bytes(s.lu_in_smem);
  if (c->smem > (size_t)smem_optin) {
    snprintf(err, SONG2_ERRLEN, "shared-memory plan %zu B exceeds the %d B limit", c->smem, smem_optin);
    return 1;
  }
  c->launch = L;
  c->kmode = L.warp_team;
  if (!classes && L.warp_team == 0) {
    /* the kernel whose registers allow two CTAs per SM when the shared-memory plan
       does too (the compiler otherwise spends up to the 255 registers of one) */
    int p0 = song2_max_ctas_per_sm(precision, 0, c->block, c->smem);
    int p5 = song2_max_ctas_per_sm(precision, 5, c->block, c->smem);
    if (p5 > p0) c->kmode = 5;
  }
  int per_sm = song2_max_ctas_per_sm(precision, classes ? 4 : c->kmode, c->block, c->smem);
  if (per_sm < 1) {
    snprintf(err, SONG2_ERRLEN, "launch configuration does not fit on an SM");
    return 1;
  }
  int ctas_needed = (s.n_items + L.teams_per_cta - 1) / L.teams_per_cta;
  c->grid = std::max(1, std::min(ctas_needed, nsm * per_sm));
  c->n_teams = c->grid * L.teams_per_cta;
  std::vector<WorkItem> gitems(items.begin(), items.end());
  c->groups.clear();
  if (classes) {
    std::vector<WorkItem> big, small;
    size_t smem_big = 0, smem_small = 0;
    for (const WorkItem &w : gitems) {
      if (!small_cls[w.cls]) { big.push_back(w); smem_big = std::max(smem_big, pb[w.cls]); }
      else { small.push_back(w); smem_small = std::max(smem_small, pb[w.cls]); }
    }
    /* the classes with large plans first (one CTA per SM, the kernel with the
       registers of a full SM), then the small ones (two CTAs per SM, the kernel
       whose registers allow two) */
    gitems = big;
    gitems.insert(gitems.end(), small.begin(), small.end());
    int nt = 0;
    for (int g = 0; g < 2; ++g) {
      song2_ctx::Group G;
      G.first = g == 0 ? 0 : (int)big.size();
      G.count = g == 0 ? (int)big.size() : (int)small.size();
      if (G.count == 0) continue;
      G.smem = g == 0 ? smem_big : smem_small;
      G.mode = g == 0 ? 3 : 4;
      int ps = song2_max_ctas_per_sm(precision, G.mode, c->block, G.smem);
      if (ps < 1) {
        snprintf(err, SONG2_ERRLEN, "launch configuration does not fit on an SM");
        return 1;
      }
      G.grid = std::max(1, std::min(G.count, nsm * ps));
      nt = std::max(nt, G.grid);
      c->groups.push_back(G);
    }
    c->n_teams = nt;
  }

  cudaStream_t st = 0;
  DevPtrs &p = c->ptrs;
  memset(&p, 0, sizeof(p));
  std::vector<double> kv(sp->k, sp->k + sp->k_size);
  if (upload(c, kv, &p.k, st, err)) return 1;
  if (upload(c, k3, &p.k3, st, err)) return 1;
  if (!first_order_mode) {
    std::vector<double> tv(sp->tau, sp->tau + sp->tau_size);
    if (upload(c, tv, &p.tau, st, err)) return 1;
  } else {
    std::vector<double> tv(1, 0.0);
    if (upload(c, tv, &p.tau, st, err)) return 1;
  }
  if (upload(c, k3_off, &p.k3_off, st, err)) return 1;
  if (upload(c, k3_size, &p.k3_size, st, err)) return 1;
  if (upload(c, pair_off, &p.pair_off, st, err)) return 1;
  size_t bgb = (size_t)tab->bg_size * SONG2_BG_SIZE * sizeof(double);
  void *tmp;
  if (upload_raw(c, tab->bg, bgb, &tmp, st, err)) return 1;
  p.bg = (const double *)tmp;
  if (upload_raw(c, tab->bg_dd, bgb, &tmp, st, err)) return 1;
  p.bg_dd = (const double *)tmp;
  if (!first_order_mode) {
    size_t fob = (size_t)tab->fo_k_size * tab->fo_tau_size * tab->fo_size * sizeof(double);
    if (upload_raw(c, tab->fo, fob, &tmp, st, err)) return 1;
    p.fo = (const double *)tmp;
    if (upload_raw(c, tab->fo_dd, fob, &tmp, st, err)) return 1;
    p.fo_dd = (const double *)tmp;
  } else {
    p.fo = p.fo_dd = p.bg;  /* never read in first-order mode */
  }
  if (upload(c, H.cmin, &p.tabs.cmin, st, err) || upload(c, H.cplu, &p.tabs.cplu, st, err) || upload(c, H.dmin, &p.tabs.dmin, st, err) ||
      upload(c, H.dplu, &p.tabs.dplu, st, err) || upload(c, H.dzer, &p.tabs.dzer, st, err))
    return 1;
  if (upload(c, H.eq_sp, &p.tabs.eq_sp, st, err) || upload(c, H.eq_l, &p.tabs.eq_l, st, err) || upload(c, H.eq_m, &p.tabs.eq_m, st, err))
    return 1;
  if (upload(c, H.idx_I, &p.tabs.idx_I, st, err) || upload(c, H.idx_E, &p.tabs.idx_E, st, err) ||
      upload(c, H.idx_B, &p.tabs.idx_B, st, err) || upload(c, H.idx_N, &p.tabs.idx_N, st, err))
    return 1;
  if (upload(c, H.qs_sp, &p.tabs.qs_sp, st, err) || upload(c, H.qs_l, &p.tabs.qs_l, st, err) || upload(c, H.qs_m, &p.tabs.qs_m, st, err))
    return 1;
  if (upload(c, H.row_slot, &p.tabs.row_slot, st, err) || upload(c, H.qs_slot, &p.tabs.qs_slot, st, err)) return 1;
  if (upload(c, H.mx_idx, &p.tabs.mx_idx, st, err) || upload(c, H.mx_pos, &p.tabs.mx_pos, st, err)) return 1;
  if (upload(c, H.qo_slot, &p.tabs.qo_slot, st, err)) return 1;
  if (upload(c, H.gen, &p.tabs.gen, st, err)) return 1;
  if (upload(c, gitems, &p.items, st, err)) return 1;
  c->h_items = gitems;
  if (classes) {
    /* per-class specs (run-level fields from the run-wide spec) and tables */
    std::vector<DevSpec> cspec;
    std::vector<ClassTabs> ctabs;
    for (auto &hc : HC) {
      DevSpec d = hc.s;
      d.n_items = s.n_items;
      d.per_type = s.per_type;
      d.team_lanes = 0;
      d.lu_stride = s.lu_stride;
      d.qtab_stride = s.qtab_stride;
      cspec.push_back(d);
      ClassTabs t;
      memset(&t, 0, sizeof(t));
      if (upload(c, hc.cmin, &t.cmin, st, err) || upload(c, hc.cplu, &t.cplu, st, err) ||
          upload(c, hc.dmin, &t.dmin, st, err) || upload(c, hc.dplu, &t.dplu, st, err) ||
          upload(c, hc.dzer, &t.dzer, st, err) || upload(c, hc.eq_sp, &t.eq_sp, st, err) ||
          upload(c, hc.eq_l, &t.eq_l, st, err) || upload(c, hc.eq_m, &t.eq_m, st, err) ||
          upload(c, hc.idx_I, &t.idx_I, st, err) || upload(c, hc.idx_E, &t.idx_E, st, err) ||
          upload(c, hc.idx_B, &t.idx_B, st, err) || upload(c, hc.idx_N, &t.idx_N, st, err) ||
          upload(c, hc.qs_sp, &t.qs_sp, st, err) || upload(c, hc.qs_l, &t.qs_l, st, err) ||
          upload(c, hc.qs_m, &t.qs_m, st, err) || upload(c, hc.row_slot, &t.row_slot, st, err) ||
          upload(c, hc.qs_slot, &t.qs_slot, st, err) || upload(c, hc.mx_idx, &t.mx_idx, st, err) ||
          upload(c, hc.mx_pos, &t.mx_pos, st, err) || upload(c, hc.qo_slot, &t.qo_slot, st, err) ||
          upload(c, hc.gen, &t.gen, st, err))
        return 1;
      ctabs.push_back(t);
    }
    if (upload(c, cspec, &p.class_spec, st, err) || upload(c, ctabs, &p.class_tabs, st, err)) return 1;
  }
  if (!first_order_mode) {
    c->sources_len = (size_t)s.tp2_size * per_type;
    if (alloc_dev(c, std::max<size_t>(1, c->sources_len) * sizeof(double), &tmp, err)) return 1;
    c->d_sources = (double *)tmp;
    CK(cudaMemsetAsync(c->d_sources, 0, std::max<size_t>(1, c->sources_len) * sizeof(double), st));
    p.sources = c->d_sources;
  } else {
    c->fo_out_len = (size_t)sp->k_size * fo_tau_size * s.nfo;
    if (alloc_dev(c, c->fo_out_len * sizeof(double), &tmp, err)) return 1;
    c->d_fo_out = (double *)tmp;
    p.fo_out = c->d_fo_out;
  }
  if (alloc_dev(c, sizeof(song2_triplet_stats) * std::max(1, s.n_items), &tmp, err)) return 1;
  c->d_stats = (song2_triplet_stats *)tmp;
  p.stats = c->d_stats;
  /* Evolver scratch: the Jacobian blocks of each resident CTA, and the LU
     blocks when they do not fit in shared memory. */
  if (alloc_dev(c, (size_t)c->n_teams * s.lu_stride * sizeof(double), &tmp, err)) return 1;
  p.jac = (double *)tmp;
  /* quadratic-source tables of the resident triplets, and the spline recurrence */
  if (s.has_qs) {
    if (alloc_dev(c, (size_t)c->n_teams * s.qtab_stride * sizeof(double), &tmp, err)) return 1;
    p.qtab = (double *)tmp;
  }
  {
    std::vector<double> cs(std::max(2, s.fo_tau_size + 1), 0.0);
    double cprev = 0.0;
    for (size_t j = 1; j < cs.size(); ++j) {
      double bb = 4.0 - cprev;
      cs[j] = 1.0 / bb;
      cprev = cs[j];
    }
    if (upload(c, cs, &p.spl_c, st, err)) return 1;
  }
  if (s.dtilde && upload(c, dt_table(s), &p.dt_coup, st, err)) return 1;
  if (!s.lu_in_smem) {
    size_t ts = precision == SONG2_PREC_MIXED ? sizeof(float) : sizeof(double);
    if (alloc_dev(c, (size_t)c->n_teams * s.lu_stride * ts, &tmp, err)) return 1;
    p.lu_global = tmp;
  }
  if (L.warp_team == 2) {
    /* team kernel: vectors, solve vectors and pivots of every resident team */
    size_t ts = precision == SONG2_PREC_MIXED ? sizeof(float) : sizeof(double);
    if (alloc_dev(c, (size_t)c->n_teams * song2_team_slab_doubles(s) * sizeof(double), &tmp, err)) return 1;
    p.tslab = (double *)tmp;
    if (alloc_dev(c, (size_t)c->n_teams * s.n * ts, &tmp, err)) return 1;
    p.txsol = tmp;
  }
  if (alloc_dev(c, sizeof(int), &tmp, err)) return 1;
  c->d_queue = (int *)tmp;
  p.queue = c->d_queue;
#ifdef SONG2_PHASE_TIMERS
  if (alloc_dev(c, 2 * S2_NPHASE * sizeof(unsigned long long), &tmp, err)) return 1;
  CK(cudaMemsetAsync(tmp, 0, 2 * S2_NPHASE * sizeof(unsigned long long), st));
  p.phase = (unsigned long long *)tmp;
#endif
  CK(cudaStreamSynchronize(st));
  c->spec = s;
  CK(cudaEventCreate(&c->ev0));
  CK(cudaEventCreate(&c->ev1));
  return 0;
}

void pair_tables(const song2_spec *sp, std::vector<int> &k3_off, std::vector<int> &k3_size,
                 std::vector<int64_t> &pair_off) {
  k3_off.clear(); k3_size.clear(); pair_off.clear();
  int off = 0;
  int64_t po = 0;
  for (int i1 = 0; i1 < sp->k_size; ++i1)
    for (int i2 = 0; i2 <= i1; ++i2) {
      int n3 = sp->k3_size[i1 * sp->k_size + i2];
      k3_off.push_back(off);
      k3_size.push_back(n3);
      pair_off.push_back(po);
      off += n3;
      po += (int64_t)sp->tau_size * n3;
    }
}

} // namespace

/* cost-sorted work list: (reference work-order index, item) */
static void sorted_items(const song2_spec *spec, const std::vector<double> &k3, const std::vector<int> &k3_off,
                         const std::vector<int> &k3_size, std::vector<WorkItem> &sorted, std::vector<int64_t> &ref_index) {
  std::vector<WorkItem> items;
  std::vector<double> cost;
  int pair = 0;
  for (int i1 = 0; i1 < spec->k_size; ++i1)
    for (int i2 = 0; i2 <= i1; ++i2, ++pair)
      for (int i3 = 0; i3 < k3_size[pair]; ++i3) {
        /* hierarchy class of an uneven batch (triplets numbered in pair order) */
        int has_cls = spec->n_classes > 0 && spec->triplet_class && spec->class_l_max && spec->class_m_max;
        int cls = has_cls ? spec->triplet_class[k3_off[pair] + i3] : 0;
        items.push_back(WorkItem{i1, i2, i3, pair, cls, 0});
        double kk = std::max(spec->k[i1], std::max(spec->k[i2], k3[k3_off[pair] + i3]));
        /* cost: steps grow with k; per-step work with the class's hierarchy size */
        if (has_cls && cls >= 0 && cls < spec->n_classes)
          kk *= (spec->class_l_max[cls] + 1.0) * (spec->class_m_max[cls] + 1.0);
        cost.push_back(kk);
      }
  /* reference order start of every pair */
  int npairs = pair;
  std::vector<int64_t> start(npairs, 0);
  int64_t acc = 0;
  for (int i1 = spec->k_size - 1; i1 >= 0; --i1)
    for (int i2 = 0; i2 <= i1; ++i2) {
      int pr = i1 * (i1 + 1) / 2 + i2;
      start[pr] = acc;
      acc += k3_size[pr];
    }
  std::vector<size_t> order(items.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return cost[a] > cost[b]; });
  sorted.resize(items.size());
  ref_index.resize(items.size());
  for (size_t i = 0; i < order.size(); ++i) {
    sorted[i] = items[order[i]];
    ref_index[i] = start[sorted[i].pair] + sorted[i].i3;
    sorted[i].ref = (int)ref_index[i];
  }
}

extern "C" {

int64_t song2_shard_items(const song2_spec *spec, int shard, int n_shards, int64_t *out) {
  if (n_shards < 1 || shard < 0 || shard >= n_shards) return -1;
  std::vector<int> k3_off, k3_size;
  std::vector<int64_t> pair_off;
  pair_tables(spec, k3_off, k3_size, pair_off);
  int n3tot = k3_off.empty() ? 0 : k3_off.back() + k3_size.back();
  std::vector<double> k3(spec->k3, spec->k3 + n3tot);
  std::vector<WorkItem> sorted;
  std::vector<int64_t> ref;
  sorted_items(spec, k3, k3_off, k3_size, sorted, ref);
  int64_t n = 0;
  for (size_t i = shard; i < sorted.size(); i += n_shards) {
    if (out) out[n] = ref[i];
    ++n;
  }
  return n;
}

static int ctx_create_impl(const song2_spec *spec, const song2_tables *tab, int precision, const song2_launch *launch,
                           int shard, int n_shards, song2_ctx **out, char *err, const int64_t *list = nullptr,
                           int64_t n_list = -1) {
  *out = nullptr;
  if (n_shards < 1 || shard < 0 || shard >= n_shards) {
    snprintf(err, SONG2_ERRLEN, "bad shard %d of %d", shard, n_shards);
    return 1;
  }
  if (precision != SONG2_PREC_FP64 && precision != SONG2_PREC_MIXED) {
    snprintf(err, SONG2_ERRLEN, "unknown precision %d", precision);
    return 1;
  }
  std::vector<int> k3_off, k3_size;
  std::vector<int64_t> pair_off;
  pair_tables(spec, k3_off, k3_size, pair_off);
  int n3tot = k3_off.empty() ? 0 : k3_off.back() + k3_size.back();
  std::vector<double> k3(spec->k3, spec->k3 + n3tot);
  /* work items, largest wavenumber first: the expensive triplets start early so the
     persistent CTAs finish together (longest-processing-time order) */
  std::vector<WorkItem> sorted, mine;
  std::vector<int64_t> ref;
  sorted_items(spec, k3, k3_off, k3_size, sorted, ref);
  if (list) {
    /* an explicit list of reference work-order indices, kept in cost order */
    std::vector<char> want(sorted.size(), 0);
    for (int64_t i = 0; i < n_list; ++i) {
      if (list[i] < 0 || list[i] >= (int64_t)sorted.size()) {
        snprintf(err, SONG2_ERRLEN, "triplet index %lld outside 0..%zu", (long long)list[i], sorted.size() - 1);
        return 1;
      }
      want[list[i]] = 1;
    }
    for (size_t i = 0; i < sorted.size(); ++i)
      if (want[ref[i]]) mine.push_back(sorted[i]);
    if (mine.empty()) {
      snprintf(err, SONG2_ERRLEN, "empty triplet list");
      return 1;
    }
  } else {
    for (size_t i = shard; i < sorted.size(); i += n_shards) mine.push_back(sorted[i]);
  }
  song2_ctx *c = new song2_ctx();
  memset((void *)&c->spec, 0, sizeof(c->spec));
  if (launch) c->launch = *launch;
  if (ctx_setup(c, spec, tab, precision, 0, mine, k3, k3_off, k3_size, pair_off, 0, 0, 0, 0, err)) {
    song2_ctx_destroy(c);
    return 1;
  }
  *out = c;
  return 0;
}

int song2_ctx_create(const song2_spec *spec, const song2_tables *tab, int precision, song2_ctx **out, char *err) {
  return ctx_create_impl(spec, tab, precision, nullptr, 0, 1, out, err);
}

int song2_ctx_create_shard(const song2_spec *spec, const song2_tables *tab, int precision, int shard, int n_shards,
                           song2_ctx **out, char *err) {
  return ctx_create_impl(spec, tab, precision, nullptr, shard, n_shards, out, err);
}

int song2_ctx_create_list(const song2_spec *spec, const song2_tables *tab, int precision, const int64_t *items,
                          int64_t n_items, song2_ctx **out, char *err) {
  if (!items || n_items < 1) {
    snprintf(err, SONG2_ERRLEN, "empty triplet list");
    return 1;
  }
  return ctx_create_impl(spec, tab, precision, nullptr, 0, 1, out, err, items, n_items);
}

int song2_ctx_create_ex(const song2_spec *spec, const song2_tables *tab, int precision, const song2_launch *launch,
                        int shard, int n_shards, song2_ctx **out, char *err) {
  return ctx_create_impl(spec, tab, precision, launch, shard, n_shards, out, err);
}

void song2_ctx_get_launch(song2_ctx *c, song2_launch *out, int *grid, int *block, size_t *smem) {
  if (out) *out = c->launch;
  if (grid) *grid = c->grid;
  if (block) *block = c->block;
  if (smem) *smem = c->smem;
}

int song2_autotune(const song2_spec *spec, const song2_tables *tab, int precision, int sample, song2_launch *best,
                   double *best_ms, char *err) {
  /* sample: the `sample` most expensive triplets (the head of the cost-sorted order),
     evolved as one run with each candidate configuration */
  if (sample < 1) sample = 1;
  std::vector<int> k3_off, k3_size;
  std::vector<int64_t> pair_off;
  pair_tables(spec, k3_off, k3_size, pair_off);
  int n3tot = k3_off.empty() ? 0 : k3_off.back() + k3_size.back();
  std::vector<double> k3(spec->k3, spec->k3 + n3tot);
  std::vector<WorkItem> sorted;
  std::vector<int64_t> ref;
  sorted_items(spec, k3, k3_off, k3_size, sorted, ref);
  /* spread the sample over the cost range so that the timing reflects the mix */
  std::vector<WorkItem> pick;
  size_t stride = std::max<size_t>(1, sorted.size() / (size_t)sample);
  for (size_t i = 0; i < sorted.size() && (int)pick.size() < sample; i += stride) pick.push_back(sorted[i]);
  /* candidates: CTA teams of 128, 192 or 256 threads with the factors in shared
     or global memory, warp teams, lane teams; uneven batches (hierarchy classes)
     run CTA teams only */
  const song2_launch all[] = {
      {0, 1, 256, 1}, {0, 1, 192, 1}, {0, 1, 128, 1}, {0, 1, 256, 0}, {1, 4, 32, 0}, {1, 8, 32, 0}, {2, 16, 8, 0},
  };
  int ncand = spec->n_classes > 0 ? 3 : (int)(sizeof(all) / sizeof(all[0]));
  double bestv = 1e300;
  int found = 0;
  for (int ci = 0; ci < ncand; ++ci) {
    const song2_launch &cand = all[ci];
    song2_ctx *c = new song2_ctx();
    memset((void *)&c->spec, 0, sizeof(c->spec));
    c->launch = cand;
    char lerr[SONG2_ERRLEN];
    if (ctx_setup(c, spec, tab, precision, 0, pick, k3, k3_off, k3_size, pair_off, 0, 0, 0, 0, lerr) ||
        song2_ctx_run(c, nullptr, lerr)) {
      song2_ctx_destroy(c);
      continue;
    }
    double ms = c->last_ms;
    if (ms < bestv) {
      bestv = ms;
      *best = c->launch;
      found = 1;
    }
    song2_ctx_destroy(c);
  }
  if (!found) {
    snprintf(err, SONG2_ERRLEN, "autotune: no candidate configuration ran");
    return 1;
  }
  if (best_ms) *best_ms = bestv;
  return 0;
}

int song2_ctx_destroy(song2_ctx *c) {
  if (!c) return 0;
  if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
  if (c->graph) cudaGraphDestroy(c->graph);
  if (c->cap_stream) cudaStreamDestroy(c->cap_stream);
  for (void *p : c->allocs) cudaFree(p);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  delete c;
  return 0;
}

/* the stream work of a part of a run: for every launch group, the items
   [first, first + count) of the work list, one launch each */
static int enqueue_part(song2_ctx *c, int part, cudaStream_t st, char *err) {
  int ng = c->groups.empty() ? 1 : (int)c->groups.size();
  c->last_launches = 0;
  for (int g = 0; g < ng; ++g) {
    int first = c->part_first[g * c->parts + part], count = c->part_count[g * c->parts + part];
    if (count == 0) continue;
    int grid = c->groups.empty() ? c->grid : c->groups[g].grid;
    size_t smem = c->groups.empty() ? c->smem : c->groups[g].smem;
    int per_cta = c->groups.empty() ? c->launch.teams_per_cta : 1;
    int mode = c->groups.empty() ? c->kmode : c->groups[g].mode;
    grid = std::max(1, std::min(grid, (count + per_cta - 1) / per_cta));
    DevSpec sg = c->spec;
    sg.n_items = count;
    DevPtrs pg = c->ptrs;
    pg.items = c->ptrs.items + first;
    pg.stats = c->ptrs.stats + first;
    CK(cudaMemsetAsync(c->d_queue, 0, sizeof(int), st));
    if (song2_launch_evolver(sg, pg, c->precision, mode, grid, c->block, smem, st)) {
      snprintf(err, SONG2_ERRLEN, "evolver launch failed: %s", cudaGetErrorString(cudaGetLastError()));
      return 1;
    }
    c->last_launches++;
  }
  return 0;
}

/* the stream work of one run: queue resets and the evolver launch(es) */
static int enqueue_run(song2_ctx *c, cudaStream_t st, char *err) {
  CK(cudaMemsetAsync(c->d_queue, 0, sizeof(int), st));
  if (c->groups.empty()) {
    if (song2_launch_evolver(c->spec, c->ptrs, c->precision, c->kmode, c->grid, c->block, c->smem, st)) {
      snprintf(err, SONG2_ERRLEN, "evolver launch failed: %s", cudaGetErrorString(cudaGetLastError()));
      return 1;
    }
    c->last_launches = 1;
  } else {
    for (const song2_ctx::Group &G : c->groups) {
      DevSpec sg = c->spec;
      sg.n_items = G.count;
      DevPtrs pg = c->ptrs;
      pg.items = c->ptrs.items + G.first;
      pg.stats = c->ptrs.stats + G.first;
      if (G.first > 0) CK(cudaMemsetAsync(c->d_queue, 0, sizeof(int), st));
      if (song2_launch_evolver(sg, pg, c->precision, G.mode, G.grid, c->block, G.smem, st)) {
        snprintf(err, SONG2_ERRLEN, "evolver launch failed: %s", cudaGetErrorString(cudaGetLastError()));
        return 1;
      }
    }
    c->last_launches = (int)c->groups.size();
  }
  return 0;
}

int song2_ctx_run(song2_ctx *c, void *stream, char *err) {
  cudaStream_t st = (cudaStream_t)stream;
  CK(cudaEventRecord(c->ev0, st));
  if (enqueue_run(c, st, err)) return 1;
  CK(cudaEventRecord(c->ev1, st));
  CK(cudaStreamSynchronize(st));
  CK(cudaEventElapsedTime(&c->last_ms, c->ev0, c->ev1));
  return 0;
}

static int regroup_parts(song2_ctx *c, int part, int n_parts, cudaStream_t st, char *err) {
  if (n_parts < 1 || part < 0 || part >= n_parts) {
    snprintf(err, SONG2_ERRLEN, "bad part %d of %d", part, n_parts);
    return 1;
  }
  if (c->parts != n_parts) {
    /* regroup the work list part-major within every launch group: part q takes
       every n_parts-th item of the group's cost-sorted list, from position q */
    int ng = c->groups.empty() ? 1 : (int)c->groups.size();
    std::vector<WorkItem> reo;
    reo.reserve(c->h_items.size());
    c->part_first.assign((size_t)ng * n_parts, 0);
    c->part_count.assign((size_t)ng * n_parts, 0);
    for (int g = 0; g < ng; ++g) {
      int gf = c->groups.empty() ? 0 : c->groups[g].first;
      int gc = c->groups.empty() ? c->n_items : c->groups[g].count;
      for (int q = 0; q < n_parts; ++q) {
        c->part_first[(size_t)g * n_parts + q] = (int)reo.size();
        for (int i = gf + q; i < gf + gc; i += n_parts) reo.push_back(c->h_items[i]);
        c->part_count[(size_t)g * n_parts + q] = (int)reo.size() - c->part_first[(size_t)g * n_parts + q];
      }
    }
    c->h_items = reo;
    c->parts = n_parts;
    CK(cudaMemcpyAsync((void *)c->ptrs.items, reo.data(), sizeof(WorkItem) * reo.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(c->d_stats, 0, sizeof(song2_triplet_stats) * std::max(1, c->n_items), st));
    CK(cudaStreamSynchronize(st));
  }
  return 0;
}

int song2_ctx_enqueue_part(song2_ctx *c, int part, int n_parts, void *stream, char *err) {
  cudaStream_t st = (cudaStream_t)stream;
  if (regroup_parts(c, part, n_parts, st, err)) return 1;
  return enqueue_part(c, part, st, err);
}

int song2_ctx_run_part(song2_ctx *c, int part, int n_parts, void *stream, char *err) {
  cudaStream_t st = (cudaStream_t)stream;
  if (regroup_parts(c, part, n_parts, st, err)) return 1;
  CK(cudaEventRecord(c->ev0, st));
  if (enqueue_part(c, part, st, err)) return 1;
  CK(cudaEventRecord(c->ev1, st));
  CK(cudaStreamSynchronize(st));
  CK(cudaEventElapsedTime(&c->last_ms, c->ev0, c->ev1));
  return 0;
}

int song2_ctx_run_graph(song2_ctx *c, void *stream, char *err) {
  cudaStream_t st = (cudaStream_t)stream;
  if (!c->graph_exec) {
    if (!c->cap_stream) CK(cudaStreamCreateWithFlags(&c->cap_stream, cudaStreamNonBlocking));
    CK(cudaStreamBeginCapture(c->cap_stream, cudaStreamCaptureModeThreadLocal));
    if (enqueue_run(c, c->cap_stream, err)) {
      cudaGraph_t g = nullptr;
      cudaStreamEndCapture(c->cap_stream, &g);
      if (g) cudaGraphDestroy(g);
      return 1;
    }
    CK(cudaStreamEndCapture(c->cap_stream, &c->graph));
    CK(cudaGraphInstantiate(&c->graph_exec, c->graph, 0));
  }
  CK(cudaEventRecord(c->ev0, st));
  CK(cudaGraphLaunch(c->graph_exec, st));
  CK(cudaEventRecord(c->ev1, st));
  CK(cudaStreamSynchronize(st));
  CK(cudaEventElapsedTime(&c->last_ms, c->ev0, c->ev1));
  return 0;
}

int song2_ctx_phase_cycles(song2_ctx *c, unsigned long long *out, int n) {
#ifdef SONG2_PHASE_TIMERS
  if (!c->ptrs.phase || n < 2 * S2_NPHASE) return 0;
  if (cudaMemcpy(out, c->ptrs.phase, 2 * S2_NPHASE * sizeof(unsigned long long), cudaMemcpyDeviceToHost) != cudaSuccess)
    return 0;
  return S2_NPHASE;
#else
  (void)c; (void)out; (void)n;
  return 0;
#endif
}

double *song2_ctx_device_sources(song2_ctx *c) { return c->d_sources; }
song2_triplet_stats *song2_ctx_device_stats(song2_ctx *c) { return c->d_stats; }
double song2_ctx_last_kernel_ms(song2_ctx *c) { return c->last_ms; }
int song2_ctx_last_launches(song2_ctx *c) { return c->last_launches; }

int song2_ctx_download(song2_ctx *c, double *flat, song2_triplet_stats *stats, char *err) {
  if (flat && c->sources_len) CK(cudaMemcpy(flat, c->d_sources, c->sources_len * sizeof(double), cudaMemcpyDeviceToHost));
  if (stats && c->n_items) {
    /* stats are stored per sorted work item: return them in the reference's
       work order (k1 descending, k2 <= k1, k3) */
    std::vector<song2_triplet_stats> tmp(c->n_items);
    std::vector<WorkItem> items(c->n_items);
    CK(cudaMemcpy(tmp.data(), c->d_stats, sizeof(song2_triplet_stats) * c->n_items, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(items.data(), c->ptrs.items, sizeof(WorkItem) * c->n_items, cudaMemcpyDeviceToHost));
    /* rank of (i1,i2,i3) in the reference order */
    int ksz = c->spec.k_size;
    std::vector<int64_t> k3s;
    std::vector<int> k3size(c->n_items);
    std::vector<int> h_k3size;
    /* pair sizes */
    int npairs = ksz * (ksz + 1) / 2;
    h_k3size.resize(npairs);
    CK(cudaMemcpy(h_k3size.data(), c->ptrs.k3_size, sizeof(int) * npairs, cudaMemcpyDeviceToHost));
    std::vector<int64_t> start(npairs, 0);
    int64_t acc = 0;
    for (int i1 = ksz - 1; i1 >= 0; --i1)
      for (int i2 = 0; i2 <= i1; ++i2) {
        int pr = i1 * (i1 + 1) / 2 + i2;
        start[pr] = acc;
        acc += h_k3size[pr];
      }
    for (int i = 0; i < c->n_items; ++i) stats[start[items[i].pair] + items[i].i3] = tmp[i];
  }
  return 0;
}

/* reference work-order index -> (k1, k2, k3) indices */
static void work_order_triplets(const song2_spec *spec, std::vector<int> &i1s, std::vector<int> &i2s,
                                std::vector<int> &i3s) {
  i1s.clear(); i2s.clear(); i3s.clear();
  for (int i1 = spec->k_size - 1; i1 >= 0; --i1)
    for (int i2 = 0; i2 <= i1; ++i2)
      for (int i3 = 0; i3 < spec->k3_size[i1 * spec->k_size + i2]; ++i3) {
        i1s.push_back(i1); i2s.push_back(i2); i3s.push_back(i3);
      }
}

int song2_gpu_evolve(const song2_spec *spec, const song2_tables *tab, int precision, double ****sources_out,
                     song2_triplet_stats *per_triplet, char *err) {
  song2_ctx *c = nullptr;
  if (song2_ctx_create(spec, tab, precision, &c, err)) return 1;
  int rc = song2_ctx_run(c, nullptr, err);
  std::vector<double> flat;
  int64_t nt = song2_n_triplets(spec);
  std::vector<song2_triplet_stats> stv(nt);
  if (!rc) {
    flat.resize(c->sources_len);
    rc = song2_ctx_download(c, flat.data(), stv.data(), err);
  }
  if (!rc) {
    /* exit strategy for the triplets that failed: evolve them again in plain FP64
       with a larger step budget, and take their sources and stats from that run */
    std::vector<int64_t> failed;
    for (int64_t i = 0; i < nt; ++i)
      if (stv[i].status != SONG2_OK) failed.push_back(i);
    if (!failed.empty()) {
      song2_spec rs = *spec;
      rs.max_steps = spec->max_steps > (1 << 27) ? (1 << 30) : spec->max_steps * 8;
      song2_ctx *r = nullptr;
      rc = song2_ctx_create_list(&rs, tab, SONG2_PREC_FP64, failed.data(), (int64_t)failed.size(), &r, err);
      if (!rc) rc = song2_ctx_run(r, nullptr, err);
      std::vector<double> flat2;
      std::vector<song2_triplet_stats> st2(nt);
      if (!rc) {
        flat2.resize(r->sources_len);
        rc = song2_ctx_download(r, flat2.data(), st2.data(), err);
      }
      if (!rc) {
        std::vector<int> i1s, i2s, i3s;
        work_order_triplets(spec, i1s, i2s, i3s);
        for (int64_t i : failed) {
          int nk3 = spec->k3_size[i1s[i] * spec->k_size + i2s[i]];
          int64_t off = song2_pair_offset(spec, i1s[i], i2s[i]) + i3s[i];
          for (int tp = 0; tp < c->tp2_size; ++tp)
            for (int j = 0; j < spec->tau_size; ++j) {
              size_t e = (size_t)tp * c->per_type + off + (size_t)j * nk3;
              flat[e] = flat2[e];
            }
          stv[i] = st2[i];
          stv[i].retried = 1;
        }
      }
      song2_ctx_destroy(r);
    }
  }
  if (!rc && per_triplet) memcpy(per_triplet, stv.data(), sizeof(song2_triplet_stats) * nt);
  if (!rc && sources_out) {
    for (int tp = 0; tp < c->tp2_size; ++tp)
      for (int i1 = 0; i1 < spec->k_size; ++i1)
        for (int i2 = 0; i2 <= i1; ++i2) {
          int64_t off = song2_pair_offset(spec, i1, i2);
          int64_t len = (int64_t)spec->tau_size * spec->k3_size[i1 * spec->k_size + i2];
          memcpy(sources_out[tp][i1][i2], flat.data() + (size_t)tp * c->per_type + off, sizeof(double) * len);
        }
  }
  if (!rc)
    for (int64_t i = 0; i < nt; ++i)
      if (stv[i].status != SONG2_OK) {
        snprintf(err, SONG2_ERRLEN, "triplet %lld failed with status %d, also on its plain-FP64 re-run", (long long)i,
                 stv[i].status);
        rc = 1;
        break;
      }
  song2_ctx_destroy(c);
  return rc;
}

int song2_gpu_first_order(const song2_spec *spec2, const song2_tables *bg_only, int fo_l_max, int fo_tau_size,
                          double fo_lntau0, double fo_dlntau, double *fo_out, char *err) {
  song2_spec s = *spec2;
  s.ic = SONG2_IC_AD_FIRST_ORDER;
  /* first-order normalisation: primordial curvature zeta = 1 (C = -1/2) */
  s.primordial_local_fnl_phi = 5.0 / 6.0;
  s.m_size = 1;
  s.m[0] = 0;
  s.has_quadratic_sources = 0;
  s.has_source_T = s.has_source_E = s.has_source_B = s.has_source_delta_cdm = 0;
  /* evolve more multipoles than stored, so the truncation stays away from the table */
  s.l_max_g = s.l_max_pol_g = s.l_max_ur = fo_l_max + 5;
  s.l_max_los_t = s.l_max_los_p = 0;
  /* one "triplet" (k, k, k) per k: without quadratic sources only k matters */
  std::vector<int> k3_size_full((size_t)s.k_size * s.k_size, 0);
  std::vector<WorkItem> items;
  std::vector<double> k3;
  std::vector<int> k3_off, k3_size;
  std::vector<int64_t> pair_off;
  for (int ik = 0; ik < s.k_size; ++ik) {
    items.push_back(WorkItem{ik, ik, 0, ik, 0, ik});
    k3.push_back(s.k[ik]);
    k3_off.push_back(ik);
    k3_size.push_back(1);
    pair_off.push_back(0);
  }
  std::reverse(items.begin(), items.end());
  song2_ctx *c = new song2_ctx();
  memset((void *)&c->spec, 0, sizeof(c->spec));
  song2_tables t = *bg_only;
  if (ctx_setup(c, &s, &t, SONG2_PREC_FP64, 1, items, k3, k3_off, k3_size, pair_off, fo_tau_size, fo_lntau0, fo_dlntau,
                fo_l_max, err)) {
    song2_ctx_destroy(c);
    return 1;
  }
  int rc = song2_ctx_run(c, nullptr, err);
  if (!rc) {
    cudaError_t e = cudaMemcpy(fo_out, c->d_fo_out, c->fo_out_len * sizeof(double), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) { snprintf(err, SONG2_ERRLEN, "download: %s", cudaGetErrorString(e)); rc = 1; }
  }
  if (!rc) {
    std::vector<song2_triplet_stats> st(c->n_items);
    cudaMemcpy(st.data(), c->d_stats, sizeof(song2_triplet_stats) * c->n_items, cudaMemcpyDeviceToHost);
    for (auto &x : st)
      if (x.status != SONG2_OK) {
        snprintf(err, SONG2_ERRLEN, "first-order mode failed with status %d", x.status);
        rc = 1;
        break;
      }
  }
  song2_ctx_destroy(c);
  return rc;
}

} /* extern "C" */

/* ------------------------------------------------------------ allocation-free entry */
/* Scratch of song2_gpu_evolve_noalloc: every GPU that loads this library holds
   these SONG2_NOALLOC_BYTES until the process exits.  Host code must not use the
   name as an address; the device address comes from cudaGetSymbolAddress. */
#define SONG2_NOALLOC_BYTES ((size_t)64 << 20)
static __device__ __align__(256) unsigned char song2_noalloc_scratch[SONG2_NOALLOC_BYTES];

#define SONG2_NOALLOC_MAX_DEVICES 64
static void *g_noalloc_addr[SONG2_NOALLOC_MAX_DEVICES];
static std::mutex g_noalloc_mutex;   /* guards the lazy resolve of g_noalloc_addr */

static size_t na_align(size_t x) { return (x + 255) & ~(size_t)255; }

extern "C" int song2_gpu_evolve_noalloc(const song2_spec *spec, const song2_tables *tab_dev, int precision,
                                        double *sources_dev, song2_triplet_stats *stats_dev, void *stream,
                                        char *err) {
  if (precision != SONG2_PREC_FP64 && precision != SONG2_PREC_MIXED) {
    snprintf(err, SONG2_ERRLEN, "unknown precision %d", precision);
    return 1;
  }
  if (!sources_dev || !stats_dev) {
    snprintf(err, SONG2_ERRLEN, "sources_dev and stats_dev must be device buffers");
    return 1;
  }
  int dev = 0;
  CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= SONG2_NOALLOC_MAX_DEVICES) {
    snprintf(err, SONG2_ERRLEN, "device %d beyond the %d supported", dev, SONG2_NOALLOC_MAX_DEVICES);
    return 1;
  }
  /* first call on this device (which must be current): resolve the scratch address */
  char *base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_addr[dev]) {
      void *ptr = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&ptr, song2_noalloc_scratch);
      if (e != cudaSuccess || !ptr) {
        snprintf(err, SONG2_ERRLEN, "cudaGetSymbolAddress of the scratch failed: %s", cudaGetErrorString(e));
        return 1;
      }
      g_noalloc_addr[dev] = ptr;
    }
    base = (char *)g_noalloc_addr[dev];
  }
  cudaStream_t st = (cudaStream_t)stream;

  if (spec->n_classes > 0) {
    snprintf(err, SONG2_ERRLEN, "hierarchy classes are not supported by the allocation-free entry");
    return 1;
  }
  HostLayout H;
  if (build_layout(spec, tab_dev, 0, H, err)) return 1;
  DevSpec s = H.s;
  std::vector<int> k3_off, k3_size;
  std::vector<int64_t> pair_off;
  pair_tables(spec, k3_off, k3_size, pair_off);
  int n3tot = k3_off.empty() ? 0 : k3_off.back() + k3_size.back();
  std::vector<double> k3(spec->k3, spec->k3 + n3tot);
  std::vector<WorkItem> items;
  std::vector<int64_t> ref;
  sorted_items(spec, k3, k3_off, k3_size, items, ref);
  s.n_items = (int)items.size();
  s.per_type = song2_sources_per_type(spec);

  /* carve the scratch: small tables first, then the per-team Jacobian blocks */
  size_t off = 0;
  auto take = [&](size_t bytes) { size_t o = off; off = na_align(off + std::max<size_t>(bytes, 1)); return o; };
  size_t o_k = take(sizeof(double) * spec->k_size), o_k3 = take(sizeof(double) * k3.size());
  size_t o_tau = take(sizeof(double) * spec->tau_size);
  size_t o_k3off = take(sizeof(int) * k3_off.size()), o_k3sz = take(sizeof(int) * k3_size.size());
  size_t o_poff = take(sizeof(int64_t) * pair_off.size());
  size_t nc = H.cmin.size() * sizeof(double);
  size_t o_cm = take(nc), o_cp = take(nc), o_dm = take(nc), o_dp = take(nc), o_dz = take(nc);
  size_t ne = sizeof(short) * H.eq_sp.size(), ni = sizeof(short) * H.idx_I.size(), nq = sizeof(short) * H.qs_sp.size();
  size_t o_esp = take(ne), o_el = take(ne), o_em = take(ne);
  size_t o_iI = take(ni), o_iE = take(ni), o_iB = take(ni), o_iN = take(ni);
  size_t o_qsp = take(nq), o_ql = take(nq), o_qm = take(nq);
  size_t nrs = sizeof(short) * H.row_slot.size(), nqs = sizeof(short) * H.qs_slot.size();
  size_t o_rsl = take(nrs), o_qsl = take(nqs);
  size_t nmx = sizeof(short) * H.mx_idx.size(), nqo = sizeof(short) * H.qo_slot.size();
  size_t o_mxi = take(nmx), o_mxp = take(nmx), o_qo = take(nqo);
  size_t ngen = sizeof(GenRow) * H.gen.size();
  size_t o_gen = take(ngen);
  size_t o_items = take(sizeof(WorkItem) * items.size());
  size_t o_queue = take(sizeof(int));
  std::vector<double> cs(std::max(2, s.fo_tau_size + 1), 0.0);
  for (size_t j = 1; j < cs.size(); ++j) cs[j] = 1.0 / (4.0 - cs[j - 1]);
  size_t o_splc = take(sizeof(double) * cs.size());
  std::vector<double> dtc = dt_table(s);
  size_t o_dt = take(sizeof(double) * dtc.size());
  size_t fixed = off;
  if (fixed > SONG2_NOALLOC_BYTES) {
    snprintf(err, SONG2_ERRLEN, "problem tables need %zu B, more than the %zu B scratch", fixed,
             (size_t)SONG2_NOALLOC_BYTES);
    return 1;
  }
  int nsm = 0, smem_optin = 0;
  CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  CK(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  int block = 256;
  s.lu_in_smem = song2_smem_bytes(s, precision, block, 1) <= (size_t)smem_optin ? 1 : 0;
  size_t smem = song2_smem_bytes(s, precision, block, s.lu_in_smem);
  if (smem > (size_t)smem_optin) {
    snprintf(err, SONG2_ERRLEN, "shared-memory plan %zu B exceeds the %d B limit", smem, smem_optin);
    return 1;
  }
  size_t ts = precision == SONG2_PREC_MIXED ? sizeof(float) : sizeof(double);
  size_t qtab_team = s.has_qs ? (size_t)s.fo_tau_size * 2 * s.qs2_size * sizeof(double) : 0;
  size_t per_team = na_align((size_t)s.lu_elems * sizeof(double)) + (s.lu_in_smem ? 0 : na_align((size_t)s.lu_elems * ts)) +
                    na_align(qtab_team);
  size_t teams_fit = (SONG2_NOALLOC_BYTES - fixed) / per_team;
  if (teams_fit < 1) {
    snprintf(err, SONG2_ERRLEN, "per-triplet scratch of %zu B (iteration matrices, source table) does not fit in the %zu B scratch",
             per_team, (size_t)SONG2_NOALLOC_BYTES - fixed);
    return 1;
  }
  int per_sm = song2_max_ctas_per_sm(precision, 0, block, smem);
  if (per_sm < 1) {
    snprintf(err, SONG2_ERRLEN, "launch configuration does not fit on an SM");
    return 1;
  }
  int grid = std::max(1, std::min(s.n_items, nsm * per_sm));
  grid = (int)std::min<size_t>((size_t)grid, teams_fit);
  size_t o_jac = take((size_t)grid * s.lu_elems * sizeof(double));
  size_t o_lu = s.lu_in_smem ? 0 : take((size_t)grid * s.lu_elems * ts);
  size_t o_qtab = s.has_qs ? take((size_t)grid * qtab_team) : 0;
  if (off > SONG2_NOALLOC_BYTES) {
    snprintf(err, SONG2_ERRLEN, "scratch plan of %zu B exceeds the %zu B scratch", off, (size_t)SONG2_NOALLOC_BYTES);
    return 1;
  }

  auto put = [&](size_t o, const void *src, size_t bytes) -> cudaError_t {
    return bytes ? cudaMemcpyAsync(base + o, src, bytes, cudaMemcpyHostToDevice, st) : cudaSuccess;
  };
  CK(put(o_k, spec->k, sizeof(double) * spec->k_size));
  CK(put(o_k3, k3.data(), sizeof(double) * k3.size()));
  CK(put(o_tau, spec->tau, sizeof(double) * spec->tau_size));
  CK(put(o_k3off, k3_off.data(), sizeof(int) * k3_off.size()));
  CK(put(o_k3sz, k3_size.data(), sizeof(int) * k3_size.size()));
  CK(put(o_poff, pair_off.data(), sizeof(int64_t) * pair_off.size()));
  CK(put(o_cm, H.cmin.data(), nc)); CK(put(o_cp, H.cplu.data(), nc)); CK(put(o_dm, H.dmin.data(), nc));
  CK(put(o_dp, H.dplu.data(), nc)); CK(put(o_dz, H.dzer.data(), nc));
  CK(put(o_esp, H.eq_sp.data(), ne)); CK(put(o_el, H.eq_l.data(), ne)); CK(put(o_em, H.eq_m.data(), ne));
  CK(put(o_iI, H.idx_I.data(), ni)); CK(put(o_iE, H.idx_E.data(), ni)); CK(put(o_iB, H.idx_B.data(), ni));
  CK(put(o_iN, H.idx_N.data(), ni));
  CK(put(o_qsp, H.qs_sp.data(), nq)); CK(put(o_ql, H.qs_l.data(), nq)); CK(put(o_qm, H.qs_m.data(), nq));
  CK(put(o_rsl, H.row_slot.data(), nrs)); CK(put(o_qsl, H.qs_slot.data(), nqs));
  CK(put(o_mxi, H.mx_idx.data(), nmx)); CK(put(o_mxp, H.mx_pos.data(), nmx)); CK(put(o_qo, H.qo_slot.data(), nqo));
  CK(put(o_gen, H.gen.data(), ngen));
  CK(put(o_items, items.data(), sizeof(WorkItem) * items.size()));
  CK(put(o_splc, cs.data(), sizeof(double) * cs.size()));
  CK(put(o_dt, dtc.data(), sizeof(double) * dtc.size()));
  /* the scratch keeps the previous call's contents: the work-queue counter and the
     outputs (entries the sources never write, e.g. E with l < 2) must start at zero */
  CK(cudaMemsetAsync(base + o_queue, 0, sizeof(int), st));
  CK(cudaMemsetAsync(sources_dev, 0, sizeof(double) * (size_t)s.tp2_size * s.per_type, st));

  DevPtrs p;
  memset(&p, 0, sizeof(p));
  p.k = (const double *)(base + o_k);
  p.k3 = (const double *)(base + o_k3);
  p.tau = (const double *)(base + o_tau);
  p.k3_off = (const int *)(base + o_k3off);
  p.k3_size = (const int *)(base + o_k3sz);
  p.pair_off = (const int64_t *)(base + o_poff);
  p.bg = tab_dev->bg; p.bg_dd = tab_dev->bg_dd; p.fo = tab_dev->fo; p.fo_dd = tab_dev->fo_dd;
  p.tabs.cmin = (const double *)(base + o_cm); p.tabs.cplu = (const double *)(base + o_cp);
  p.tabs.dmin = (const double *)(base + o_dm); p.tabs.dplu = (const double *)(base + o_dp);
  p.tabs.dzer = (const double *)(base + o_dz);
  p.tabs.eq_sp = (const short *)(base + o_esp); p.tabs.eq_l = (const short *)(base + o_el); p.tabs.eq_m = (const short *)(base + o_em);
  p.tabs.idx_I = (const short *)(base + o_iI); p.tabs.idx_E = (const short *)(base + o_iE);
  p.tabs.idx_B = (const short *)(base + o_iB); p.tabs.idx_N = (const short *)(base + o_iN);
  p.tabs.qs_sp = (const short *)(base + o_qsp); p.tabs.qs_l = (const short *)(base + o_ql); p.tabs.qs_m = (const short *)(base + o_qm);
  p.tabs.row_slot = (const short *)(base + o_rsl); p.tabs.qs_slot = (const short *)(base + o_qsl);
  p.tabs.mx_idx = (const short *)(base + o_mxi); p.tabs.mx_pos = (const short *)(base + o_mxp);
  p.tabs.qo_slot = (const short *)(base + o_qo);
  p.tabs.gen = (const GenRow *)(base + o_gen);
  p.items = (const WorkItem *)(base + o_items);
  p.sources = sources_dev;
  p.stats = stats_dev;
  p.stats_by_ref = 1;
  p.jac = (double *)(base + o_jac);
  p.lu_global = s.lu_in_smem ? nullptr : (void *)(base + o_lu);
  p.qtab = s.has_qs ? (double *)(base + o_qtab) : nullptr;
  p.spl_c = (const double *)(base + o_splc);
  p.dt_coup = s.dtilde ? (const double *)(base + o_dt) : nullptr;
  p.queue = (int *)(base + o_queue);
  if (song2_launch_evolver(s, p, precision, 0, grid, block, smem, st)) {
    snprintf(err, SONG2_ERRLEN, "evolver launch failed: %s", cudaGetErrorString(cudaGetLastError()));
    return 1;
  }
  return 0;
}
