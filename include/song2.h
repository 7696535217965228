/*
 * song2.h - C ABI of the GB300 second-order perturbation evolver.
 *
 * This header is the drop-in boundary that replaces the "Solve differential
 * system" block of SONG's perturb2_init (source/perturbations2.c:283-362),
 * i.e. the OpenMP loop that calls perturb2_solve() for every (k1,k2,k3)
 * triplet and fills ppt2->sources.  Every entry point takes plain C types:
 * pointers, sizes and flat arrays; no torch or CUDA type appears here.
 *
 * Output layout (unchanged from the reference, include/perturbations2.h:397-414
 * and include/perturbations2_macros.h:35-38):
 *
 *   sources[index_tp2][index_k1][index_k2][index_tau*k3_size[k1][k2] + index_k3]
 *
 * with index_k2 <= index_k1.  The flat device/host buffer used internally stores
 * the same rows back to back: for each tp2, pairs (k1,k2<=k1) in row-major order,
 * each pair a block of tau_size*k3_size doubles (see song2_pair_offset()).
 *
 * Error convention (perturbations2.h:1802-1814): 0 on success, 1 on failure
 * with a message in the caller's char[SONG2_ERRLEN] buffer; nothing aborts.
 */
#ifndef SONG2_H
#define SONG2_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SONG2_ERRLEN 1024
#define SONG2_MAX_M 5          /* azimuthal modes m = 0..4 */
#define SONG2_MAX_L 64         /* largest hierarchy l_max supported */

/* Per-triplet status codes.  A triplet that breaches an iteration limit
   retires with one of these codes; no kernel traps or hangs. */
enum song2_status_code {
  SONG2_OK = 0,
  SONG2_E_MAXSTEPS = 1,   /* more than spec.max_steps accepted+rejected steps */
  SONG2_E_HMIN = 2,       /* step size fell below the minimum */
  SONG2_E_NAN = 3,        /* non-finite value in the state or the sources */
  SONG2_E_NEWTON = 4,     /* Newton iteration failed with a current Jacobian at h_min */
  SONG2_E_SINGULAR = 5,   /* zero pivot in the iteration matrix */
  SONG2_E_CONFIG = 6      /* geometry or configuration check failed */
};

/* Initial conditions (source/input2.c:2116-2121, perturbations2.c:3789-4210) */
enum song2_ic { SONG2_IC_AD = 0, SONG2_IC_AD_FIRST_ORDER = 1, SONG2_IC_ZERO = 2 };

/* Iteration-matrix precision of the GPU evolver */
enum song2_precision { SONG2_PREC_FP64 = 0, SONG2_PREC_MIXED = 1 };

/* Background/thermodynamics table columns.  Values are tabulated on a uniform
   grid in x = ln(tau) and interpolated with a natural cubic spline in x.
   Densities follow CLASS units (8 pi G/3 rho, Mpc^-2). */
enum song2_bg_column {
  SONG2_BG_LN_A = 0,        /* ln a */
  SONG2_BG_LN_HC,           /* ln (a H), conformal Hubble rate [1/Mpc] */
  SONG2_BG_HC_PRIME_TAU2,   /* (d(aH)/dtau) * tau^2 */
  SONG2_BG_LN_RHO_G,        /* ln rho_photon */
  SONG2_BG_LN_RHO_B,        /* ln rho_baryon */
  SONG2_BG_LN_RHO_CDM,      /* ln rho_cdm */
  SONG2_BG_LN_RHO_UR,       /* ln rho_massless_neutrinos */
  SONG2_BG_LN_KAPPA_DOT,    /* ln (a n_e sigma_T) [1/Mpc] */
  SONG2_BG_KAPPA,           /* optical depth from tau to today */
  SONG2_BG_SIZE
};

/* First-order quantity layout (the replacement for CLASS's ppt->index_qs_*,
   perturbations2.c:3782-3822, 9173-9332, 10794-10923).  The multipole blocks
   start at SONG2_FO_I etc. and hold l = 0..fo_l_max. */
enum song2_fo_index {
  SONG2_FO_PHI = 0, SONG2_FO_PSI, SONG2_FO_PHI_P, SONG2_FO_PSI_P, SONG2_FO_PHI_PP,
  SONG2_FO_DELTA_G, SONG2_FO_V_G,
  SONG2_FO_DELTA_B, SONG2_FO_V_B, SONG2_FO_DELTA_B_P, SONG2_FO_V_B_P,
  SONG2_FO_DELTA_CDM, SONG2_FO_V_CDM, SONG2_FO_V_CDM_P,
  SONG2_FO_DELTA_UR, SONG2_FO_V_UR,
  SONG2_FO_DIPOLE_B, SONG2_FO_DIPOLE_CDM,
  SONG2_FO_I  /* first multipole block; E, N follow, see song2_fo_size() */
};

/* Cosmological parameters of the flat LCDM background.  z_reio > 0 adds
   reionisation in the form of CLASS's reio_camb: hydrogen and helium's first
   ionisation by a tanh in (1+z)^{3/2} of width 0.5 in z centred on z_reio,
   helium's second by a tanh of width 0.5 at z = 3.5; z_reio = 0: none. */
typedef struct {
  double h, omega_b, omega_cdm, N_eff, T_cmb, YHe;
  double z_reio;
} song2_cosmo;

/* Problem specification: the hot-path subset of SONG's precision2/perturbs2
   (include/common2.h:24-214, source/input2.c:2027-2371). */
typedef struct {
  /* hierarchies (ppr2->l_max_g, l_max_pol_g, l_max_ur) */
  int l_max_g, l_max_pol_g, l_max_ur;
  int l_max_los_t, l_max_los_p;            /* LOS source multipoles */
  int m_size;                              /* modes_song */
  int m[SONG2_MAX_M];                      /* ascending */
  /* physics switches (input2.c:2059-2121) */
  int has_polarization2;
  int has_quadratic_sources, has_quadratic_liouville, has_quadratic_collision;
  int tight_coupling;                      /* 0: tca2_none, 1: tca2_first_order_pitrou */
  double tca_trigger_tau_c_over_tau_h;     /* 0.01 */
  double tca_trigger_tau_c_over_tau_k;     /* 0.007 */
  int ic;                                  /* enum song2_ic */
  double primordial_local_fnl_phi;
  /* line-of-sight source switches (input2.c:619-690) */
  int has_pure_scattering_in_los, has_quad_scattering_in_los;
  int has_pure_metric_in_los, has_quad_metric_in_los;
  int has_time_delay_in_los, has_redshift_in_los, has_lensing_in_los;
  int has_sw, has_isw, use_exponential_potentials;
  int has_source_T, has_source_E, has_source_B, has_source_delta_cdm;
  /* integrator (tol_perturb_integration_song, smallest variation) */
  double rtol;                             /* relative tolerance */
  double threshold;                        /* absolute floor of the error weights */
  int max_steps;                           /* per triplet (steps + rejections) */
  double start_small_k_at_tau_c_over_tau_h;/* 0.0015 */
  double start_large_k_at_tau_h_over_tau_k;/* 0.07 */
  double tol_tau_approx;                   /* relative bisection tolerance */
  /* grids (ppt2->k, k3, tau_sampling) */
  int k_size;
  const double *k;                         /* [k_size] ascending */
  const int *k3_size;                      /* [k_size*k_size]; entry i1*k_size+i2 for i2<=i1 */
  const double *k3;                        /* concatenated k3 grids of the pairs, pair order */
  int tau_size;
  const double *tau;                       /* [tau_size] ascending */
  /* Uneven batches (no counterpart in the reference, whose hierarchy sizes are
     run-wide).  n_classes > 0 gives every triplet a class; triplets are numbered
     in pair order (k1 ascending, k2 <= k1, k3 ascending: the order of the
     concatenated k3 grids).  A class sets l_max of the photon intensity,
     polarisation and neutrino hierarchies and evolves the modes m = 0..m_max.
     The run-wide l_max and mode list above must cover every class: they fix the
     source types (a class's sources for modes it does not evolve are zero) and
     the first-order tables.  n_classes = 0: every triplet uses the run-wide
     hierarchy. */
  int n_classes;
  const int *class_l_max;                  /* [n_classes] */
  const int *class_m_max;                  /* [n_classes] */
  const int *triplet_class;                /* [n_triplets], pair order */
  /* delta-tilde line-of-sight sources (use_delta_tilde_in_los, input2.c:680-683;
     incompatible with has_redshift_in_los, input2.c:742-744): the T, E, B sources
     gain -2 kappa' (delta*delta/2 + delta*collision), perturbations2.c:12339-12398,
     12509-12561, 12658-12710, summed over first-order multipoles
     l1, l2 <= l_max_los_quadratic_t (T) or l_max_los_quadratic_p (E, B);
     input2.c:1788-1789, defaults 2 (input2.c:2265-2266). */
  int use_delta_tilde_in_los;
  int l_max_los_quadratic_t, l_max_los_quadratic_p;
  /* rotation coefficients divided by sin(theta_k1)^m (ppt2->rescale_cmb_sources,
     perturbations2.c:5635-5652; on in the reference's bispectrum runs with m > 0,
     input2.c:1962-1971): every m-multipole of the second-order solution and of the
     sources is multiplied by sin(theta_k1)^-m. */
  int rescale_cmb_sources;
  /* radiation-streaming approximation (radiation_streaming_approximation_song,
     input2.c:824-829; reference default rsa2_MD with triggers 90 and 10,
     input2.c:2139-2141; the precision files shipped in pre/ use MD_with_reio
     with triggers 45 and 5): SONG2_RSA_NONE, SONG2_RSA_MD or
     SONG2_RSA_MD_WITH_REIO, which adds the first-order collision terms in tau_c
     (perturbations2.c:9929-9953, 10064-10084).  After photon
     decoupling (tau > tables.tau_free_streaming) and once k tau exceeds
     radiation_streaming_trigger_tau_over_tau_k, the photon and neutrino
     hierarchies are no longer evolved and their monopoles and dipoles follow the
     algebraic RSA solution (perturbations2.c:5309-5321, 6778-6796, 8777-8809,
     9773-10164). */
  int radiation_streaming_approximation;
  double radiation_streaming_trigger_tau_over_tau_k;
} song2_spec;

enum { SONG2_RSA_NONE = 0, SONG2_RSA_MD = 1, SONG2_RSA_MD_WITH_REIO = 2 };

/* Background/thermo and first-order interpolation tables, owned by the caller
   (the replacement for CLASS's pba/pth/ppt->quadsources). */
typedef struct {
  double tau0;                             /* conformal age [Mpc] */
  double a_eq;                             /* scale factor at equality */
  int bg_size;                             /* number of ln tau nodes */
  double bg_lntau0, bg_dlntau;             /* uniform grid */
  const double *bg;                        /* [bg_size][SONG2_BG_SIZE] values */
  const double *bg_dd;                     /* [bg_size][SONG2_BG_SIZE] spline d2/dx2 */
  int fo_k_size;                           /* must equal spec.k_size (same k nodes) */
  int fo_tau_size;
  double fo_lntau0, fo_dlntau;             /* uniform ln tau grid of the first-order table */
  int fo_l_max;                            /* multipoles stored: l = 0..fo_l_max */
  int fo_size;                             /* quantities per node = song2_fo_size(fo_l_max) */
  const double *fo;                        /* [k][tau][q] values */
  const double *fo_dd;                     /* [k][tau][q] spline d2/dx2 */
  /* start of photon free streaming (CLASS pth->tau_free_streaming): the time
     after recombination at which tau_c/tau exceeds
     radiation_streaming_trigger_tau_c_over_tau; needed by the RSA only, see
     song2_free_streaming_time() */
  double tau_free_streaming;
} song2_tables;

/* Per-triplet diagnostics (the reference's per-workspace counters,
   perturbations2.h:1594-1602). */
typedef struct {
  int32_t status;
  int32_t n_steps, n_rejected, n_rhs, n_jac, n_lu, n_newton_fail, sources_calls;
  int32_t retried;        /* song2_gpu_evolve: the triplet failed its first pass and was
                             re-run in plain FP64 (the counters are the re-run's) */
} song2_triplet_stats;

typedef struct song2_ctx song2_ctx;

/* Launch configuration of the persistent evolver.  A "team" evolves one
   triplet: one CTA of threads_per_team threads (warp_team = 0), one warp
   (warp_team = 1, teams_per_cta warps per CTA), or threads_per_team lanes of a
   warp (warp_team = 2: 1, 2, 4, ... 32 lanes, the 32/threads_per_team teams of a
   warp interleaved in global memory so that they advance side by side;
   teams_per_cta is rounded to whole warps, at most four).  lu_in_smem keeps the
   iteration-matrix blocks in shared memory instead of a global scratch (modes 0
   and 1).  Zeros everywhere mean "choose automatically". */
typedef struct {
  int warp_team;
  int teams_per_cta;
  int threads_per_team;
  int lu_in_smem;
} song2_launch;

/* ---------------------------------------------------------------- host side */

/* Number of first-order quantities per node for a given stored l_max. */
int song2_fo_size(int fo_l_max);
/* Total number of triplets and of source types for a spec. */
int64_t song2_n_triplets(const song2_spec *spec);
int song2_tp2_size(const song2_spec *spec);
/* Offset (in doubles, within one source type) of the (k1,k2) block of the flat
   source buffer, and the length of one source type. */
int64_t song2_pair_offset(const song2_spec *spec, int index_k1, int index_k2);
int64_t song2_sources_per_type(const song2_spec *spec);
/* The reference's raw source files (store_sources = yes): <dir>/sources_%03d.dat
   holds, for one k1, every source type and every k2 <= k1 the tau_size*k3_size
   doubles of ppt2->sources[tp][k1][k2] in native byte order, no header.  Writes /
   reads the k1 slab of the flat buffer.  Replace perturb2_store_sources_to_disk
   (perturbations2.c:15347-15387, with perturb2_store_sources_k3_tau :15397-15419,
   path :1062) and perturb2_load_sources_from_disk (:521-563, with
   perturb2_load_sources_k3_tau :575-602), so transfer2 reads the files unchanged. */
int song2_store_sources(const song2_spec *spec, const double *flat, const char *dir, int index_k1, char *err);
int song2_load_sources(const song2_spec *spec, double *flat, const char *dir, int index_k1, char *err);
/* Self-describing source files in the layout of perturb2_output
   (perturbations2.c:14688-15340) that the reference's python/songy.py reads:
   song2_write_sources_k writes the sources of one (k1, k2 <= k1) pair as a
   function of (k3, tau) with the pair's grids, the scale factor and Hubble rate
   at every source time and the first-order quantities of k1 and k2 (songy
   Fixedk1k2File, the reference's sources_song_k%03d.dat); song2_write_sources_tau
   writes every triplet's sources at source time index_tau with the k and k3
   grids and the first-order quantities of every k (songy FixedTauFile, the
   reference's sources_song_tau%03d.dat).  An ASCII header (file type on the
   first line, then a block map) precedes the binary blocks.  The tables must
   hold the first-order quantities. */
int song2_write_sources_k(const song2_spec *spec, const song2_tables *tab, const double *flat, int index_k1,
                          int index_k2, const char *path, char *err);
int song2_write_sources_tau(const song2_spec *spec, const song2_tables *tab, const double *flat, int index_tau,
                            const char *path, char *err);
/* Default spec values from source/input2.c:2027-2371 (pointers left NULL). */
void song2_spec_defaults(song2_spec *spec);

/* Background + recombination of a flat LCDM model on a uniform ln(tau) grid
   (replaces CLASS background_init/thermodynamics_init, called at
   main/song.c:55-60).  bg and bg_dd must hold bg_size*SONG2_BG_SIZE doubles. */
int song2_background_compute(const song2_cosmo *cosmo, int bg_size,
                             double *bg, double *bg_dd,
                             double *lntau0, double *dlntau,
                             double *tau0, double *a_eq, char *err);

/* Table providers: the adapter from the caller's own first-order and background
   modules (CLASS in the reference) to song2_tables.

   A first-order provider has the shape of CLASS's perturb_song_sources_at_tau_and_k
   as the reference calls it (perturbations2.c:9133-9163, 10217-10248,
   10727-10762): it writes the first-order quantities of wavenumber k =
   spec->k[index_k] at conformal time tau into out[0 .. n_provided - 1] in its own
   order (CLASS: ppt->index_qs_*), interpolating its own time sampling
   (ppt->tau_sampling_quadsources) as it does for the reference, and returns 0 on
   success.  song2_first_order_from_provider samples it on the uniform ln(tau)
   grid of fo_tau_size nodes from fo_lntau0 (step fo_dlntau), stores out[qs_map[q]]
   as quantity q of enum song2_fo_index (qs_map has song2_fo_size(fo_l_max)
   entries; -1 stores zero, for quantities the run never reads), computes the
   spline second derivatives, and points tab's first-order fields at fo_out and
   fo_dd_out (k_size * fo_tau_size * song2_fo_size(fo_l_max) doubles each).  For
   CLASS, the map sends SONG2_FO_PHI to ppt->index_qs_phi, SONG2_FO_I + l to
   ppt->index_qs_monopole_g + l, and so on; the grid should reach from before the
   earliest start time (song2_start_time at the largest k) to tau0 with a step of
   about 0.01 in ln tau.

   A background provider writes the SONG2_BG_SIZE columns of enum song2_bg_column
   at conformal time tau (from CLASS: background_at_tau and thermodynamics_at_z;
   ln a, ln of the conformal Hubble rate a H, (aH)' tau^2, the logarithms of the
   densities in CLASS units, ln kappa', and kappa = -ln(exp_m_kappa)).
   song2_background_from_provider samples it on bg_size nodes uniform in ln tau
   and points tab's background fields at bg_out and bg_dd_out
   (bg_size * SONG2_BG_SIZE doubles each); the caller sets tab->tau0, a_eq and
   tau_free_streaming.  Both return 0, or 1 with a message. */
typedef int (*song2_fo_provider)(void *user, int index_k, double k, double tau, double *out);
typedef int (*song2_bg_provider)(void *user, double tau, double *columns);
int song2_first_order_from_provider(const song2_spec *spec, int fo_l_max, int fo_tau_size, double fo_lntau0,
                                    double fo_dlntau, song2_fo_provider provider, void *user, int n_provided,
                                    const int *qs_map, double *fo_out, double *fo_dd_out, song2_tables *tab,
                                    char *err);
int song2_background_from_provider(int bg_size, double bg_lntau0, double bg_dlntau, song2_bg_provider provider,
                                   void *user, double *bg_out, double *bg_dd_out, song2_tables *tab, char *err);

/* Natural cubic spline second derivatives in x on a uniform grid, column-wise:
   y[n][ncol] -> dd[n][ncol]. */
void song2_spline_uniform(int n, int ncol, double dx, const double *y, double *dd);

/* Coupling coefficients C and D (perturbations2.c:1236-1271) of one (l,m1,m),
   closed forms derived from Clebsch-Gordan coefficients. */
double song2_coupling_c_minus(int l, int m1, int m);
double song2_coupling_c_plus(int l, int m1, int m);
double song2_coupling_d_minus(int l, int m1, int m);
double song2_coupling_d_plus(int l, int m1, int m);
double song2_coupling_d_zero(int l, int m1, int m);

/* Conformal time at which tau_c/tau = 1/(kappa' tau) first exceeds trigger
   (radiation_streaming_trigger_tau_c_over_tau, 10 by default, input2.c:2141)
   on the background table of tab (bisection in ln tau; without reionisation
   tau_c/tau - trigger changes sign once).  Returns tab->tau0 if it never does. */
double song2_free_streaming_time(const song2_tables *tab, double trigger);

/* Coupling coefficient of the delta-tilde sources, the value the reference stores
   in ppt2->coupling_coefficients[index_pf][lm(l,m)][l1][m1+l1_max][l2]
   (perturbations2.c:1285-1527): field 0 (T, spin F = 0, prefactor 1/2),
   1 (E) or 2 (B) (F = 2, prefactor 1), with m2 = m - m1 and L = l - l1 - l2,
     prefactor * i^L (T, E; L even) or i^(L-1) (B; L odd)
       * (-1)^m (2l+1) (l1 l2 l; 0 F -F) (l1 l2 l; m1 m2 -m),
   zero for the other parity and for l2 < F or l < F. */
double song2_delta_tilde_coupling(int field, int l, int m, int l1, int m1, int l2);

/* Grids: lin/log k sampling (sources2_k_sampling = lin/log), per-pair k3 grids
   with the reference's clipping (sources2_k3_sampling = lin/log), custom tau
   sampling (custom_time_sampling_song_sources).  k3_size_out has k_size*k_size
   entries; k3_out receives the concatenated grids in pair order and may be NULL
   to query the sizes. */
int song2_k_grid(int log_sampling, double k_min, double k_max, int k_size, double *k_out);
int song2_k3_grids(const double *k, int k_size, int k3_size, int log_sampling, int *k3_size_out,
                   double *k3_out, char *err);
int song2_tau_grid(int log_sampling, double tau_ini, double tau_end, int tau_size, double *out);

/* Evolution start time for wavenumber k (perturbations2.c:3388-3524). */
int song2_start_time(const song2_spec *spec, const song2_tables *tab, double k,
                     double tau_upper, double *tau_ini, char *err);

/* Sharding over ranks (one GPU per rank, triplets are independent: no data
   exchange).  Triplets are ordered by decreasing cost estimate max(k1,k2,k3)
   and dealt round-robin, so every shard gets a similar mix.  Writes the
   reference work-order indices of shard `shard` (k1 descending, k2 <= k1, k3)
   into out (may be NULL) and returns their number.  Replaces nothing in the
   reference, whose OpenMP loop shares one node (perturbations2.c:291-333). */
int64_t song2_shard_items(const song2_spec *spec, int shard, int n_shards, int64_t *out);

/* ---------------------------------------------------------------- GPU side */

/* Create a context on the current CUDA device: uploads the spec grids and the
   tables once to a device arena (cudaMemcpyAsync).  Not thread safe per ctx. */
int song2_ctx_create(const song2_spec *spec, const song2_tables *tab,
                     int precision, song2_ctx **out, char *err);
/* Same with an explicit launch configuration (NULL = automatic) and shard. */
int song2_ctx_create_ex(const song2_spec *spec, const song2_tables *tab, int precision,
                        const song2_launch *launch, int shard, int n_shards, song2_ctx **out, char *err);
/* The launch configuration a context uses. */
void song2_ctx_get_launch(song2_ctx *ctx, song2_launch *out, int *grid, int *block, size_t *smem);
/* Autotuner: times every candidate launch configuration (CTA teams of 128, 192
   or 256 threads, warp teams, lane teams; CTA teams only for uneven batches) on
   `sample` triplets spread over the cost-sorted work list and returns the
   fastest, with its time on the sample. */
int song2_autotune(const song2_spec *spec, const song2_tables *tab, int precision, int sample,
                   song2_launch *best, double *best_ms, char *err);
/* Same, restricted to the given triplets (indices in the reference work order:
   k1 descending, k2 <= k1, k3 ascending); spec may differ from the run's in its
   integrator fields (rtol, max_steps).  The flat source buffer keeps the full
   layout; the entries of the other triplets stay 0.  No counterpart in the
   reference (its re-runs go through what_if_ndf15_fails, perturbations2.c:12877-12957). */
int song2_ctx_create_list(const song2_spec *spec, const song2_tables *tab, int precision, const int64_t *items,
                          int64_t n_items, song2_ctx **out, char *err);
/* Same, restricted to the triplets of song2_shard_items(spec, shard, n_shards);
   the flat source buffer keeps the full layout, entries of other shards stay 0. */
int song2_ctx_create_shard(const song2_spec *spec, const song2_tables *tab, int precision,
                           int shard, int n_shards, song2_ctx **out, char *err);
int song2_ctx_destroy(song2_ctx *ctx);

/* Evolve every triplet on the device and leave the sources in device memory.
   stream may be NULL (legacy default stream).  Blocking on return. */
int song2_ctx_run(song2_ctx *ctx, void *stream, char *err);
/* Evolve only part `part` of n_parts of the context's triplets: every launch
   group's cost-sorted work list is dealt round-robin into n_parts parts, so the
   parts carry similar work.  The sources of the part's triplets are written into
   the context's flat buffer (the other entries keep their values), so n_parts
   calls with part = 0..n_parts-1 fill the whole buffer.  The first call with a
   new n_parts regroups the device work list and clears the per-triplet stats.
   Blocking on return; song2_ctx_last_kernel_ms() gives the part's device time.
   No counterpart in the reference (its OpenMP loop runs every triplet at once). */
int song2_ctx_run_part(song2_ctx *ctx, int part, int n_parts, void *stream, char *err);
/* As song2_ctx_run_part without waiting: the part's launches are enqueued on
   `stream` and the call returns (the first call with a new n_parts regroups the
   work list first, blocking).  Parts of one context must not run concurrently
   (they share the context's scratch); parts of two contexts may, on two streams,
   so that one part's last triplets overlap the next part's first ones. */
int song2_ctx_enqueue_part(song2_ctx *ctx, int part, int n_parts, void *stream, char *err);
/* As song2_ctx_run, with the run's stream work (queue resets and the evolver
   launches of every launch group) captured into a CUDA graph on the first call
   and replayed on the later ones (no counterpart in the reference). */
int song2_ctx_run_graph(song2_ctx *ctx, void *stream, char *err);
/* Device pointer of the flat source buffer and of the per-triplet stats. */
double *song2_ctx_device_sources(song2_ctx *ctx);
song2_triplet_stats *song2_ctx_device_stats(song2_ctx *ctx);
/* Copy the flat sources / stats to host memory. */
int song2_ctx_download(song2_ctx *ctx, double *flat_sources_host,
                       song2_triplet_stats *stats_host, char *err);
/* Device time of the last run's evolver kernel, milliseconds (CUDA events on
   the launching stream), and its launch count. */
double song2_ctx_last_kernel_ms(song2_ctx *ctx);
int song2_ctx_last_launches(song2_ctx *ctx);

/* Diagnostics of builds compiled with -DSONG2_PHASE_TIMERS (no counterpart in
   the reference): the SM clock cycles and the number of visits of each evolver
   phase, summed over the runs of the context so far, as out[2*phase] and
   out[2*phase+1] (out holds n >= 48 entries).  Returns the number of phases, or
   0 for a build without the timers. */
int song2_ctx_phase_cycles(song2_ctx *ctx, unsigned long long *out, int n);

/* One-shot drop-in for the reference's triplet loop: creates a context,
   evolves every triplet and scatters the result into the caller-allocated
   ppt2->sources slabs sources[tp2][k1][k2][tau*k3_size+k3].  Triplets whose
   first pass retires with an error status are evolved again, in plain FP64 with
   eight times spec.max_steps (the exit strategy of what_if_ndf15_fails,
   perturbations2.c:12877-12957, which re-integrates a failed triplet with another
   evolver and stops the run if that fails too); their stats carry retried = 1.
   Returns 1 if a triplet still fails, with its index and status in err. */
int song2_gpu_evolve(const song2_spec *spec, const song2_tables *tab, int precision,
                     double ****sources_out, song2_triplet_stats *per_triplet,
                     char *err);

/* Allocation-free evolver, for callers that cannot allocate device memory:
   applications whose device memory is owned by a fixed-size pool or by another
   runtime (a framework's caching allocator, a solver that reserves the GPU's
   memory at start-up), or hosts that forbid cudaMalloc after initialisation.  It
   has no counterpart in the reference.  It calls no cudaMalloc, cudaFree or other
   allocating routine: its device scratch (layout tables, work list, work-queue
   counter, the per-triplet Jacobians and quadratic-source tables) lives in one
   64 MiB array compiled into this library, which every GPU that loads the library
   holds until the process exits.  (As for any kernel, the CUDA driver may reserve
   local memory for the evolver's stack frame at its first launch on a device.)
   Problems whose tables do not fit are rejected with an error, and fewer
   triplets run at once when their per-triplet scratch does not all fit.  The
   caller passes the inputs and outputs on the device: tab_dev is a song2_tables
   whose bg, bg_dd, fo and fo_dd point to device memory (spec and its k/k3/tau
   grids stay in host memory and may be freed when the call returns);
   sources_dev holds tp2_size * song2_sources_per_type() doubles (cleared by the
   call) and stats_dev song2_n_triplets() entries in the reference work order (k1
   descending, k2 <= k1, k3 ascending).  Work is enqueued on `stream` (NULL =
   legacy default stream) and the outputs are valid once it has completed.  The
   first call on a device resolves the scratch address with that device current.
   Calls share the scratch and find the previous call's contents in it (each call
   clears what must start at zero): two calls that overlap on the GPU race and
   corrupt each other's results. */
int song2_gpu_evolve_noalloc(const song2_spec *spec, const song2_tables *tab_dev, int precision,
                             double *sources_dev, song2_triplet_stats *stats_dev, void *stream,
                             char *err);

/* First-order provider: evolves SONG's own equations in first-order mode
   (quadratic sources off, has_ad_first_order initial conditions, m = 0)
   for every k of spec->k and fills the first-order table fo[k][tau][q] on the
   given uniform ln(tau) grid (values only; call song2_spline_uniform for the
   second derivatives).  Replaces CLASS perturb_init (perturbations2.c:153). */
int song2_gpu_first_order(const song2_spec *spec2, const song2_tables *bg_only,
                          int fo_l_max, int fo_tau_size, double fo_lntau0,
                          double fo_dlntau, double *fo_out, char *err);

/* ------------------------------------------- line-of-sight integration */
/* The second-order transfer functions of transfer2_init (source/transfer2.c:79-636):
   for every (k1, k2 <= k1) pair, every k of the pair's transfer k grid and every
   transfer type (T, E, B) x (l, m),

     T_lm(k1,k2,k) = 1/16/(2l+1) * sum_tau dtau_tau * sum_L J_Llm(k (tau0 - tau)) S_Lm(k1,k2,k,tau)

   (transfer2_integrate, transfer2.c:2140-2365, with the trapezoid measure
   dtau_i = tau_{i+1} - tau_{i-1} and its 1/2, and the factors 1/4, 1/(2l+1), 1/2 of
   transfer2_compute, :1861-2138; E adds the B->E mixing J_EB S_B for m != 0, B is
   J_EE S_B - J_EB S_E).  The sources are interpolated from the evolver's k3 grid
   onto the transfer k grid (:2612-2780) and from the source time sampling onto the
   integration grid (:2366-2610, :2783-2926).  The projection functions J_Llm(x)
   are sums of spherical Bessel functions j_l1(x) with 3j coefficients
   (bessel2_J_for_Llm / bessel2_J_Llm, bessel2.c:1041-1600), tabulated on a uniform
   x grid and cut below the first x where |J| >= J_cut.

   Transfer output layout (ptr2->transfer[index_tt][index_k1][index_k2][index_k],
   transfer2.c:1007-1040): a flat buffer of tt2_size * (sum over pairs of the
   pair's transfer k size) doubles; per tt, the pairs (k1 ascending, k2 <= k1) back
   to back.  The tt index runs over T, then E, then B (the types the spec has),
   each over (index_l, index_m) with m <= l, l major (transfer2_get_lm_lists,
   :1121-1320). */
enum song2_k3_sampling { SONG2_K3_SAMPLING_CLASS = 0, SONG2_K3_SAMPLING_BESSEL = 1 };
enum song2_tau_sampling { SONG2_TAU_SAMPLING_SOURCES = 0, SONG2_TAU_SAMPLING_CUSTOM = 1,
                          SONG2_TAU_SAMPLING_BESSEL = 2 };
enum song2_interpolation { SONG2_INTERP_LINEAR = 0, SONG2_INTERP_CUBIC = 1 };
enum song2_k3_extrapolation { SONG2_K3_EXTRAP_NONE = 0, SONG2_K3_EXTRAP_FLAT = 1 };
enum song2_transfer_type { SONG2_TT_T = 0, SONG2_TT_E = 1, SONG2_TT_B = 2 };

/* The transfer2/bessel2 parameters (precision2 / transfers2 / bessels2 fields,
   input2.c:1433-1543, 1975-2016, defaults :2206, :2291-2331). */
typedef struct {
  int l_size;                       /* multipoles today: ptr2->l = pbs->l (song2_l_list) */
  const int *l;                     /* ascending, >= 0 */
  int k3_sampling;                  /* transfer2_k3_sampling: class (default) or bessel */
  double q_linstep;                 /* q_linstep_song, 0.45 */
  int tau_sampling;                 /* transfer2_tau_sampling: sources (default), custom, bessel */
  double tau_linstep;               /* tau_linstep_song, 0.6 */
  int k3_interpolation;             /* sources_k3_interpolation, linear */
  int time_interpolation;           /* sources_time_interpolation, linear */
  int bessel_interpolation;         /* bessels_interpolation (CLASS), linear */
  int k3_extrapolation;             /* bispectra_k3_extrapolation: none or flat */
  double extra_k3_oscillations_left, extra_k3_oscillations_right;
  double x_step;                    /* pbs2->xx_step = bessel_x_step_song, 0.2 */
  double x_max;                     /* pbs2->xx_max (song2_los_defaults applies input2.c:1982-2006) */
  double j_cut;                     /* bessel_j_cut_song, 1e-12 */
  double J_cut;                     /* bessel_J_cut_song, 1e-6 */
  double bessel_tol_x_min;          /* CLASS bessel_tol_x_min, 1e-4 */
  double tau0;                      /* conformal age (pba->conformal_age) */
  double tau_rec;                   /* visibility peak (pth->tau_rec), song2_recombination_time() */
} song2_los_spec;

/* ------------------------------------------------ parameter files */
/* The reference's ini/pre files (input2.c) read for the keys of the hot path. */
enum song2_sampling { SONG2_SAMPLING_LIN = 0, SONG2_SAMPLING_LOG = 1, SONG2_SAMPLING_SMART = 2,
                      SONG2_SAMPLING_SYM = 3, SONG2_SAMPLING_THETA12 = 4 };
/* Grid settings of a parameter file (defaults of input2.c:2071-2075, 2316-2325). */
typedef struct {
  int k_sampling;            /* sources2_k_sampling (default smart) */
  double k_min, k_max;       /* k_min_custom_song, k_max_custom_song (lin/log) */
  int k_size;                /* k_size_custom_song */
  int k3_sampling;           /* sources2_k3_sampling (default smart) */
  int k3_size;               /* k3_size (lin/log) */
  int custom_tau;            /* custom_time_sampling_song_sources */
  int tau_sampling;          /* custom_tau_mode_song_sources: SONG2_SAMPLING_LIN / _LOG */
  double tau_ini, tau_end;   /* custom_tau_ini/end_song_sources (tau_end 0: today) */
  int tau_size;              /* custom_tau_size_song_sources */
  int l_max_scalars;         /* CLASS l sampling: l_max_scalars, l_logstep, l_linstep */
  double l_logstep;
  int l_linstep;
  /* smart k1/k2 sampling (input2.c:386-470, defaults :2290-2299) */
  double k_min_tau0, k_max_tau0_over_l_max, k_step_sub, k_step_super, k_logstep_super, k_step_transition;
  double k_per_decade_for_pk, k_per_decade_for_bao, k_bao_center, k_bao_width;
  double k_max_for_pk;       /* 1/Mpc (P_k_max_1/Mpc_song, or P_k_max_h/Mpc_song times h) */
  double h;                  /* the cosmology's h (CLASS key h), for P_k_max_h/Mpc_song */
  int k3_size_min;           /* smart k3 sampling: at least this many k3 per pair */
  int has_cmb, has_lss;      /* from the output string (perturbations2.c:836-950) */
  /* source time sampling without a custom grid (song2_tau_grid_class) */
  double tau_stepsize;       /* perturb_sampling_stepsize_song (default 0.4) */
  double tau_late_boost;     /* perturb_sampling_late_time_boost (default 1) */
  double tau_start_c_over_h; /* start_sources_at_tau_c_over_tau_h (CLASS default 0.008) */
  /* intrinsic bispectrum (song2_bispectra_spec) */
  int bi_k1_interpolation;   /* transfers_k1_interpolation: SONG2_INTERP_LINEAR (default) / _CUBIC */
  int bi_k2_interpolation;   /* transfers_k2_interpolation */
  int bi_r_size;             /* r_size (0: not given) */
} song2_params;
void song2_params_defaults(song2_params *grids);
/* The source time sampling of perturb2_timesampling_for_sources when no custom
   sampling is asked for (perturbations2.c:2604-2869): the first time by bisection
   for (aH)/kappa' = start_tau_c_over_tau_h between z = 1e4 and the visibility peak
   (only with CMB outputs; else the peak itself), then steps of
   stepsize / sqrt(rate^2 + late_boost^2 |2 a''/a - (aH)^2|) with CLASS's
   variation rate of the thermodynamics, rate = sqrt(kappa1^2 + (kappa2/kappa1)^2 +
   |kappa3/kappa1|) for the first three conformal-time derivatives of the optical
   depth (CMB outputs; else stepsize / (aH)), until tau0, the last time exactly
   tau0.  The bisection stops at tau_upper - tau_lower <= tol_tau (CLASS's
   tol_tau_approx, 1e-10).  Writes out (NULL to query) and returns the size, at
   most 1e6, or -1 with a message. */
int song2_tau_grid_class(const song2_tables *tab, double stepsize, double late_boost, double start_tau_c_over_tau_h,
                         double tol_tau, int has_cmb, double *out, char *err);
/* Comoving sound horizon int_0^tau c_s dtau', c_s^2 = 1/(3 (1 + 3 rho_b / 4 rho_g)),
   on the background table (CLASS's pth->rs_rec at tau = song2_recombination_time). */
double song2_sound_horizon(const song2_tables *tab, double tau);
/* The smart k1/k2 sampling of perturb2_get_k_lists (perturbations2.c:1610-1766):
   from k_min_tau0/tau0 by the smaller of a logarithmic and a tanh-blended linear
   step in units of k_rec = 2 pi / rs_rec up to k_max_tau0_over_l_max l_scalar_max /
   tau0 (CMB outputs), then logarithmically with the BAO-weighted density up to
   k_max_for_pk (LSS outputs); the last value is exactly the larger k_max.  Writes
   k_out when not NULL and returns the size, or -1 with a message. */
int song2_k_grid_smart(const song2_params *grids, double tau0, double rs_rec, int l_scalar_max, double *k_out,
                       char *err);
/* The smart k3 sampling (perturbations2.c:2086-2178): for every pair the points of
   the k grid within [k3_min, k3_max] (the same limits as song2_k3_grids), merged
   with the two limits, and with k3_size_min - n + 2 evenly spaced points between
   them merged in when the pair has n < k3_size_min points; sorted, duplicates
   removed (CLASS's merge_arrays_double).  Same outputs as song2_k3_grids. */
/* The theta_12 k3 sampling of perturb2_get_k_lists (perturbations2.c:2029-2060):
   for every pair, k3_size values linear in the angle between k1 and k2 over the
   limits of the lin/log samplings, k3 = sqrt(k1^2 + k2^2 + 2 cos(theta) k1 k2);
   for k1 = k2 the first angle moves a fifth of a step inwards.  Same outputs as
   song2_k3_grids. */
int song2_k3_grids_theta12(const double *k, int k_size, int k3_size, int *k3_size_out, double *k3_out, char *err);
int song2_k3_grids_smart(const double *k, int k_size, int k3_size_min, int *k3_size_out, double *k3_out,
                         char *err);
/* Reads an ini and a pre file (either may be NULL; a name may appear once in
   the two) into spec (starting from song2_spec_defaults with the reference's
   default radiation-streaming approximation, rsa2_MD), the grid settings and,
   when los is not NULL, the line-of-sight settings (its l list, tau0 and
   tau_rec are kept).  Names and their obsolete aliases, the yes/no rules and
   the output string follow input2.c:137-2016 and perturb2_indices_of_perturbs
   (perturbations2.c:843-945).  Settings the evolver does not implement
   (imperfect fluids, perturbed recombination, other phi equations) are errors.
   The smart, sym and theta_12 samplings are reported in grids; building their
   grids is the caller's (the drop-in takes ppt2->k and ppt2->k3 as they are).
   Not reentrant. */
int song2_read_params(const char *ini_path, const char *pre_path, song2_spec *spec, song2_params *grids,
                      song2_los_spec *los, char *err);
/* The cosmology keys of the same files (CLASS's input names): h or H0, T_cmb,
   omega_b or Omega_b, omega_cdm or Omega_cdm, N_ur or N_eff, YHe, and
   reio_parametrization = reio_none or reio_camb with z_reio; absent keys take
   the benchmark cosmology (h 0.678, omega_b 0.0224, omega_cdm 0.120, N_eff
   3.046, T_cmb 2.7255, YHe 0.24, no reionisation).  Settings the input
   provider cannot honour (100*theta_s, massive neutrinos, curvature,
   YHe = BBN, tau_reio) are errors.  Not reentrant. */
int song2_read_cosmo(const char *ini_path, const char *pre_path, song2_cosmo *cosmo, char *err);

/* Defaults of the reference (input2.c) for the spec's k range and tables:
   x_max = k_max * 18000 for the lin/log k samplings (input2.c:1986-1989), plus
   one step, times 1.05; tau0 and tau_rec from the tables.  l and l_size are left
   for the caller (song2_l_list). */
void song2_los_defaults(song2_los_spec *los, const song2_spec *spec, const song2_tables *tab);
/* The l sampling of the first-order Bessel module that transfer2 copies
   (transfer2_get_l_list, transfer2.c:1081-1110; CLASS's l list: l = 2, then
   steps of max(1, (int)(l (l_logstep - 1))) while below l_linstep, then steps
   of l_linstep, and l_max last).  Writes the list into out (may be NULL) and
   returns its length. */
int song2_l_list(int l_max, double l_logstep, int l_linstep, int *out);
/* Conformal time of the visibility peak, max of kappa' exp(-kappa) (pth->tau_rec). */
double song2_recombination_time(const song2_tables *tab);
/* Number of transfer types (ptr2->tt2_size) and, for each, its type, l and m
   (any of the arrays may be NULL). */
int song2_transfer_types(const song2_spec *spec, const song2_los_spec *los, int *type, int *l, int *m);
/* Transfer k grid of every (k1, k2 <= k1) pair, in pair order (transfer2_get_k3_sizes
   / _get_k3_size / _get_k3_list, transfer2.c:1329-1860): sizes[n_pairs],
   physical_start[n_pairs] and physical_size[n_pairs] (any may be NULL), and the
   grids back to back in k_out (NULL to query; its length is the return value of
   the first call).  Returns the total number of k values, or -1 with a message. */
int64_t song2_transfer_k_grids(const song2_spec *spec, const song2_los_spec *los, int *sizes, int *physical_start,
                               int *physical_size, double *k_out, char *err);
/* Row of 3j symbols (l1 l2 l3; -m2-m3 m2 m3) for every l1 from l1_min to
   l1_max = l2 + l3, by the Schulten-Gordon recursion in l1 (the drc3jj routine the
   reference calls at bessel2.c:1151-1197); out holds l1_max - l1_min + 1 values.
   Returns 0, or 1 if the row is empty. */
int song2_wigner3j_row(int l2, int l3, int m2, int m3, int *l1_min, int *l1_max, double *out, int out_size);

/* Line-of-sight handle: the projection-function tables on the device
   (bessel2_init, bessel2.c:75-497: the spherical Bessel functions j_l1(x) of the
   extended l1 list, J_TT, J_EE and J_EB for every (L, l, m) with their x_min)
   and the transfer k grids, for one spec and los spec. */
typedef struct song2_los song2_los;
int song2_los_create(const song2_spec *spec, const song2_los_spec *los, song2_los **out, char *err);
void song2_los_destroy(song2_los *h);
/* Doubles of the flat transfer output. */
int64_t song2_los_transfer_size(const song2_los *h);
/* The transfer functions of device-resident sources (the flat layout of
   song2_ctx_download, e.g. song2_ctx_device_sources()) into transfer_dev
   (song2_los_transfer_size() doubles), enqueued on `stream` (NULL = legacy
   default stream); returns once the work is enqueued. */
int song2_los_run(song2_los *h, const double *sources_dev, double *transfer_dev, void *stream, char *err);
/* Device time (ms) of the last song2_los_run's kernels and of song2_los_create's
   table build. */
float song2_los_last_ms(const song2_los *h);
float song2_los_tables_ms(const song2_los *h);
/* Copies of the device tables, for checks: j_l1 on the x grid for each l1 of the
   extended list ([n_l1][x_size], x below the l1's x_min zero) and J for every
   projection row ([rows][x_size], row = ((J*L_size + L)*l_size + index_l)*m_size
   + index_m with J = TT, EE, EB), with the rows' first non-negligible x index.
   Sizes: song2_los_table_sizes.  Any pointer may be NULL. */
void song2_los_table_sizes(const song2_los *h, int *x_size, int *n_l1, int *L_size, int *m_size, int *n_rows);
int song2_los_tables(song2_los *h, int *l1, double *j_l1, double *J, int *J_xmin, char *err);
/* One-shot drop-in for the transfer2_init compute loop: host sources in the flat
   layout (or ppt2->sources gathered into it) to host transfers in the flat
   transfer layout. */
int song2_gpu_transfer(const song2_spec *spec, const song2_los_spec *los, const double *sources_flat,
                       double *transfer_flat, char *err);

/* ------------------------------------------------ intrinsic bispectrum
   bispectra2_intrinsic_init and its integrals (bispectra2.c:300-3030): for every
   second-order field X, azimuthal number M3 of the spec's m list and offset L3 =
   |l3 - M3| + offset_L3 allowed by the parity, the k3 integral
   I_l3(r,k1,k2) = 2 c_M3 int dk3 k3^2 j_L3(r k3) T^(2)_l3M3(k1,k2,k3), then for
   every first-order field Y the k2 integral of I_l3, interpolated in k2 onto the
   first-order grid q with the window 1/k^2, times P(q) T^(1)_l2(q) j_l2(r q);
   for every even offset L1 = |l1 - M3| + offset_L1 and field Z the k1 integral
   with j_L1(r q) T^(1)_l1(q) P(q), the r integral int dr r^2, and the
   geometrical factors (four 3j symbols and a 6j symbol); the result is
   symmetrised over the position of the second-order field
   (bispectra2.c:760-790).  All integrals are trapezoidal on the grids given,
   j_l from the line-of-sight handle's Bessel table (bessel2_convolution,
   bessel2.c:499-600).

   Fields are the transfer types SONG2_TT_T, _E, _B; the field parity (0 for T
   and E, 1 for B) of the last field combination governs every combination, as
   the reference sets it once (bispectra2.c:967).  With an m list of {0} only,
   the reduced bispectrum is 8/pi^3 times the integral for every (l1, l2, l3)
   (bispectra2.c:2824-2832).

   Output layout: [X][Y][Z][conf] doubles (bf_size^3 * n_conf), conf running
   over index_l1 ascending, index_l2 <= index_l1 and index_l3 from the first l
   >= |l1 - l2| to min(index_l2, the last l <= l1 + l2), as song2_bispectra_configs
   lists them (the reference's loop order at bispectra2.c:760-764). */
typedef struct {
  int bf_size;                /* fields (pbi->bf_size) */
  const int *bf;              /* SONG2_TT_T / _E / _B each, distinct */
  int r_size;                 /* integration grid in r (pwb->r), ascending, positive */
  const double *r;
  int q_size;                 /* first-order transfer grid (ptr->q), ascending, within the spec's k range */
  const double *q;
  const double *pk;           /* primordial spectrum on q (pbi->pk) */
  const double *transfer1;    /* first-order transfers [bf][index_l][q] on the line-of-sight l list
                                 (ptr->transfer, scalar adiabatic) */
  int k1_interpolation;       /* transfers_k1_interpolation: SONG2_INTERP_LINEAR / _CUBIC */
  int k2_interpolation;       /* transfers_k2_interpolation */
} song2_bispectra_spec;
/* The (index_l1, index_l2, index_l3) configurations of the output, in order
   (any array may be NULL); returns their number. */
int64_t song2_bispectra_configs(int l_size, const int *l, int *i1, int *i2, int *i3);
typedef struct song2_bispectra song2_bispectra;
/* Binds a bispectrum run to a line-of-sight handle (its l list, transfer k grids,
   transfer types and Bessel table) and uploads the first-order inputs. */
int song2_bispectra_create(song2_los *los, const song2_bispectra_spec *bs, song2_bispectra **out, char *err);
void song2_bispectra_destroy(song2_bispectra *h);
/* Doubles of the output (bf_size^3 * n_conf). */
int64_t song2_bispectra_size(const song2_bispectra *h);
/* The bispectra of device-resident second-order transfers (the flat layout of
   song2_los_run) into out_dev (song2_bispectra_size() doubles), on `stream`
   (NULL = legacy default stream); returns when the result is complete. */
int song2_bispectra_run(song2_bispectra *h, const double *transfer2_dev, double *out_dev, void *stream, char *err);
/* Device time (ms) of the last song2_bispectra_run. */
float song2_bispectra_last_ms(const song2_bispectra *h);
/* One shot: host second-order transfers in the flat layout to host bispectra. */
int song2_gpu_bispectra(const song2_spec *spec, const song2_los_spec *los, const song2_bispectra_spec *bs,
                        const double *transfer2_flat, double *out, char *err);
/* bispectra2_add_quadratic_corrections (bispectra2.c:3031-3106): adds to the
   intrinsic bispectrum -3/8 of the quadratic bispectrum (bolometric temperature)
   and, with use_delta_tilde, +4/8 of it (the redshift term the delta-tilde
   sources absorb); b and b_quadratic share the output layout. */
void song2_bispectra_add_quadratic(double *b, const double *b_quadratic, int64_t n, int use_delta_tilde);

#ifdef __cplusplus
}
#endif
#endif /* SONG2_H */
