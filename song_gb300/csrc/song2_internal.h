/*
 * song2_internal.h - device-side data layout shared by the evolver kernel
 * (song2_evolver.cuh, song2_launch.cu) and the C ABI host code (song2_capi.cu).
 */
#ifndef SONG2_INTERNAL_H
#define SONG2_INTERNAL_H

#include <cuda_runtime.h>
#include <stdint.h>

#include "song2.h"

#define S2_LMAXP (SONG2_MAX_L + 4)
#define S2_MAXBLK SONG2_MAX_M
#define S2_MAXTP 64
#define S2_MAXCH 3          /* moment chains per m block (I, E/B, N) */
#define S2_MAXCORE 16       /* largest dense core of an m block */

/* species codes of the state vector and of the quadratic-source vector */
enum { SP_I = 0, SP_E, SP_B, SP_N, SP_B000, SP_B11, SP_C000, SP_C11, SP_PHI, SP_PHIP, SP_OMEGA, SP_GAMMA, SP_GAMMAP,
       SP_METRIC, SP_NONE };

/* source types */
enum { TP_T = 0, TP_E, TP_B, TP_D };

/* Everything that is constant for a run; passed to the kernel by value. */
struct DevSpec {
  int l_max_g, l_max_pol, l_max_ur, l_los_t, l_los_p;
  /* closure coefficients of the hierarchies at their l_max per m
     (perturbations2.c:7931-7941, 8024-8036, 8120-8130): the l_max - 1 coupling of
     I and N, of E and B, and the E-B mixing m / l_max_pol */
  double cl_I[SONG2_MAX_M], cl_N[SONG2_MAX_M], cl_P[SONG2_MAX_M], cmix_P[SONG2_MAX_M];
  int m_size, m[SONG2_MAX_M], compute_m[SONG2_MAX_M], index_m[SONG2_MAX_M];
  int index_m_max[S2_LMAXP];
  int L_big, Lq, mq_max;          /* rotation coefficients for l <= Lq, 0 <= m <= mq_max */
  int has_pol, has_qs, has_liou, has_coll, tca_on;
  double tca_h, tca_k;
  int ic;
  double fnl;
  int los_pure_scat, los_quad_scat, los_pure_metric, los_quad_metric, los_time_delay, los_redshift, los_lensing;
  int los_sw, los_isw, los_exp_pot;
  int dtilde, dt_qt, dt_qp, dt_Q, dt_L;  /* delta-tilde sources: l1, l2 cuts of T and E/B, table extents */
  int rescale;                     /* rotation coefficients / sin(theta_k1)^m */
  int rsa;                         /* radiation-streaming approximation: 0 off, 1 MD, 2 MD with reionisation */
  double rsa_k, tau_fs;            /* its k tau trigger and the start of free streaming */
  double rtol, threshold;
  int max_steps;
  double start_h, start_k, tol_tau;
  /* (l,m) tables */
  int n_lm;                        /* pairs l <= Lq, m in the list, m <= l */
  short lm_array[S2_LMAXP][SONG2_MAX_M];
  int n_lmq;                       /* pairs l <= Lq, 0 <= m <= min(l, mq_max) */
  short lmq[S2_LMAXP][SONG2_MAX_M + 2];
  /* quadratic-source layout */
  int qs2_size, iq_g, iq_E, iq_B, iq_ur, iq_b, iq_cdm;
  int iq_psi, iq_psi_prime, iq_phi_prime_poisson, iq_phi_prime_longitudinal, iq_phi_prime_prime;
  int iq_omega_m1_prime, iq_gamma_m2_prime_prime, iq_vv_g, iq_vv_ur, iq_dd_b, iq_vv_b, iq_vv_cdm;
  int iq_vvp_b, iq_vvp_cdm;        /* d/dtau of the velocity products (psi') */
  int n_row_slots, n_qs_slots;     /* species-grouped, warp-padded evaluation orders (rows: the
                                      core rows; the chain rows come from the GenRow table) */
  int n_gen;                       /* chain rows (GenRow entries) */
  int n_qo_slots;                  /* the same for the entries an output time needs */
  short iq_b11[2], iq_c11[2], iq_b000, iq_c000;
  /* state layout (grouped by m blocks) */
  int n;
  int nblk, blk_start[S2_MAXBLK], blk_size[S2_MAXBLK];
  int idx_phi, idx_phip, idx_omega, idx_gamma, idx_gammap, idx_b000, idx_c000, idx_b11[2], idx_c11[2];
  /* first-order table */
  int fo_l_max, nfo, fo_E, fo_N, fo_CG, fo_tau_size, fo_k_size;
  double fo_lntau0, fo_dlntau, fo_inv_dx, fo_dx2_6;    /* 1/dlntau, dlntau^2/6 (spline evaluation) */
  int bg_size;
  double bg_lntau0, bg_dlntau, bg_inv_dx, bg_dx2_6;
  /* sources */
  int tp2_size;
  int tp_kind[S2_MAXTP], tp_l[S2_MAXTP], tp_m[S2_MAXTP];
  int mode_first_order;
  int tau_size;
  int64_t per_type;
  int k_size;
  int n_items;
  /* launch: lanes per triplet of the team kernel (1..32) */
  int team_lanes;
  /* shared-memory plan */
  int lu_in_smem;                  /* factors of the iteration matrix in shared memory */
  int lu_elems;                    /* elements of the structured Jacobian (and of its factors) */
  int lu_stride;                   /* per-team Jacobian/factor scratch (>= lu_elems; the largest class) */
  long qtab_stride;                /* per-team quadratic-source table (doubles) */
  /* Structured iteration matrix of every m block.  The block's state splits into a
     dense core (metric and matter variables and the moments with l <= 2) and up to
     S2_MAXCH chains of moments with l >= 3 (I; E, or E and B paired when the block
     has B; N), each coupling only neighbouring l, and coupling to the core only
     through its first node.  Per block: the core's size, the offset of its state
     indices in the mx_idx table and of its storage; per chain: the node dimension
     d (1, or 2 for E/B pairs), the number of nodes, and the same two offsets.  The
     Jacobian and its factors share one layout (lu_elems elements):
       chain: per node k, three d x d blocks (J: diagonal, lower, upper coupling;
              factors: Q_k, Theta_k^-1, P_k), then a d x core block (J: node 0 on
              the core; factors: R) and a core x d block (J and factors: the core
              rows on node 0);
       core:  core x core (J: the core block; factors: the inverse Schur complement). */
  int core_n[S2_MAXBLK], core_idx[S2_MAXBLK], core_off[S2_MAXBLK];
  int ch_n[S2_MAXBLK];
  int ch_d[S2_MAXBLK][S2_MAXCH], ch_len[S2_MAXBLK][S2_MAXCH], ch_idx[S2_MAXBLK][S2_MAXCH], ch_off[S2_MAXBLK][S2_MAXCH];
  /* the chains of every block listed by node dimension (block << 4 | chain), so
     that the lanes of a warp sweep chains of one kind along one code path */
  int n_ch1, n_ch2;
  short ch1[S2_MAXBLK * S2_MAXCH], ch2[S2_MAXBLK * S2_MAXCH];
};

/* A hierarchy moment with l >= 3 (a chain row) as a table entry: its derivative is
     k (c1 y[j1] + c2 y[j2] + c3 y[j3] - cd y[i] / (k tau)) - kappa' y[i] [I, E, B]
       + qs[q]
   (perturbations2.c:7931-7941, 8024-8036, 8120-8130 and the free-streaming rows
   around them): j1, j2 the same species at l - 1 and l + 1, j3 the E-B partner at
   the same l (-1: none), cd the closure's 1/(k tau) coefficient at l_max. */
struct GenRow {
  double c1, c2, c3, cd;
  short i, j1, j2, j3, q, kind;    /* kind: 0 I, 1 E, 2 B, 3 N */
};

/* Per-triplet work item: indices and where its sources go. */
struct WorkItem {
  int i1, i2, i3, pair;            /* pair = index of (i1,i2) in pair order */
  int cls;                         /* hierarchy class (uneven batches), else 0 */
  int ref;                         /* index in the reference work order (k1 descending, k2 <= k1, k3) */
};

/* Tables that depend on the hierarchy layout (one set per class in uneven batches). */
struct ClassTabs {
  const double *cmin, *cplu, *dmin, *dplu, *dzer;   /* [n_lm][3] */
  const short *eq_sp, *eq_l, *eq_m;                  /* [n] */
  const short *idx_I, *idx_E, *idx_B, *idx_N;        /* [n_lm] -> state index or -1 */
  const short *qs_sp, *qs_l, *qs_m;                  /* [qs2_size] */
  const short *row_slot, *qs_slot;                   /* [n_row_slots], [n_qs_slots]: index or -1 */
  const GenRow *gen;                                 /* [n_gen]: the chain rows */
  const short *qo_slot;                              /* [n_qo_slots]: entries read at output times */
  const short *mx_idx;                               /* [n]: state indices of the cores and chain nodes */
  const short *mx_pos;                               /* [n]: position of a state index in its block's
                                                        structure: (chain + 1) << 8 | component << 7 | node,
                                                        or the core position (chain field 0) */
};

/* Device pointers of a run. */
struct DevPtrs {
  const double *k, *k3, *tau;
  const int *k3_off, *k3_size;     /* per pair */
  const int64_t *pair_off;         /* per pair, in doubles, within one source type */
  const double *bg, *bg_dd, *fo, *fo_dd;
  ClassTabs tabs;                  /* uniform runs */
  const DevSpec *class_spec;       /* uneven batches: per class, else null */
  const ClassTabs *class_tabs;
  const WorkItem *items;
  double *sources;                 /* [tp2][per_type] */
  double *fo_out;                  /* first-order mode: [k][tau][q] */
  song2_triplet_stats *stats;      /* [n_items], or [n_triplets] in reference work order (stats_by_ref) */
  int stats_by_ref;                /* write a triplet's stats at its WorkItem::ref */
  double *jac;                     /* per-team structured Jacobian: lu_stride elements of the
                                      iteration-matrix precision */
  double *qtab;                    /* per-team quadratic-source table: fo_tau_size x 2 x qs2_size doubles */
  const double *spl_c;             /* Thomas recurrence of the natural spline on a uniform grid */
  const double *dt_coup;           /* delta-tilde couplings, see dt_index() */
  void *lu_global;                 /* per-team factor scratch when not in smem */
  double *tslab;                   /* team kernel: per-team vectors, 32/G teams interleaved per warp */
  void *txsol;                     /* team kernel: solve vectors (iteration-matrix precision) */
  int *queue;                      /* work-queue counter */
  unsigned long long *phase;       /* builds with SONG2_PHASE_TIMERS: [S2_NPHASE][2] cycles, count */
};

/* Phases of the per-phase cycle counters (builds with SONG2_PHASE_TIMERS only):
   thread 0 of each team attributes the SM clock cycles since its previous mark to
   the phase that has just ended. */
enum {
  PH_SETUP = 0,   /* work item, geometry, start time and approximation intervals */
  PH_QTAB,        /* per-triplet quadratic-source table and its spline */
  PH_IC,          /* interval start: initial conditions or TCA remap */
  PH_START,       /* NDF start: first right-hand side, Jacobian, factorisation */
  PH_RESCALE,     /* backward differences rescaled for a new step size or order */
  PH_FACT,        /* iteration matrix formed and factorised (and inverted) */
  PH_PRED,        /* predictor, error weights and their norm */
  PH_PREP,        /* background and interpolated quadratic sources at t_new */
  PH_WS,          /* workspace scalars of the Newton right-hand side */
  PH_ROWS,        /* rows of the Newton right-hand side */
  PH_SOLVE,       /* linear solve */
  PH_NUPD,        /* Newton update, norm and convergence test */
  PH_JAC,         /* Jacobian refresh after a failed Newton iteration */
  PH_ERR,         /* local error estimate, rejection and its step-size choice */
  PH_ACCEPT,      /* backward differences of the accepted step */
  PH_OUT_RHS,     /* output: state interpolated, derivs at the sampling time */
  PH_OUT_QS,      /* output: direct quadratic sources and workspace */
  PH_OUT_STORE,   /* output: source functions written */
  PH_CTRL,        /* step-size and order selection, state copy */
  PH_ITEM,        /* whole triplets (count = triplets) */
  PH_SOLVE_BACK,  /* linear solve: backward sweeps of the chains (PH_SOLVE: the forward sweeps) */
  PH_SOLVE_CORE,  /* linear solve: the cores */
  PH_FACT_CHAIN,  /* factorisation: the chains (PH_FACT: the cores and the rest) */
  S2_NPHASE = 24
};

/* Position of the delta-tilde coupling of (field, l, m, l1, m1, l2) in
   DevPtrs::dt_coup: field 0..2 (T, E, B), l <= dt_L, 0 <= m < SONG2_MAX_M,
   l1, l2 <= dt_Q, |m1| <= dt_Q. */
__host__ __device__ inline int dt_index(const DevSpec &s, int field, int l, int m, int l1, int m1, int l2) {
  return ((((field * (s.dt_L + 1) + l) * SONG2_MAX_M + m) * (s.dt_Q + 1) + l1) * (2 * s.dt_Q + 1) + m1 + s.dt_Q) *
             (s.dt_Q + 1) + l2;
}
inline int dt_table_size(const DevSpec &s) { return 3 * (s.dt_L + 1) * SONG2_MAX_M * (s.dt_Q + 1) * (2 * s.dt_Q + 1) * (s.dt_Q + 1); }

/* host-side launcher implemented in song2_launch.cu.  mode 0: one CTA per
   triplet; 1: one warp per triplet (several per CTA); 2: spec.team_lanes lanes per
   triplet, arrays in global slabs (tslab, txsol, jac, lu_global, qtab);
   3: one CTA per triplet with hierarchy classes (ptrs.class_spec set; the dynamic
   shared memory starts with song2_class_spec_bytes() for the class spec copy);
   4: the same with registers for two CTAs per SM; 5: mode 0 with registers for two
   CTAs per SM.
   Mode 0 with ptrs.class_spec set launches mode 3. */
int song2_launch_evolver(const DevSpec &spec, const DevPtrs &ptrs, int precision, int mode, int grid, int block,
                         size_t smem, cudaStream_t stream);
/* shared memory of one team (one CTA in block mode, one warp in warp mode) */
size_t song2_smem_bytes(const DevSpec &spec, int precision, int block, int lu_in_smem);
/* shared memory of a team-kernel CTA, and the doubles of one team's slab */
size_t song2_team_smem_bytes(const DevSpec &spec, int teams_per_cta);
size_t song2_class_spec_bytes();
int song2_team_slab_doubles(const DevSpec &spec);
int song2_max_ctas_per_sm(int precision, int mode, int block, size_t smem);

#endif
