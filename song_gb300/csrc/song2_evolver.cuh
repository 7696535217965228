/*
 * song2_evolver.cuh - the GB300 evolver of SONG's second-order system: device
 * code of the persistent kernels for every team layout.  Each song2_k_*.cu
 * translation unit instantiates one kernel from it, so the kernels compile in
 * parallel; song2_launch.cu holds the host-side launcher.
 *
 * A team (a CTA by default) evolves one (k1,k2,k3) triplet at a time and pulls
 * the next one from a device work queue (persistent kernel).  Inside a team:
 *   - background/thermo and first-order interpolation (cubic splines in ln tau)
 *     and the quadratic sources (perturbations2.c:10643-11813), tabulated per
 *     triplet on the first-order nodes and splined (perturbations2.c:10407-10606),
 *     are held in shared memory;
 *   - the right-hand side of perturb2_derivs (perturbations2.c:7636-8451) is
 *     evaluated by a per-equation row function, one thread per equation, in a
 *     species-grouped order, after three warps have formed the workspace scalars
 *     of the three azimuthal numbers (workspace_at_tau, tca_variables, einstein:
 *     perturbations2.c:8484-9738);
 *   - the system is affine, dy = A(tau) y + s(tau), so the Jacobian is exact:
 *     column j is the row function applied to the unit vector e_j, one thread
 *     per column, with the sources switched off;
 *   - azimuthal modes never couple and the state is l-major within a mode, so the
 *     NDF iteration matrix I - h*gamma*J is block diagonal in m with banded
 *     blocks; every block is factorised (partial pivoting within the band) and
 *     solved by one warp, in FP64 (plain form) or FP32 (mixed form: the Newton
 *     residual, error estimate and step control stay FP64, the simplified Newton
 *     iteration doubles as iterative refinement);
 *   - the integrator is the variable-order NDF method of Shampine & Reichelt
 *     (1997), the same algorithm as the CPU restatement in oracle/;
 *   - a triplet's time range splits into up to three intervals (tight coupling,
 *     full system, radiation streaming: perturbations2.c:4854-5403); the state
 *     keeps every equation, and the ones an approximation drops have zero rows;
 *   - the source writer (perturb2_sources, perturbations2.c:11869-12823) adds the
 *     delta-tilde terms when asked; rescaled rotation coefficients
 *     (perturbations2.c:5635-5652) change only the geometry step.
 * Every loop is bounded (max_steps, 4 Newton iterations, 200 bisection steps);
 * a triplet that breaches a bound retires with a status code.  No kernel spins.
 */
#ifndef SONG2_EVOLVER_CUH
#define SONG2_EVOLVER_CUH

#include <math.h>
#include <stdio.h>

#include "song2_internal.h"

#define SQRT_2 1.4142135623730950488
#define SQRT_3 1.7320508075688772935
#define SQRT_6 2.4494897427831780982
#define FOUR_THIRDS (4.0 / 3.0)
#define ONE_THIRD (1.0 / 3.0)

namespace {

/* ------------------------------------------------------------------ smem */

/* Background and thermodynamics at one time, with the reciprocals the
   right-hand side needs (no FP64 division on the hot path).  Field q is
   bg_field(q); the order below is that of bg_field. */
struct BgV {
  double a, a_sq, Hc, Hc_prime, rho_g, rho_b, rho_cdm, rho_ur, kappa_dot, exp_m_kappa, g, r;
  double inv_kd;     /* 1 / kappa' = tau_c */
  double a2_k2;      /* a^2 / k^2 */
  double inv_ktau;   /* 1 / (k tau), the closure of the hierarchies */
};
#define S2_NBGV 15

struct Tri {
  double k1, k2, k, k_sq, cosk1k2, cosk1k, cosk2k, k1_dot_k2;
  double inv_k, inv_k_sq, lnk;
  double k1_m[3], k2_m[3], k1_ten_k2[5], k1_ten_k1[5], k2_ten_k2[5];
  double mfac[SONG2_MAX_M + 3];    /* rot(l,-m) = (-1)^m rot(l,m) mfac[m]: sin(theta_k1)^2m if rescaled, else 1 */
  double tau_ini, tau_end;
  double ivb[4];                   /* interval limits */
  int ivk[3];                      /* approximation of each interval (AP_*) */
  int i1, i2, i3, pair, item, nint, k3_size;
  int64_t pair_off;
};

/* Shared "workspace" scalars; every entry is affine in y. */
struct WS {
  double I_00, N_00, N_1m[3], I_1m[3], I_2m[3], E_2m[3], B_2m[3], C_1m[3], b_200, b_22m[3], cdm_200, cdm_22m[3];
  double I_1m_tca1[3], I_2m_tca1[3], E_2m_tca1[3], B_2m_tca1[3], Pi_tca1[3];
  double psi, phi_prime, phi_pp, omega_m1_prime, gamma_m2_pp;
};

/* Scalars of the NDF state, written by thread 0 only where noted. */
struct Shared {
  Tri tri;
  BgV bg;
  WS ws;
  double psi_prime;
  double lntau;
  int qt_j0, qt_n;
  double red[32];
  double RU[5][5], Rm[5][5];
  double ctl[4];
  int item;
  int lu_fail;
  int mx_bad;                          /* a Jacobian entry outside the structured layout */
  int ap;
  long long ph_t, ph_item;             /* phase-timer marks (SONG2_PHASE_TIMERS builds) */
};

/* Per-phase cycle counters: PH_MARK(c, id) charges the cycles since the team's
   previous mark to phase id (thread 0 of the team, fire-and-forget atomics).
   Compiled in only with -DSONG2_PHASE_TIMERS; otherwise they vanish. */
#ifdef SONG2_PHASE_TIMERS
#define PH_RESET(c)                                                     \
  do {                                                                  \
    if ((c).rank == 0) (c).sh->ph_t = (c).sh->ph_item = clock64();      \
  } while (0)
#define PH_MARK(c, id)                                                              \
  do {                                                                              \
    if ((c).rank == 0 && (c).p.phase) {                                             \
      long long now_ = clock64();                                                   \
      atomicAdd((c).p.phase + 2 * (id), (unsigned long long)(now_ - (c).sh->ph_t)); \
      atomicAdd((c).p.phase + 2 * (id) + 1, 1ull);                                  \
      (c).sh->ph_t = now_;                                                          \
    }                                                                               \
  } while (0)
#define PH_ITEM_END(c)                                                                          \
  do {                                                                                          \
    if ((c).rank == 0 && (c).p.phase) {                                                         \
      atomicAdd((c).p.phase + 2 * PH_ITEM, (unsigned long long)(clock64() - (c).sh->ph_item)); \
      atomicAdd((c).p.phase + 2 * PH_ITEM + 1, 1ull);                                           \
    }                                                                                           \
  } while (0)
#else
#define PH_RESET(c) do {} while (0)
#define PH_MARK(c, id) do {} while (0)
#define PH_ITEM_END(c) do {} while (0)
#endif

/* Offsets (in bytes) of the dynamic shared-memory plan. */
struct Plan {
  size_t y, f, ynew, difkp1, psiv, del, invwt, yout, dyout, dif, fo1, fo2, qs, qc, rot1, rot2, sc, bgraw, shared,
      tab, xsol, lu, jac, total;
};

__host__ __device__ inline size_t al(size_t x) { return (x + 15) & ~(size_t)15; }

__host__ __device__ inline Plan make_plan(const DevSpec &s, int prec, int lu_in_smem) {
  Plan p;
  size_t o = 0, n = (size_t)s.n, d = sizeof(double);
  p.y = o; o = al(o + n * d);
  p.f = o; o = al(o + n * d);
  p.ynew = o; o = al(o + n * d);
  p.difkp1 = o; o = al(o + n * d);
  p.psiv = o; o = al(o + n * d);
  p.del = o; o = al(o + n * d);
  p.invwt = o; o = al(o + n * d);
  /* the dense-output state lives in the Newton scratch (psiv, del), which is dead
     between an accepted step and the next predictor */
  p.yout = p.psiv;
  p.dyout = p.del;
  p.dif = o; o = al(o + 7 * n * d);
  p.fo1 = o; o = al(o + (size_t)s.nfo * d);
  p.fo2 = o; o = al(o + (size_t)s.nfo * d);
  p.qs = o; o = al(o + (size_t)s.qs2_size * d);
  p.qc = o; o = al(o + (size_t)s.qs2_size * d);
  p.rot1 = o; o = al(o + (size_t)s.n_lmq * d);
  p.rot2 = o; o = al(o + (size_t)s.n_lmq * d);
  p.sc = o; o = al(o + 20 * (size_t)s.n_lm * d);
  p.bgraw = o; o = al(o + 16 * d);
  p.shared = o; o = al(o + sizeof(Shared));
  /* index tables copied from the launch parameters / global memory: the hot
     loops index them per thread, which the constant bank would serialise */
  p.tab = o;
  o = al(o + sizeof(short) * ((size_t)(s.Lq + 1) * (SONG2_MAX_M + SONG2_MAX_M + 2) + SONG2_MAX_M + 4 * n +
                              4 * (size_t)s.n_lm + 3 * (size_t)s.qs2_size + s.n_row_slots + s.n_qs_slots +
                              s.n_qo_slots));
  size_t ts = prec == SONG2_PREC_MIXED ? sizeof(float) : sizeof(double);
  p.xsol = o; o = al(o + n * ts);
  /* the structured Jacobian and the factors of the iteration matrix (O(n)
     elements each) */
  p.lu = o;
  if (lu_in_smem) o = al(o + (size_t)s.lu_elems * ts);
  p.jac = o;
  if (lu_in_smem) o = al(o + (size_t)s.lu_elems * ts);
  p.total = o;
  return p;
}

/* ------------------------------------------------------------------ context */

/* A team solves one triplet.  MODE_BLOCK: the CTA; MODE_WARP: one warp; MODE_TEAM:
   G lanes of a warp (G = 1, 2, 4, ... 32), the 32/G teams of a warp interleaved in
   global slabs so that the same element of every team is one coalesced access. */
enum { MODE_BLOCK = 0, MODE_WARP = 1, MODE_TEAM = 2 };
/* approximation of an integration interval (Shared::ap, the `ap` arguments):
   none, tight coupling, radiation streaming */
enum { AP_NONE = 0, AP_TCA = 1, AP_RSA = 2 };

/* per-team array: element i at p[i] (the team owns the array) or p[i * T] (T teams
   interleaved) */
template <typename E, int STRIDED> struct View;
template <typename E> struct View<E, 0> {
  E *p;
  __device__ E &operator[](int i) const { return p[i]; }
  __device__ View operator+(int o) const { return View{p + o}; }
};
template <typename E> struct View<E, 1> {
  E *p;
  int T;
  __device__ E &operator[](int i) const { return p[(long)i * T]; }
  __device__ View operator+(int o) const { return View{p + (long)o * T, T}; }
};

/* Element offsets (in doubles) of one team's arrays in the global slab of MODE_TEAM. */
struct TeamPlan {
  int y, f, ynew, difkp1, psiv, del, invwt, yout, dyout, dif, fo1, fo2, qs, qc, rot1, rot2, sc, bgraw, total;
};

__host__ __device__ inline TeamPlan make_team_plan(const DevSpec &s) {
  TeamPlan t;
  int o = 0, n = s.n;
  t.y = o; o += n;
  t.f = o; o += n;
  t.ynew = o; o += n;
  t.difkp1 = o; o += n;
  t.psiv = o; o += n;
  t.del = o; o += n;
  t.invwt = o; o += n;
  t.yout = t.psiv;
  t.dyout = t.del;
  t.dif = o; o += 7 * n;
  t.fo1 = o; o += s.nfo;
  t.fo2 = o; o += s.nfo;
  t.qs = o; o += s.qs2_size;
  t.qc = o; o += s.qs2_size;
  t.rot1 = o; o += s.n_lmq;
  t.rot2 = o; o += s.n_lmq;
  t.sc = o; o += 20 * s.n_lm;
  t.bgraw = o; o += 16;
  t.total = o;
  return t;
}

/* shared memory of MODE_TEAM: the index tables once per CTA, then one Shared per team */
__host__ __device__ inline size_t team_tables_bytes(const DevSpec &s) {
  return al(sizeof(short) * ((size_t)(s.Lq + 1) * (SONG2_MAX_M + SONG2_MAX_M + 2) + SONG2_MAX_M + 4 * (size_t)s.n +
                             4 * (size_t)s.n_lm + 3 * (size_t)s.qs2_size + s.n_row_slots + s.n_qs_slots +
                             s.n_qo_slots));
}

template <int MODE> struct KX {
  static constexpr int STR = MODE == MODE_TEAM ? 1 : 0;
  using DA = View<double, STR>;
  const DevSpec &s;
  const DevPtrs &p;
  const ClassTabs &ct;
  int rank, size;          /* this thread's rank in its team, team size */
  long team;               /* global team index (per-team global scratch) */
  unsigned tmask;          /* lanes of the team (MODE_TEAM) */
  int nt;                  /* teams interleaved in the slabs (MODE_TEAM), else 1 */
  DA y, f, ynew, difkp1, psiv, del, invwt, yout, dyout, dif, fo1, fo2, qs, qc, rot1, rot2, sc, bgraw;
  Shared *sh;
  short *lm_s, *lmq_s, *im_s, *eq_sp, *eq_l, *eq_m, *idx_I, *idx_E, *idx_B, *idx_N, *qs_sp, *qs_l, *qs_m, *row_slot,
      *qs_slot, *qo_slot, *mx_s;
  char *xsol_b, *lu_b;     /* element 0 of this team's solve vector and iteration-matrix factors */
  char *jac_b;             /* element 0 of this team's structured Jacobian */
  DA qtab;

  template <typename E> __device__ View<E, STR> mk(char *b) const {
    if constexpr (STR) return View<E, 1>{(E *)b, nt};
    else return View<E, 0>{(E *)b};
  }
  __device__ DA da(double *b) const {
    if constexpr (STR) return DA{b, nt};
    else return DA{b};
  }
  template <typename E> __device__ View<E, STR> xsol() const { return mk<E>(xsol_b); }
  template <typename E> __device__ View<E, STR> lu() const { return mk<E>(lu_b); }
  /* the structured Jacobian, stored in the iteration-matrix precision: in shared
     memory beside the factors, or in global scratch at an element offset counted in
     elements of that precision, so the teams' regions stay disjoint whatever the
     element size */
  template <typename E> __device__ View<E, STR> jacv() const { return mk<E>(jac_b); }

  __device__ void set_tables(short *tb) {
    lm_s = tb; tb += (s.Lq + 1) * SONG2_MAX_M;
    lmq_s = tb; tb += (s.Lq + 1) * (SONG2_MAX_M + 2);
    im_s = tb; tb += SONG2_MAX_M;
    eq_sp = tb; tb += s.n;
    eq_l = tb; tb += s.n;
    eq_m = tb; tb += s.n;
    idx_I = tb; tb += s.n_lm;
    idx_E = tb; tb += s.n_lm;
    idx_B = tb; tb += s.n_lm;
    idx_N = tb; tb += s.n_lm;
    qs_sp = tb; tb += s.qs2_size;
    qs_l = tb; tb += s.qs2_size;
    qs_m = tb; tb += s.qs2_size;
    row_slot = tb; tb += s.n_row_slots;
    qs_slot = tb; tb += s.n_qs_slots;
    qo_slot = tb; tb += s.n_qo_slots;
    mx_s = tb;
  }

  __device__ KX(const DevSpec &s_, const DevPtrs &p_, const ClassTabs &ct_, char *smem_all, int prec)
      : s(s_), p(p_), ct(ct_) {
    size_t ts = prec == SONG2_PREC_MIXED ? sizeof(float) : sizeof(double);
    if constexpr (MODE == MODE_TEAM) {
      int G = s_.team_lanes, lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpc = blockDim.x >> 5;
      nt = 32 / G;
      int tiw = lane / G;
      rank = lane % G;
      size = G;
      tmask = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << (tiw * G));
      long gw = (long)blockIdx.x * wpc + warp;
      team = gw * nt + tiw;
      TeamPlan tp = make_team_plan(s_);
      double *base = p_.tslab + gw * (long)tp.total * nt + tiw;
      y = da(base + (long)tp.y * nt); f = da(base + (long)tp.f * nt); ynew = da(base + (long)tp.ynew * nt);
      difkp1 = da(base + (long)tp.difkp1 * nt); psiv = da(base + (long)tp.psiv * nt); del = da(base + (long)tp.del * nt);
      invwt = da(base + (long)tp.invwt * nt); yout = da(base + (long)tp.yout * nt); dyout = da(base + (long)tp.dyout * nt);
      dif = da(base + (long)tp.dif * nt); fo1 = da(base + (long)tp.fo1 * nt); fo2 = da(base + (long)tp.fo2 * nt);
      qs = da(base + (long)tp.qs * nt); qc = da(base + (long)tp.qc * nt); rot1 = da(base + (long)tp.rot1 * nt);
      rot2 = da(base + (long)tp.rot2 * nt); sc = da(base + (long)tp.sc * nt); bgraw = da(base + (long)tp.bgraw * nt);
      set_tables((short *)smem_all);
      sh = (Shared *)(smem_all + team_tables_bytes(s_)) + (long)warp * nt + tiw;
      xsol_b = (char *)p_.txsol + (gw * (long)s_.n * nt + tiw) * ts;
      lu_b = (char *)p_.lu_global + (gw * (long)s_.lu_stride * nt + tiw) * ts;
      jac_b = (char *)p_.jac + (gw * (long)s_.lu_stride * nt + tiw) * ts;
      qtab = da(p_.qtab ? p_.qtab + gw * s_.qtab_stride * nt + tiw : nullptr);
    } else {
      Plan pl = make_plan(s_, prec, s_.lu_in_smem);
      char *smem = smem_all;
      nt = 1;
      tmask = 0xffffffffu;
      if constexpr (MODE == MODE_WARP) {
        rank = threadIdx.x & 31;
        size = 32;
        team = (long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
        smem = smem_all + (size_t)(threadIdx.x >> 5) * pl.total;
      } else {
        rank = threadIdx.x;
        size = blockDim.x;
        team = blockIdx.x;
      }
      y = da((double *)(smem + pl.y)); f = da((double *)(smem + pl.f)); ynew = da((double *)(smem + pl.ynew));
      difkp1 = da((double *)(smem + pl.difkp1)); psiv = da((double *)(smem + pl.psiv)); del = da((double *)(smem + pl.del));
      invwt = da((double *)(smem + pl.invwt)); yout = da((double *)(smem + pl.yout)); dyout = da((double *)(smem + pl.dyout));
      dif = da((double *)(smem + pl.dif)); fo1 = da((double *)(smem + pl.fo1)); fo2 = da((double *)(smem + pl.fo2));
      qs = da((double *)(smem + pl.qs)); qc = da((double *)(smem + pl.qc)); rot1 = da((double *)(smem + pl.rot1));
      rot2 = da((double *)(smem + pl.rot2)); sc = da((double *)(smem + pl.sc)); bgraw = da((double *)(smem + pl.bgraw));
      sh = (Shared *)(smem + pl.shared);
      set_tables((short *)(smem + pl.tab));
      xsol_b = smem + pl.xsol;
      if (s_.lu_in_smem) lu_b = smem + pl.lu;
      else lu_b = (char *)p_.lu_global + (size_t)team * s_.lu_stride * ts;
      if (s_.lu_in_smem) jac_b = smem + pl.jac;
      else jac_b = (char *)p_.jac + (size_t)team * s_.lu_stride * ts;
      qtab = da(p_.qtab ? p_.qtab + (size_t)team * s_.qtab_stride : nullptr);
    }
  }
  __device__ void sync() const {
    if constexpr (MODE == MODE_BLOCK) __syncthreads();
    else if constexpr (MODE == MODE_WARP) __syncwarp();
    else __syncwarp(tmask);
  }
  __device__ int LM(int l, int m) const { return lm_s[l * SONG2_MAX_M + im_s[m]]; }
  __device__ int LMQ(int l, int m) const { return lmq_s[l * (SONG2_MAX_M + 2) + m]; }
  /* copy the index tables into shared memory (once per kernel; by the CTA in
     MODE_TEAM, by the team otherwise) */
  __device__ void load_tables() const {
    int r = rank, z = size;
    if constexpr (MODE == MODE_TEAM) { r = threadIdx.x; z = blockDim.x; }
    for (int e = r; e < (s.Lq + 1) * SONG2_MAX_M; e += z) lm_s[e] = s.lm_array[e / SONG2_MAX_M][e % SONG2_MAX_M];
    for (int e = r; e < (s.Lq + 1) * (SONG2_MAX_M + 2); e += z)
      lmq_s[e] = s.lmq[e / (SONG2_MAX_M + 2)][e % (SONG2_MAX_M + 2)];
    for (int e = r; e < SONG2_MAX_M; e += z) im_s[e] = (short)s.index_m[e];
    for (int e = r; e < s.n; e += z) {
      eq_sp[e] = ct.eq_sp[e]; eq_l[e] = ct.eq_l[e]; eq_m[e] = ct.eq_m[e];
    }
    for (int e = r; e < s.n_lm; e += z) {
      idx_I[e] = ct.idx_I[e]; idx_E[e] = ct.idx_E[e]; idx_B[e] = ct.idx_B[e]; idx_N[e] = ct.idx_N[e];
    }
    for (int e = r; e < s.qs2_size; e += z) {
      qs_sp[e] = ct.qs_sp[e]; qs_l[e] = ct.qs_l[e]; qs_m[e] = ct.qs_m[e];
    }
    for (int e = r; e < s.n_row_slots; e += z) row_slot[e] = ct.row_slot[e];
    for (int e = r; e < s.n_qs_slots; e += z) qs_slot[e] = ct.qs_slot[e];
    for (int e = r; e < s.n_qo_slots; e += z) qo_slot[e] = ct.qo_slot[e];
    for (int e = r; e < s.n; e += z) mx_s[e] = ct.mx_idx[e];
  }
  /* summed couplings, index X in 0..19 */
  __device__ double S(int X, int l, int m) const { return sc[X * s.n_lm + LM(l, m)]; }
  __device__ double cmin(int l, int m1, int m) const { return __ldg(ct.cmin + LM(l, m) * 3 + m - m1 + 1); }
  __device__ double cplu(int l, int m1, int m) const { return __ldg(ct.cplu + LM(l, m) * 3 + m - m1 + 1); }
  __device__ double dmin(int l, int m1, int m) const { return __ldg(ct.dmin + LM(l, m) * 3 + m - m1 + 1); }
  __device__ double dplu(int l, int m1, int m) const { return __ldg(ct.dplu + LM(l, m) * 3 + m - m1 + 1); }
  __device__ double dzer(int l, int m1, int m) const { return __ldg(ct.dzer + LM(l, m) * 3 + m - m1 + 1); }
  __device__ double rot_1(int l, int m) const {
    if (l < 0 || abs(m) > l) return 0.0;
    double v = rot1[LMQ(l, abs(m))];
    if (m < 0) v *= sh->tri.mfac[-m];
    return (m < 0 && (m & 1)) ? -v : v;
  }
  __device__ double rot_2(int l, int m) const {
    if (l < 0 || abs(m) > l) return 0.0;
    double v = rot2[LMQ(l, abs(m))];
    if (m < 0) v *= sh->tri.mfac[-m];
    return (m < 0 && (m & 1)) ? -v : v;
  }
  __device__ double I1r(int l) const { return l < 0 ? 0.0 : fo1[SONG2_FO_I + l]; }
  __device__ double I2r(int l) const { return l < 0 ? 0.0 : fo2[SONG2_FO_I + l]; }
  __device__ double E1r(int l) const { return (l < 0 || !s.has_pol) ? 0.0 : fo1[s.fo_E + l]; }
  __device__ double E2r(int l) const { return (l < 0 || !s.has_pol) ? 0.0 : fo2[s.fo_E + l]; }
  __device__ double N1r(int l) const { return l < 0 ? 0.0 : fo1[s.fo_N + l]; }
  __device__ double N2r(int l) const { return l < 0 ? 0.0 : fo2[s.fo_N + l]; }
};

enum { CM12 = 0, CM21, CP12, CP21, CM11, CM22, CP11, CP22, DM12, DM21, DP12, DP21, DM11, DM22, DP11, DP22, DZ12, DZ21,
       DZ11, DZ22 };

/* ------------------------------------------------------------------ state accessors */

template <class A> struct YVec {
  A v;
  __device__ double operator()(int i) const { return i < 0 ? 0.0 : v[i]; }
};
template <class A> __device__ inline YVec<A> yvec(const A &a) { return YVec<A>{a}; }
struct YUnit {
  int j;
  __device__ double operator()(int i) const { return (i >= 0 && i == j) ? 1.0 : 0.0; }
};

template <class Y, class C> __device__ inline double getI(const C &c, int ap, const Y &y, int l, int m) {
  if (l < 0 || m < 0 || m > l || l > c.s.l_max_g || (ap == AP_TCA && l >= 1) || ap == AP_RSA) return 0.0;
  return y(c.idx_I[c.LM(l, m)]);
}
template <class Y, class C> __device__ inline double getE(const C &c, int ap, const Y &y, int l, int m) {
  if (!c.s.has_pol || ap || l < 2 || m < 0 || m > l || l > c.s.l_max_pol) return 0.0;
  return y(c.idx_E[c.LM(l, m)]);
}
template <class Y, class C> __device__ inline double getB(const C &c, int ap, const Y &y, int l, int m) {
  if (!c.s.has_pol || ap || l < 2 || m <= 0 || m > l || l > c.s.l_max_pol) return 0.0;
  return y(c.idx_B[c.LM(l, m)]);
}
template <class Y, class C> __device__ inline double getN(const C &c, const Y &y, int l, int m) {
  if (l < 0 || m < 0 || m > l || l > c.s.l_max_ur) return 0.0;
  return y(c.idx_N[c.LM(l, m)]);
}
template <class Y, class C> __device__ inline double getb(const C &c, const Y &y, int n, int m) {
  /* n = 0: b000 ; n = 1: b11m */
  if (n == 0) return y(c.s.idx_b000);
  return (m <= 1) ? y(c.s.idx_b11[m]) : 0.0;
}
template <class Y, class C> __device__ inline double getc(const C &c, const Y &y, int n, int m) {
  if (n == 0) return y(c.s.idx_c000);
  return (m <= 1) ? y(c.s.idx_c11[m]) : 0.0;
}

/* ------------------------------------------------------------------ interpolation */

/* natural cubic spline on a uniform grid, column q at x; inv_dx = 1/dx and
   dx2_6 = dx^2/6 come precomputed (no FP64 division) */
__device__ inline double spl(const double *yv, const double *dd, int n, int ncol, double x0, double inv_dx, double dx2_6,
                             int q, double x) {
  double u = (x - x0) * inv_dx;
  int i = (int)floor(u);
  i = i < 0 ? 0 : (i > n - 2 ? n - 2 : i);
  double b = u - i, a = 1.0 - b;
  const double *y0 = yv + (size_t)i * ncol, *d0 = dd + (size_t)i * ncol;
  return a * __ldg(y0 + q) + b * __ldg(y0 + ncol + q) +
         ((a * a * a - a) * __ldg(d0 + q) + (b * b * b - b) * __ldg(d0 + ncol + q)) * dx2_6;
}

/* d/dx of the same spline */
__device__ inline double spl_dx(const double *yv, const double *dd, int n, int ncol, double x0, double dx, int q,
                                double x) {
  double u = (x - x0) / dx;
  int i = (int)floor(u);
  i = i < 0 ? 0 : (i > n - 2 ? n - 2 : i);
  double b = u - i, a = 1.0 - b;
  const double *y0 = yv + (size_t)i * ncol, *d0 = dd + (size_t)i * ncol;
  return (__ldg(y0 + ncol + q) - __ldg(y0 + q)) / dx +
         ((1.0 - 3 * a * a) * __ldg(d0 + q) + (3 * b * b - 1.0) * __ldg(d0 + ncol + q)) * dx / 6.0;
}

template <class C> __device__ inline double bg_col(const C &c, int q, double tau) {
  return spl(c.p.bg, c.p.bg_dd, c.s.bg_size, SONG2_BG_SIZE, c.s.bg_lntau0, c.s.bg_inv_dx, c.s.bg_dx2_6, q, log(tau));
}

/* Field q of BgV from the spline values v[] of the background columns at
   x = ln tau: every field is exp(c1 v[i1] + c2 v[i2] + cx x + ck ln k), except
   Hc' = v[Hc' tau^2] exp(-2x), so the fields run on separate lanes along one
   code path (one exponential each, no division). */
template <class A> __device__ inline double bg_field(const A &v, int q, double x, double lnk) {
  int i1 = 0, i2 = 0;
  double c1 = 0.0, c2 = 0.0, cx = 0.0, ck = 0.0;
  switch (q) {
  case 0: i1 = SONG2_BG_LN_A; c1 = 1; break;                                           /* a */
  case 1: i1 = SONG2_BG_LN_A; c1 = 2; break;                                           /* a^2 */
  case 2: i1 = SONG2_BG_LN_HC; c1 = 1; break;                                          /* Hc */
  case 3: cx = -2; break;                                                              /* Hc' */
  case 4: i1 = SONG2_BG_LN_RHO_G; c1 = 1; break;
  case 5: i1 = SONG2_BG_LN_RHO_B; c1 = 1; break;
  case 6: i1 = SONG2_BG_LN_RHO_CDM; c1 = 1; break;
  case 7: i1 = SONG2_BG_LN_RHO_UR; c1 = 1; break;
  case 8: i1 = SONG2_BG_LN_KAPPA_DOT; c1 = 1; break;                                   /* kappa' */
  case 9: i1 = SONG2_BG_KAPPA; c1 = -1; break;                                         /* e^-kappa */
  case 10: i1 = SONG2_BG_LN_KAPPA_DOT; c1 = 1; i2 = SONG2_BG_KAPPA; c2 = -1; break;    /* g */
  case 11: i1 = SONG2_BG_LN_RHO_G; c1 = 1; i2 = SONG2_BG_LN_RHO_B; c2 = -1; break;     /* r */
  case 12: i1 = SONG2_BG_LN_KAPPA_DOT; c1 = -1; break;                                 /* 1/kappa' */
  case 13: i1 = SONG2_BG_LN_A; c1 = 2; ck = -2; break;                                 /* a^2/k^2 */
  default: cx = -1; ck = -1; break;                                                    /* 1/(k tau) */
  }
  double e = exp(c1 * v[i1] + c2 * v[i2] + cx * x + ck * lnk);
  return q == 3 ? v[SONG2_BG_HC_PRIME_TAU2] * e : e;
}

/* sh->bg at x = ln tau from the spline values in c.bgraw (the team's threads
   share the fields); the caller separates this from the spline step and from
   the readers of sh->bg by barriers */
template <class C> __device__ inline void bg_fields(const C &c, double x) {
  double *b = (double *)&c.sh->bg;
  for (int q = c.rank; q < S2_NBGV; q += c.size) b[q] = bg_field(c.bgraw, q, x, c.sh->tri.lnk);
}

/* Hc and kappa_dot only (start time, TCA trigger) */
template <class C> __device__ inline void bg_hk(const C &c, double tau, double &Hc, double &kd) {
  Hc = exp(bg_col(c, SONG2_BG_LN_HC, tau));
  kd = exp(bg_col(c, SONG2_BG_LN_KAPPA_DOT, tau));
}

/* ------------------------------------------------------------------ quadratic sources */

template <class C> __device__ double coll_I(const C &c, const BgV &bg, int l, int m) {
  const Tri &t = c.sh->tri;
  auto fo1 = c.fo1, fo2 = c.fo2;
  double vb1 = fo1[SONG2_FO_V_B], vb2 = fo2[SONG2_FO_V_B], db1 = fo1[SONG2_FO_DELTA_B], db2 = fo2[SONG2_FO_DELTA_B];
  if (l == 0) {
    double vg1 = fo1[SONG2_FO_V_G], vg2 = fo2[SONG2_FO_V_G];
    return FOUR_THIRDS * t.k1_dot_k2 * (vb1 * (vg2 - vb2) + vb2 * (vg1 - vb1));
  }
  double v01 = -t.k1 * vb1, v02 = -t.k2 * vb2;
  double A1 = fo1[SONG2_FO_PSI], A2 = fo2[SONG2_FO_PSI];
  double c1, c2, spec = 0;
  if (l == 1) {
    double ub1 = -t.k1_m[m + 1] * vb1, ub2 = -t.k2_m[m + 1] * vb2;
    c1 = 4 * ub1 - c.rot_1(1, m) * c.I1r(1);
    c2 = 4 * ub2 - c.rot_2(1, m) * c.I2r(1);
    spec = 3 * (c.S(CM12, 1, m) * v01 * c.I2r(0) + c.S(CM21, 1, m) * v02 * c.I1r(0)) - 4 * (db1 * ub2 + db2 * ub1);
  } else if (l == 2) {
    double I1 = c.rot_1(2, m) * c.I1r(2), I2 = c.rot_2(2, m) * c.I2r(2);
    double E1 = c.rot_1(2, m) * c.E1r(2), E2 = c.rot_2(2, m) * c.E2r(2);
    c1 = -I1 + 0.1 * (I1 - SQRT_6 * E1);
    c2 = -I2 + 0.1 * (I2 - SQRT_6 * E2);
    spec = c.S(CM12, 2, m) * v01 * (7 * v02 - 0.5 * c.I2r(1)) + c.S(CM21, 2, m) * v02 * (7 * v01 - 0.5 * c.I1r(1));
  } else if (l == 3) {
    c1 = -c.rot_1(3, m) * c.I1r(3);
    c2 = -c.rot_2(3, m) * c.I2r(3);
    spec = 0.5 * (c.S(CM12, 3, m) * v01 * (c.I2r(2) - SQRT_6 * c.E2r(2)) +
                  c.S(CM21, 3, m) * v02 * (c.I1r(2) - SQRT_6 * c.E1r(2)));
  } else {
    c1 = -c.rot_1(l, m) * c.I1r(l);
    c2 = -c.rot_2(l, m) * c.I2r(l);
  }
  double loss = (A1 + db1) * c2 + (A2 + db2) * c1 + c.S(CM12, l, m) * v01 * c.I2r(l - 1) -
                c.S(CP12, l, m) * v01 * c.I2r(l + 1) + c.S(CM21, l, m) * v02 * c.I1r(l - 1) -
                c.S(CP21, l, m) * v02 * c.I1r(l + 1);
  return spec + loss;
}

template <class C> __device__ double coll_E(const C &c, int l, int m) {
  const Tri &t = c.sh->tri;
  auto fo1 = c.fo1, fo2 = c.fo2;
  double vb1 = fo1[SONG2_FO_V_B], vb2 = fo2[SONG2_FO_V_B], db1 = fo1[SONG2_FO_DELTA_B], db2 = fo2[SONG2_FO_DELTA_B];
  double v01 = -t.k1 * vb1, v02 = -t.k2 * vb2;
  double A1 = fo1[SONG2_FO_PSI], A2 = fo2[SONG2_FO_PSI];
  double c1, c2, spec = 0;
  if (l == 2) {
    double I1 = c.rot_1(2, m) * c.I1r(2), I2 = c.rot_2(2, m) * c.I2r(2);
    double E1 = c.rot_1(2, m) * c.E1r(2), E2 = c.rot_2(2, m) * c.E2r(2);
    c1 = -E1 - SQRT_6 * 0.1 * (I1 - SQRT_6 * E1);
    c2 = -E2 - SQRT_6 * 0.1 * (I2 - SQRT_6 * E2);
    spec = 0.5 * SQRT_6 *
           (c.S(CM12, 2, m) * v01 * (c.I2r(1) - 2 * v02) + c.S(CM21, 2, m) * v02 * (c.I1r(1) - 2 * v01));
  } else if (l == 3) {
    c1 = -c.rot_1(3, m) * c.E1r(3);
    c2 = -c.rot_2(3, m) * c.E2r(3);
    spec = -0.5 * SQRT_6 *
           (c.S(DM12, 3, m) * v01 * (c.I2r(2) - SQRT_6 * c.E2r(2)) + c.S(DM21, 3, m) * v02 * (c.I1r(2) - SQRT_6 * c.E1r(2)));
  } else {
    c1 = -c.rot_1(l, m) * c.E1r(l);
    c2 = -c.rot_2(l, m) * c.E2r(l);
  }
  double loss = (A1 + db1) * c2 + (A2 + db2) * c1 + c.S(DM12, l, m) * v01 * c.E2r(l - 1) -
                c.S(DP12, l, m) * v01 * c.E2r(l + 1) + c.S(DM21, l, m) * v02 * c.E1r(l - 1) -
                c.S(DP21, l, m) * v02 * c.E1r(l + 1);
  return spec + loss;
}

template <class C> __device__ double coll_B(const C &c, int l, int m) {
  const Tri &t = c.sh->tri;
  double v01 = -t.k1 * c.fo1[SONG2_FO_V_B], v02 = -t.k2 * c.fo2[SONG2_FO_V_B];
  double v = 0;
  if (l == 2)
    v = -0.2 * SQRT_6 *
        (c.S(DZ12, 2, m) * v01 * (c.I2r(2) - SQRT_6 * c.E2r(2)) + c.S(DZ21, 2, m) * v02 * (c.I1r(2) - SQRT_6 * c.E1r(2)));
  return v + c.S(DZ12, l, m) * v01 * c.E2r(l) + c.S(DZ21, l, m) * v02 * c.E1r(l);
}

/* Liouville part of the photon / neutrino intensity hierarchy (before the sign flip) */
template <class C> __device__ double liou_IN(const C &c, int nu, int l, int m) {
  const Tri &t = c.sh->tri;
  auto fo1 = c.fo1, fo2 = c.fo2;
  double phi1 = fo1[SONG2_FO_PHI], phi2 = fo2[SONG2_FO_PHI], psi1 = fo1[SONG2_FO_PSI], psi2 = fo2[SONG2_FO_PSI];
  double php1 = fo1[SONG2_FO_PHI_P], php2 = fo2[SONG2_FO_PHI_P];
  double k1 = t.k1, k2 = t.k2;
  double v = 0;
  if (l == 0) v = -8 * (phi1 * php2 + phi2 * php1);
  if (l == 1) v = 4 * (t.k1_m[m + 1] * psi1 * (psi2 - phi2) + t.k2_m[m + 1] * psi2 * (psi1 - phi1));
  double R1p = c.I1r(l + 1), R1m = c.I1r(l - 1), R2p = c.I2r(l + 1), R2m = c.I2r(l - 1), X1 = c.I1r(l), X2 = c.I2r(l);
  if (nu) { R1p = c.N1r(l + 1); R1m = c.N1r(l - 1); R2p = c.N2r(l + 1); R2m = c.N2r(l - 1); X1 = c.N1r(l); X2 = c.N2r(l); }
  double cm12 = c.S(CM12, l, m), cm21 = c.S(CM21, l, m), cp12 = c.S(CP12, l, m), cp21 = c.S(CP21, l, m);
  double cm11 = c.S(CM11, l, m), cm22 = c.S(CM22, l, m), cp11 = c.S(CP11, l, m), cp22 = c.S(CP22, l, m);
  double rm12 = (l - 1) * cm12, rm21 = (l - 1) * cm21, rp12 = -(l + 2) * cp12, rp21 = -(l + 2) * cp21;
  /* the same terms as the reference, grouped as in its neutrino block (perturbations2.c:11261-11277) */
  v += -4 * php1 * c.rot_2(l, m) * X2 +
       R2p * (rp12 * k1 * (phi1 + psi1) + cp22 * k2 * (phi1 + psi1) + 4 * cp12 * k1 * psi1) -
       R2m * (rm12 * k1 * (phi1 + psi1) + cm22 * k2 * (phi1 + psi1) + 4 * cm12 * k1 * psi1) -
       4 * php2 * c.rot_1(l, m) * X1 +
       R1p * (rp21 * k2 * (phi2 + psi2) + cp11 * k1 * (phi2 + psi2) + 4 * cp21 * k2 * psi2) -
       R1m * (rm21 * k2 * (phi2 + psi2) + cm11 * k1 * (phi2 + psi2) + 4 * cm21 * k2 * psi2);
  return v;
}

template <int WANT_B, class C> __device__ double liou_EB(const C &c, int l, int m) {
  const Tri &t = c.sh->tri;
  auto fo1 = c.fo1, fo2 = c.fo2;
  double phi1 = fo1[SONG2_FO_PHI], phi2 = fo2[SONG2_FO_PHI], psi1 = fo1[SONG2_FO_PSI], psi2 = fo2[SONG2_FO_PSI];
  double php1 = fo1[SONG2_FO_PHI_P], php2 = fo2[SONG2_FO_PHI_P];
  double k1 = t.k1, k2 = t.k2;
  double dm12 = c.S(DM12, l, m), dm21 = c.S(DM21, l, m), dp12 = c.S(DP12, l, m), dp21 = c.S(DP21, l, m);
  double dm11 = c.S(DM11, l, m), dm22 = c.S(DM22, l, m), dp11 = c.S(DP11, l, m), dp22 = c.S(DP22, l, m);
  double dz12 = c.S(DZ12, l, m), dz21 = c.S(DZ21, l, m), dz11 = c.S(DZ11, l, m), dz22 = c.S(DZ22, l, m);
  double km12 = (l - 1) * dm12, km21 = (l - 1) * dm21, kp12 = -(l + 2) * dp12, kp21 = -(l + 2) * dp21;
  double kz12 = -dz12, kz21 = -dz21;
  if (WANT_B)
    return -c.E2r(l) * (kz12 * k1 * (phi1 + psi1) + dz22 * k2 * (phi1 + psi1) + 4 * dz12 * k1 * psi1) -
           c.E1r(l) * (kz21 * k2 * (phi2 + psi2) + dz11 * k1 * (phi2 + psi2) + 4 * dz21 * k2 * psi2);
  return -4 * php1 * c.rot_2(l, m) * c.E2r(l) +
      c.E2r(l + 1) * (kp12 * k1 * (phi1 + psi1) + dp22 * k2 * (phi1 + psi1) + 4 * dp12 * k1 * psi1) -
      c.E2r(l - 1) * (km12 * k1 * (phi1 + psi1) + dm22 * k2 * (phi1 + psi1) + 4 * dm12 * k1 * psi1) -
      4 * php2 * c.rot_1(l, m) * c.E1r(l) +
      c.E1r(l + 1) * (kp21 * k2 * (phi2 + psi2) + dp11 * k1 * (phi2 + psi2) + 4 * dp21 * k2 * psi2) -
      c.E1r(l - 1) * (km21 * k2 * (phi2 + psi2) + dm11 * k1 * (phi2 + psi2) + 4 * dm21 * k2 * psi2);
}

template <class C> __device__ double liou_matter(const C &c, int cdm, int n, int m) {
  const Tri &t = c.sh->tri;
  auto fo1 = c.fo1, fo2 = c.fo2;
  double phi1 = fo1[SONG2_FO_PHI], phi2 = fo2[SONG2_FO_PHI], psi1 = fo1[SONG2_FO_PSI], psi2 = fo2[SONG2_FO_PSI];
  double php1 = fo1[SONG2_FO_PHI_P], php2 = fo2[SONG2_FO_PHI_P];
  double d1 = fo1[cdm ? SONG2_FO_DELTA_CDM : SONG2_FO_DELTA_B], d2 = fo2[cdm ? SONG2_FO_DELTA_CDM : SONG2_FO_DELTA_B];
  double v1 = fo1[cdm ? SONG2_FO_V_CDM : SONG2_FO_V_B], v2 = fo2[cdm ? SONG2_FO_V_CDM : SONG2_FO_V_B];
  double k1k2 = t.k1_dot_k2, k1sq = t.k1 * t.k1, k2sq = t.k2 * t.k2;
  if (n == 0)
    return 2 * k1k2 * (psi1 - phi1) * v2 + k2sq * (phi1 + psi1) * v2 + 3 * php1 * (d2 + 2 * phi2) +
           2 * k1k2 * (psi2 - phi2) * v1 + k1sq * (phi2 + psi2) * v1 + 3 * php2 * (d1 + 2 * phi1);
  return 3 * t.k1_m[m + 1] * (d2 * psi1 - 4 * v1 * php2 + phi2 * psi1) +
         3 * t.k2_m[m + 1] * (d1 * psi2 - 4 * v2 * php1 + phi1 * psi2) - 3 * psi1 * psi2 * (t.k1_m[m + 1] + t.k2_m[m + 1]);
}

/* Einstein-tensor quadratic terms (perturbations2.c:10905-11060) into qs */
/* Quadratic metric sources (perturbations2.c:10937-11029) and the first-order
   products kept for later (:11795-11809), in seven independent parts so that
   they can run on different warps: 0 phi' (Poisson), 1 phi' (longitudinal),
   2 psi and psi', 3 phi'', 4 omega' (m = 1), 5 gamma'' (m = 2), 6 products. */
template <class C> __device__ void qs_metric_part(const C &c, const BgV &bg, int part) {
  const Tri &t = c.sh->tri;
  const DevSpec &s = c.s;
  auto fo1 = c.fo1, fo2 = c.fo2;
  auto qs = c.qs;
  double phi_1 = fo1[SONG2_FO_PHI], phi_2 = fo2[SONG2_FO_PHI], psi_1 = fo1[SONG2_FO_PSI], psi_2 = fo2[SONG2_FO_PSI];
  double psi_prime_1 = fo1[SONG2_FO_PSI_P], psi_prime_2 = fo2[SONG2_FO_PSI_P];
  double phi_prime_1 = fo1[SONG2_FO_PHI_P], phi_prime_2 = fo2[SONG2_FO_PHI_P];
  double k1 = t.k1, k2 = t.k2, k = t.k, k_sq = t.k_sq, k1_sq = k1 * k1, k2_sq = k2 * k2, k1_dot_k2 = t.k1_dot_k2;
  const double *k1_m = t.k1_m, *k2_m = t.k2_m, *k1_ten_k2 = t.k1_ten_k2, *k1_ten_k1 = t.k1_ten_k1,
               *k2_ten_k2 = t.k2_ten_k2;
  double Hc = bg.Hc, Hc_sq = Hc * Hc, Hc_prime = bg.Hc_prime, a_sq = bg.a_sq;
  auto q_tt = [&]() {
    return -12 * psi_1 * psi_2 * Hc_sq + phi_1 * phi_2 * (3 * k1_dot_k2 + 4 * k1_sq + 4 * k2_sq) +
           6 * phi_prime_2 * (phi_1 - psi_1) * Hc + 6 * phi_prime_1 * (phi_2 - psi_2) * Hc - 3 * phi_prime_1 * phi_prime_2;
  };
  auto q_ss = [&](int i) {
    return phi_1 * phi_2 * (-3 * k1_ten_k2[i] - 2 * k1_ten_k1[i] - 2 * k2_ten_k2[i]) +
           psi_1 * psi_2 * (-k1_ten_k2[i] - k1_ten_k1[i] - k2_ten_k2[i]) + psi_1 * phi_2 * (k1_ten_k2[i] + k1_ten_k1[i]) +
           psi_2 * phi_1 * (k1_ten_k2[i] + k2_ten_k2[i]);
  };
  switch (part) {
  case 0:
    if (s.compute_m[0]) {
      double Q_TT = 2 * q_tt();
      qs[s.iq_phi_prime_poisson] = -Q_TT / (6 * Hc);
    }
    break;
  case 1:
    if (s.compute_m[0]) {
      double rho_dipole_1 = bg.rho_g * c.I1r(1) + bg.rho_b * fo1[SONG2_FO_DIPOLE_B] + bg.rho_cdm * fo1[SONG2_FO_DIPOLE_CDM] +
                            bg.rho_ur * c.N1r(1);
      double rho_dipole_2 = bg.rho_g * c.I2r(1) + bg.rho_b * fo2[SONG2_FO_DIPOLE_B] + bg.rho_cdm * fo2[SONG2_FO_DIPOLE_CDM] +
                            bg.rho_ur * c.N2r(1);
      double Q_ST = +2 * psi_1 * psi_2 * Hc * (k1_m[1] + k2_m[1]) - 2 * psi_1 * phi_2 * Hc * (k1_m[1]) -
                    2 * psi_2 * phi_1 * Hc * (+k2_m[1]) - 2 * phi_1 * phi_prime_2 * (k1_m[1] + 2 * k2_m[1]) -
                    2 * phi_2 * phi_prime_1 * (2 * k1_m[1] + k2_m[1]) + psi_1 * phi_prime_2 * (k1_m[1]) +
                    psi_2 * phi_prime_1 * (k2_m[1]) +
                    0.5 * a_sq * (k1_m[1] / k1 * rho_dipole_1 * (psi_2 + phi_2) + k2_m[1] / k2 * rho_dipole_2 * (psi_1 + phi_1));
      Q_ST *= 2;
      qs[s.iq_phi_prime_longitudinal] = Q_ST / (2 * k);
    }
    break;
  case 2:
    if (s.compute_m[0]) {
      double Q_SS = q_ss(2);
      double Q_SS_prime =
          (phi_prime_1 * phi_2 + phi_1 * phi_prime_2) * (-3 * k1_ten_k2[2] - 2 * k1_ten_k1[2] - 2 * k2_ten_k2[2]) +
          (psi_prime_1 * psi_2 + psi_1 * psi_prime_2) * (-k1_ten_k2[2] - k1_ten_k1[2] - k2_ten_k2[2]) +
          (psi_prime_1 * phi_2 + psi_1 * phi_prime_2) * (k1_ten_k2[2] + k1_ten_k1[2]) +
          (psi_prime_2 * phi_1 + psi_2 * phi_prime_1) * (k1_ten_k2[2] + k2_ten_k2[2]);
      Q_SS *= 2;
      Q_SS_prime *= 2;
      qs[s.iq_psi] = -Q_SS * 3 / (2 * k_sq);
      qs[s.iq_psi_prime] = -Q_SS_prime * 3 / (2 * k_sq) - Q_SS * 3 * Hc / k_sq;
    }
    break;
  case 3:
    if (s.compute_m[0]) {
      double phi_prime_prime_1 = fo1[SONG2_FO_PHI_PP], phi_prime_prime_2 = fo2[SONG2_FO_PHI_PP];
      double Q_TT = q_tt();
      double Q_TR = -12 * psi_1 * psi_2 * (Hc * Hc + 2 * Hc_prime) + psi_1 * psi_2 * (k_sq + k1_sq + k2_sq) +
                    phi_1 * phi_2 * (3 * k1_dot_k2 + 4 * k1_sq + 4 * k2_sq) + phi_1 * psi_2 * (k1_dot_k2 - 2 * k2_sq) +
                    phi_2 * psi_1 * (k1_dot_k2 - 2 * k1_sq) + 6 * (phi_prime_prime_2 + 2 * Hc * phi_prime_2) * (phi_1 - psi_1) +
                    6 * (phi_prime_prime_1 + 2 * Hc * phi_prime_1) * (phi_2 - psi_2) -
                    3 * psi_prime_2 * (4 * Hc * psi_1 + phi_prime_1) - 3 * psi_prime_1 * (4 * Hc * psi_2 + phi_prime_2) +
                    3 * phi_prime_1 * phi_prime_2;
      Q_TT *= 2;
      Q_TR *= 2;
      qs[s.iq_phi_prime_prime] = -(Q_TR + Q_TT) / 6;
    }
    break;
  case 4:
    if (s.compute_m[1]) qs[s.iq_omega_m1_prime] = SQRT_3 / k * 2 * q_ss(3);
    break;
  case 5:
    if (s.compute_m[2]) qs[s.iq_gamma_m2_prime_prime] = -2 * q_ss(4);
    break;
  default:
    qs[s.iq_vv_g] = fo1[SONG2_FO_V_G] * fo2[SONG2_FO_V_G];
    qs[s.iq_vv_ur] = fo1[SONG2_FO_V_UR] * fo2[SONG2_FO_V_UR];
    qs[s.iq_dd_b] = fo1[SONG2_FO_DELTA_B] * fo2[SONG2_FO_DELTA_B];
    qs[s.iq_vv_b] = fo1[SONG2_FO_V_B] * fo2[SONG2_FO_V_B];
    qs[s.iq_vv_cdm] = fo1[SONG2_FO_V_CDM] * fo2[SONG2_FO_V_CDM];
    qs[s.iq_vvp_b] = fo1[SONG2_FO_V_B_P] * fo2[SONG2_FO_V_B] + fo1[SONG2_FO_V_B] * fo2[SONG2_FO_V_B_P];
    qs[s.iq_vvp_cdm] = fo1[SONG2_FO_V_CDM_P] * fo2[SONG2_FO_V_CDM] + fo1[SONG2_FO_V_CDM] * fo2[SONG2_FO_V_CDM_P];
  }
}

/* One entry of the quadratic-source vector: total (qs) and collisional (qc) part. */
template <class C> __device__ void qs_entry(const C &c, const BgV &bg, int q) {
  const DevSpec &s = c.s;
  int sp = c.qs_sp[q], l = c.qs_l[q], m = c.qs_m[q];
  double lv = 0, cv = 0;
  switch (sp) {
  case SP_I:
    if (s.has_liou) lv = -liou_IN(c, 0, l, m);
    if (s.has_coll) cv = coll_I(c, bg, l, m) * bg.kappa_dot;
    break;
  case SP_E:
    if (l >= 2) {
      if (s.has_liou) lv = -liou_EB<0>(c, l, m);
      if (s.has_coll) cv = coll_E(c, l, m) * bg.kappa_dot;
    }
    break;
  case SP_B:
    if (l >= 2) {
      if (s.has_liou) lv = -liou_EB<1>(c, l, m);
      if (s.has_coll) cv = coll_B(c, l, m) * bg.kappa_dot;
    }
    break;
  case SP_N:
    if (s.has_liou) lv = -liou_IN(c, 1, l, m);
    break;
  case SP_B000:
    if (s.has_liou) lv = liou_matter(c, 0, 0, 0);
    if (s.has_coll) cv = -bg.r * coll_I(c, bg, 0, 0) * bg.kappa_dot;
    break;
  case SP_B11:
    if (s.has_liou) lv = liou_matter(c, 0, 1, m);
    if (s.has_coll) cv = -bg.r * coll_I(c, bg, 1, m) * bg.kappa_dot;
    break;
  case SP_C000:
    if (s.has_liou) lv = liou_matter(c, 1, 0, 0);
    break;
  case SP_C11:
    if (s.has_liou) lv = liou_matter(c, 1, 1, m);
    break;
  case SP_METRIC: {
    /* the metric part carried by this entry (none for the entries it fills) */
    int part = q == s.iq_phi_prime_poisson ? 0 : q == s.iq_phi_prime_longitudinal ? 1 : q == s.iq_psi ? 2
             : q == s.iq_phi_prime_prime ? 3 : q == s.iq_omega_m1_prime ? 4 : q == s.iq_gamma_m2_prime_prime ? 5
             : q == s.iq_vv_g ? 6 : -1;
    if (part >= 0) qs_metric_part(c, bg, part);
    return;
  }
  default:
    return;
  }
  c.qs[q] = lv + cv;
  c.qc[q] = cv;
}

/* Collision part only, the quantities perturb2_tca_variables takes directly
   from the interpolated first-order solution (perturbations2.c:9440-9456). */
template <class C> __device__ void qc_entry(const C &c, const BgV &bg, int q) {
  const DevSpec &s = c.s;
  int sp = c.qs_sp[q], l = c.qs_l[q], m = c.qs_m[q];
  double cv = 0.0;
  if (s.has_coll) {
    if (sp == SP_I) cv = coll_I(c, bg, l, m) * bg.kappa_dot;
    else if (sp == SP_E && l >= 2) cv = coll_E(c, l, m) * bg.kappa_dot;
    else if (sp == SP_B && l >= 2) cv = coll_B(c, l, m) * bg.kappa_dot;
    else if (sp == SP_B000) cv = -bg.r * coll_I(c, bg, 0, 0) * bg.kappa_dot;
    else if (sp == SP_B11) cv = -bg.r * coll_I(c, bg, 1, m) * bg.kappa_dot;
  }
  c.qc[q] = cv;
}

/* ------------------------------------------------------------------ prepare(tau) */

/* Background, first-order quantities and quadratic sources at tau, block-wide:
   the entries an output time or an interval start reads (qo_slot: moments up to
   the line-of-sight l, matter, metric; the others are left at zero).  Leaves
   sh->bg and the qs/qc/fo arrays ready; ends with a barrier. */
template <class C> __device__ void prepare(const C &c, double tau, int with_sources) {
  const DevSpec &s = c.s;
  const Tri &t = c.sh->tri;
  int tid = c.rank, nt = c.size;
  /* one FP64 logarithm per call, shared through the workspace */
  if (tid == 0) c.sh->lntau = log(tau);
  c.sync();
  double x = c.sh->lntau;
  for (int q = tid; q < SONG2_BG_SIZE; q += nt)
    c.bgraw[q] = spl(c.p.bg, c.p.bg_dd, s.bg_size, SONG2_BG_SIZE, s.bg_lntau0, s.bg_inv_dx, s.bg_dx2_6, q, x);
  int use_fo = with_sources && s.has_qs && !s.mode_first_order;
  for (int q = tid; q < 2 * s.nfo; q += nt) {
    int which = q >= s.nfo, qq = which ? q - s.nfo : q;
    double v = 0.0;
    if (use_fo) {
      int ik = which ? t.i2 : t.i1;
      size_t stride = (size_t)s.fo_tau_size * s.nfo;
      v = spl(c.p.fo + stride * ik, c.p.fo_dd + stride * ik, s.fo_tau_size, s.nfo, s.fo_lntau0, s.fo_inv_dx,
              s.fo_dx2_6, qq, x);
    }
    (which ? c.fo2 : c.fo1)[qq] = v;
  }
  c.sync();
  bg_fields(c, x);
  for (int q = tid; q < s.qs2_size; q += nt) {
    c.qs[q] = 0.0;
    c.qc[q] = 0.0;
  }
  c.sync();
  if (use_fo) {
    const BgV &bg = c.sh->bg;
    for (int e = tid; e < s.n_qo_slots; e += nt) {
      int q = c.qo_slot[e];
      if (q >= 0) qs_entry(c, bg, q);
    }
  }
  c.sync();
}

/* The derivs path of the reference (perturb2_quadratic_sources_at_tau,
   perturbations2.c:14366-14688): background by spline, quadratic sources by
   cubic-spline interpolation of the triplet's table; in tight coupling also the
   first-order quantities and the direct collision terms.  Ends with a barrier. */
template <class C> __device__ void prepare_table(const C &c, double tau, int ap) {
  /* ap != AP_NONE (TCA or RSA): first-order values and collision terms computed
     directly, as perturb2_tca_variables and perturb2_rsa_variables do */
  const DevSpec &s = c.s;
  const Tri &t = c.sh->tri;
  int tid = c.rank, nt = c.size;
  if (tid == 0) c.sh->lntau = log(tau);
  c.sync();
  double x = c.sh->lntau;
  for (int q = tid; q < SONG2_BG_SIZE; q += nt)
    c.bgraw[q] = spl(c.p.bg, c.p.bg_dd, s.bg_size, SONG2_BG_SIZE, s.bg_lntau0, s.bg_inv_dx, s.bg_dx2_6, q, x);
  int use = s.has_qs && !s.mode_first_order && c.qtab.p != nullptr;
  if (use) {
    double u = (x - s.fo_lntau0) * s.fo_inv_dx;
    int j0 = c.sh->qt_j0, n = c.sh->qt_n;
    int i = (int)floor(u);
    if (i < j0) i = j0;
    if (i > j0 + n - 2) i = j0 + n - 2;
    double b = u - i, a = 1.0 - b;
    double ca = (a * a * a - a) * s.fo_dx2_6, cb = (b * b * b - b) * s.fo_dx2_6;
    int nq = s.qs2_size;
    auto r0 = c.qtab + (i - j0) * 2 * nq, r1 = r0 + 2 * nq;
    /* radiation streaming: the rows of the moments with l >= 3 are not evaluated,
       so neither are their quadratic sources */
    const bool rsa = ap == AP_RSA;
    for (int q = tid; q < nq; q += nt) {
      if (rsa && c.qs_sp[q] <= SP_N && c.qs_l[q] >= 3) continue;
      c.qs[q] = a * r0[q] + b * r1[q] + ca * r0[nq + q] + cb * r1[nq + q];
    }
    if (ap) {
      size_t stride = (size_t)s.fo_tau_size * s.nfo;
      for (int q = tid; q < 2 * s.nfo; q += nt) {
        int which = q >= s.nfo, qq = which ? q - s.nfo : q;
        int ik = which ? t.i2 : t.i1;
        (which ? c.fo2 : c.fo1)[qq] =
            spl(c.p.fo + stride * ik, c.p.fo_dd + stride * ik, s.fo_tau_size, s.nfo, s.fo_lntau0, s.fo_inv_dx,
              s.fo_dx2_6, qq, x);
      }
    }
  } else {
    for (int q = tid; q < s.qs2_size; q += nt) c.qs[q] = 0.0;
  }
  if (!(use && ap))
    for (int q = tid; q < s.qs2_size; q += nt) c.qc[q] = 0.0;
  c.sync();
  bg_fields(c, x);
  c.sync();
  if (use && ap) {
    const BgV &bg = c.sh->bg;
    for (int e = tid; e < s.n_qs_slots; e += nt) {
      int q = c.qs_slot[e];
      if (q >= 0 && !(ap == AP_RSA && c.qs_sp[q] <= SP_N && c.qs_l[q] >= 3)) qc_entry(c, bg, q);
    }
    c.sync();
  }
}

/* Quadratic sources of the triplet at the first-order time nodes covering
   [tau_ini, tau_end] (exact first-order values at the nodes, background by
   spline) and their natural cubic splines in ln tau: the per-triplet table of
   perturb2_quadratic_sources_for_k1k2k (perturbations2.c:10407-10606). */
template <class C> __device__ void build_qs_table(const C &c) {
  const DevSpec &s = c.s;
  Tri &t = c.sh->tri;
  int tid = c.rank, nt = c.size;
  if (!s.has_qs || s.mode_first_order || c.qtab.p == nullptr) return;
  int N = s.fo_tau_size, nq = s.qs2_size;
  double x0 = s.fo_lntau0, dx = s.fo_dlntau, six_idx2 = 6.0 * s.fo_inv_dx * s.fo_inv_dx;
  if (tid == 0) {
    int j0 = (int)floor((log(t.tau_ini) - x0) / dx);
    int j1 = (int)ceil((log(t.tau_end) - x0) / dx);
    if (j0 < 0) j0 = 0;
    if (j0 > N - 2) j0 = N - 2;
    if (j1 > N - 1) j1 = N - 1;
    if (j1 < j0 + 1) j1 = j0 + 1;
    c.sh->qt_j0 = j0;
    c.sh->qt_n = j1 - j0 + 1;
  }
  c.sync();
  int j0 = c.sh->qt_j0, M = c.sh->qt_n;
  size_t stride = (size_t)s.fo_tau_size * s.nfo;
  const double *v1 = c.p.fo + stride * t.i1, *v2 = c.p.fo + stride * t.i2;
  for (int j = 0; j < M; ++j) {
    double x = x0 + (j0 + j) * dx;
    for (int q = tid; q < SONG2_BG_SIZE; q += nt)
      c.bgraw[q] = spl(c.p.bg, c.p.bg_dd, s.bg_size, SONG2_BG_SIZE, s.bg_lntau0, s.bg_inv_dx, s.bg_dx2_6, q, x);
    for (int q = tid; q < 2 * s.nfo; q += nt) {
      int which = q >= s.nfo, qq = which ? q - s.nfo : q;
      (which ? c.fo2 : c.fo1)[qq] = __ldg((which ? v2 : v1) + (size_t)(j0 + j) * s.nfo + qq);
    }
    c.sync();
    bg_fields(c, x);
    c.sync();
    {
      const BgV &bg = c.sh->bg;
      for (int e = tid; e < s.n_qs_slots; e += nt) {
        int q = c.qs_slot[e];
        if (q >= 0) qs_entry(c, bg, q);
      }
    }
    c.sync();
    auto row = c.qtab + j * 2 * nq;
    for (int q = tid; q < nq; q += nt) row[q] = c.qs[q];
  }
  c.sync();
  /* natural spline per entry: Thomas sweeps along the nodes (same recurrence as
     song2_spline_uniform; spl_c[j] = 1/(4 - spl_c[j-1])) */
  for (int q = tid; q < nq; q += nt) {
    double prev = 0.0;
    c.qtab[nq + q] = 0.0;
    for (int j = 1; j < M - 1; ++j) {
      double ym = c.qtab[(j - 1) * 2 * nq + q], y0 = c.qtab[j * 2 * nq + q];
      double yp = c.qtab[(j + 1) * 2 * nq + q];
      double r = (yp - 2.0 * y0 + ym) * six_idx2;
      /* 1 / (4 - spl_c[j-1]) = spl_c[j] */
      prev = (r - prev) * __ldg(c.p.spl_c + j);
      c.qtab[j * 2 * nq + nq + q] = prev;
    }
    c.qtab[(M - 1) * 2 * nq + nq + q] = 0.0;
    for (int j = M - 2; j >= 1; --j)
      c.qtab[j * 2 * nq + nq + q] -= __ldg(c.p.spl_c + j) * c.qtab[(j + 1) * 2 * nq + nq + q];
  }
  c.sync();
}

/* ------------------------------------------------------------------ workspace */

/* perturb2_rsa_variables (perturbations2.c:9773-10164), rsa2_MD without the
   quadratic-source derivative terms (compute_quadsources_derivatives = no),
   applied after the Einstein equations as perturbations2.c:8777-8809 does: the
   photon and neutrino monopoles and dipoles, and the photon collision dipole of
   the baryon equation; the m = 1 dipoles are zero (:10094-10098).  Kept out of
   line: the RSA interval is the rare path, and inlining it into every
   right-hand-side evaluation costs registers in the NDF loop. */
template <class Y, class C> __device__ __noinline__ void rsa_moments(const C &c, const Y &y, int lin, WS &w, int m) {
  const DevSpec &s = c.s;
  const Tri &t = c.sh->tri;
  const BgV &bg = c.sh->bg;
  auto qs = c.qs, qc = c.qc, fo1 = c.fo1, fo2 = c.fo2;
  double k = t.k, Hc = bg.Hc, kd = bg.kappa_dot;
  double I1 = 0.0, N1 = 0.0;
  /* MD_with_reio: tau_c = 1/kappa', tau_c'/tau_c = -kappa''/kappa' = -(d ln kappa'/d ln tau)/tau */
  const int reio = s.rsa == SONG2_RSA_MD_WITH_REIO;
  double tau_c = 1.0 / kd, tcd_over_tc = 0.0;
  if (reio) {
    double x = c.sh->lntau;
    tcd_over_tc = -spl_dx(c.p.bg, c.p.bg_dd, s.bg_size, SONG2_BG_SIZE, s.bg_lntau0, s.bg_dlntau,
                          SONG2_BG_LN_KAPPA_DOT, x) / exp(x);
  }
  double vpot_g_1 = lin ? 0.0 : fo1[SONG2_FO_V_G], vpot_g_2 = lin ? 0.0 : fo2[SONG2_FO_V_G];
  double delta_g_1 = lin ? 0.0 : fo1[SONG2_FO_DELTA_G], delta_g_2 = lin ? 0.0 : fo2[SONG2_FO_DELTA_G];
  double vpot_ur_1 = lin ? 0.0 : fo1[SONG2_FO_V_UR], vpot_ur_2 = lin ? 0.0 : fo2[SONG2_FO_V_UR];
  double delta_ur_1 = lin ? 0.0 : fo1[SONG2_FO_DELTA_UR], delta_ur_2 = lin ? 0.0 : fo2[SONG2_FO_DELTA_UR];
  if (m == 0) {
    double v_dot_v_g = -t.k1_dot_k2 * vpot_g_1 * vpot_g_2, v_dot_v_ur = -t.k1_dot_k2 * vpot_ur_1 * vpot_ur_2;
    int lm00 = c.LM(0, 0), lm10 = c.LM(1, 0);
    double qsI00 = lin ? 0.0 : qs[s.iq_g + lm00], qcI00 = lin ? 0.0 : qc[s.iq_g + lm00];
    double qsI10 = lin ? 0.0 : qs[s.iq_g + lm10], qcI10 = lin ? 0.0 : qc[s.iq_g + lm10];
    double qsN00 = lin ? 0.0 : qs[s.iq_ur + lm00], qsN10 = lin ? 0.0 : qs[s.iq_ur + lm10];
    double quadL_I_10 = -(qsI10 - qcI10), quadL_N_10 = -qsN10;
    double delta_g_rsa = -4 * w.psi + quadL_I_10 / k;
    if (reio) {
      delta_g_rsa += -FOUR_THIRDS * getb(c, y, 1, 0) / (k * tau_c);
      delta_g_rsa += -(qcI10 / kd) / (k * tau_c);
    }
    w.I_00 = delta_g_rsa + 8 * v_dot_v_g / 3;
    double delta_ur_rsa = -4 * w.psi + quadL_N_10 / k;
    w.N_00 = delta_ur_rsa + 8 * v_dot_v_ur / 3;
    double psi_prime_quad = lin ? 0.0 : qs[s.iq_psi_prime] - 2 * Hc * qs[s.iq_psi];
    double psi_prime = w.phi_prime + psi_prime_quad;
    double u_g_1 = -t.k1_m[1] * vpot_g_1, u_g_2 = -t.k2_m[1] * vpot_g_2;
    double u_ur_1 = -t.k1_m[1] * vpot_ur_1, u_ur_2 = -t.k2_m[1] * vpot_ur_2;
    double quadL_I_00 = -(qsI00 - qcI00), quadL_N_00 = -qsN00;
    double u_g = 3 / k * (w.phi_prime + psi_prime);
    u_g += -(u_g_1 * delta_g_2 + u_g_2 * delta_g_1) - 3 / (4 * k) * quadL_I_00;
    if (reio) {
      double quadC_I_00 = qcI00 / kd, quadC_I_10 = qcI10 / kd, tau_c_dot = tcd_over_tc * tau_c;
      u_g += 1 / (k * tau_c) *
             (-(3 * Hc + tcd_over_tc) / k * getb(c, y, 1, 0) + 9 * w.psi + 3 / 4. * quadC_I_00 -
              3 * tau_c_dot * quadC_I_10 / (4 * k * tau_c));
    }
    I1 = 4 * (u_g + delta_g_1 * u_g_2 + delta_g_2 * u_g_1);
    double u_ur = 3 / k * (w.phi_prime + psi_prime);
    u_ur += -(u_ur_1 * delta_ur_2 + u_ur_2 * delta_ur_1) - 3 / (4 * k) * quadL_N_00;
    N1 = 4 * (u_ur + delta_ur_1 * u_ur_2 + delta_ur_2 * u_ur_1);
  }
  w.I_1m[m] = I1;
  w.C_1m[m] = kd * (FOUR_THIRDS * getb(c, y, 1, m) - I1);
  w.N_1m[m] = N1;
}

/* The workspace of perturb2_workspace_at_tau / perturb2_tca_variables /
   perturb2_einstein for one azimuthal number m in {0, 1, 2}: every field of WS
   belongs to exactly one m, so the three parts can be evaluated side by side. */
template <class Y, class C> __device__ void compute_ws_m(const C &c, int ap, const Y &y, int lin, WS &w, int m) {
  const DevSpec &s = c.s;
  const Tri &t = c.sh->tri;
  const BgV &bg = c.sh->bg;
  auto qs = c.qs, qc = c.qc, fo1 = c.fo1, fo2 = c.fo2;
  double k = t.k, Hc = bg.Hc, kd = bg.kappa_dot, r = bg.r;
  w.N_1m[m] = w.I_1m[m] = w.I_2m[m] = w.E_2m[m] = w.B_2m[m] = w.C_1m[m] = 0;
  w.b_22m[m] = w.cdm_22m[m] = 0;
  w.I_1m_tca1[m] = w.I_2m_tca1[m] = w.E_2m_tca1[m] = w.B_2m_tca1[m] = w.Pi_tca1[m] = 0;
  if (m == 0) {
    w.I_00 = w.N_00 = 0;
    w.b_200 = w.cdm_200 = 0;
    w.psi = w.phi_prime = w.phi_pp = 0;
  }
  if (m == 1) w.omega_m1_prime = 0;
  if (m == 2) w.gamma_m2_pp = 0;
  if (!s.compute_m[m]) return;
  const int rsa = ap == AP_RSA;
  auto gN = [&](int l_, int m_) { return rsa ? 0.0 : getN(c, y, l_, m_); };
  if (m == 0) {
    w.I_00 = getI(c, ap, y, 0, 0);
    w.N_00 = gN(0, 0);
  }
  if (m <= 1) {
    w.I_1m[m] = getI(c, ap, y, 1, m);
    w.N_1m[m] = gN(1, m);
    w.C_1m[m] = kd * (FOUR_THIRDS * getb(c, y, 1, m) - getI(c, ap, y, 1, m));
  }
  w.I_2m[m] = getI(c, ap, y, 2, m);
  w.E_2m[m] = getE(c, ap, y, 2, m);
  w.B_2m[m] = getB(c, ap, y, 2, m);
  double vv_b = lin ? 0.0 : qs[s.iq_vv_b], vv_cdm = lin ? 0.0 : qs[s.iq_vv_cdm];
  if (m == 0) {
    w.b_200 = -2 * t.k1_dot_k2 * vv_b;
    w.cdm_200 = -2 * t.k1_dot_k2 * vv_cdm;
  }
  w.b_22m[m] = 15 * t.k1_ten_k2[m + 2] * vv_b;
  w.cdm_22m[m] = 15 * t.k1_ten_k2[m + 2] * vv_cdm;
  if (ap == AP_TCA) {
    /* perturb2_tca_variables (perturbations2.c:9374-9738) */
    double tau_c = bg.inv_kd;
    double vpot_g_1 = lin ? 0.0 : fo1[SONG2_FO_V_G], vpot_g_2 = lin ? 0.0 : fo2[SONG2_FO_V_G];
    double delta_g_1 = lin ? 0.0 : fo1[SONG2_FO_DELTA_G], delta_g_2 = lin ? 0.0 : fo2[SONG2_FO_DELTA_G];
    double vpot_b_1 = lin ? 0.0 : fo1[SONG2_FO_V_B], vpot_b_2 = lin ? 0.0 : fo2[SONG2_FO_V_B];
    double vpot_b_1_prime = lin ? 0.0 : fo1[SONG2_FO_V_B_P], vpot_b_2_prime = lin ? 0.0 : fo2[SONG2_FO_V_B_P];
    double c1tca = 0.0;
    if (m <= 1) {
      double delta_b_1 = lin ? 0.0 : fo1[SONG2_FO_DELTA_B], delta_b_2 = lin ? 0.0 : fo2[SONG2_FO_DELTA_B];
      double delta_b_1_prime = lin ? 0.0 : fo1[SONG2_FO_DELTA_B_P], delta_b_2_prime = lin ? 0.0 : fo2[SONG2_FO_DELTA_B_P];
      double delta_g = 0.0;
      if (m == 0) {
        double v_dot_v_g = -t.k1_dot_k2 * vpot_g_1 * vpot_g_2;
        delta_g = w.I_00 - 8 / 3. * v_dot_v_g;
      }
      double u_g_1 = -t.k1_m[m + 1] * vpot_g_1, u_g_2 = -t.k2_m[m + 1] * vpot_g_2;
      double u_b_1 = -t.k1_m[m + 1] * vpot_b_1, u_b_2 = -t.k2_m[m + 1] * vpot_b_2;
      double u_b_1_prime = -t.k1_m[m + 1] * vpot_b_1_prime, u_b_2_prime = -t.k2_m[m + 1] * vpot_b_2_prime;
      double u_b = getb(c, y, 1, m) * ONE_THIRD - delta_b_1 * u_b_2 - delta_b_2 * u_b_1;
      double qcI1 = lin ? 0.0 : qc[s.iq_g + c.LM(1, m)];
      double qsI1 = lin ? 0.0 : qs[s.iq_g + c.LM(1, m)];
      double qsb = lin ? 0.0 : qs[s.iq_b11[m]], qcb = lin ? 0.0 : qc[s.iq_b11[m]];
      double quadC_u_g_m = qcI1 * tau_c * 0.25 + (u_b_1 * delta_b_2 + u_b_2 * delta_b_1) - (u_g_1 * delta_g_2 + u_g_2 * delta_g_1);
      double delta_u_prime_b_m = delta_b_1_prime * u_b_2 + delta_b_2_prime * u_b_1 + delta_b_1 * u_b_2_prime +
                                 delta_b_2 * u_b_1_prime;
      double quadL_b_11M = -(qsb - qcb), quadL_I_1M = -(qsI1 - qcI1);
      double quadL_diff = quadL_b_11M * ONE_THIRD - quadL_I_1M * 0.25 - FOUR_THIRDS * delta_u_prime_b_m * 0.25 +
                          Hc * (u_b_1 * delta_b_2 + u_b_2 * delta_b_1);
      /* R / (1 + R) with R = 3 / (4 r) */
      double Rf = 1.0 / (1.0 + FOUR_THIRDS * r);
      double om = (m == 1) ? y(s.idx_omega) : 0.0;
      double core = Hc * (u_b + om) + k * 0.25 * (m == 0 ? delta_g : 0) + quadL_diff;
      double U_slip = -quadC_u_g_m - Rf * tau_c * core;
      c1tca = -qcI1 - 4 * Rf * core;
      double u_g_tca1 = u_b - U_slip;
      w.I_1m_tca1[m] = 4 * (u_g_tca1 + delta_g_1 * u_g_2 + delta_g_2 * u_g_1);
    }
    {
      double v_ten_v_g = -t.k1_ten_k2[m + 2] * vpot_g_1 * vpot_g_2;
      double v_ten_v_b_prime = -t.k1_ten_k2[m + 2] * (vpot_b_1 * vpot_b_2_prime + vpot_b_2 * vpot_b_1_prime);
      double gp = (m == 2) ? y(s.idx_gammap) : 0.0;
      double cm2 = c.cmin(2, m, m);
      double shear = 8 / 45. * tau_c * (-k * w.I_1m_tca1[m] * cm2 - 4 * gp);
      double quadC_I_2M = (lin ? 0.0 : qc[s.iq_g + c.LM(2, m)]) * tau_c;
      double quadC_E_2M = 0, quadC_B_2M = 0, quadL_E_2M = 0;
      double quadL_I_2M = lin ? 0.0 : -(qs[s.iq_g + c.LM(2, m)] - qc[s.iq_g + c.LM(2, m)]);
      if (s.has_pol && !lin) {
        quadC_E_2M = qc[s.iq_E + c.LM(2, m)] * tau_c;
        quadC_B_2M = (m != 0 ? qc[s.iq_B + c.LM(2, m)] : 0.0) * tau_c;
        quadL_E_2M = -(qs[s.iq_E + c.LM(2, m)] - qc[s.iq_E + c.LM(2, m)]);
      }
      shear += 8 / 45. * (-quadC_I_2M + SQRT_6 / 4 * quadC_E_2M - 15 * v_ten_v_g);
      shear += 8 / 45. * tau_c * (quadL_I_2M - SQRT_6 / 4 * quadL_E_2M - 20 * v_ten_v_b_prime);
      if (!s.has_pol)
        shear = -4 / 27. * (quadC_I_2M + 18 * v_ten_v_g -
                            tau_c * (-20 * v_ten_v_b_prime - k * w.I_1m[m] * cm2 - 4 * gp + quadL_I_2M));
      w.I_2m_tca1[m] = -15 / 2. * shear - 20 * v_ten_v_g;
      if (s.has_pol) {
        w.Pi_tca1[m] = (w.I_2m_tca1[m] - SQRT_6 * (quadC_E_2M - tau_c * quadL_E_2M)) * 0.25;
        w.E_2m_tca1[m] = -SQRT_6 * w.Pi_tca1[m] + quadC_E_2M - tau_c * quadL_E_2M;
        w.B_2m_tca1[m] = (m != 0 ? quadC_B_2M : 0.0);
      } else {
        w.Pi_tca1[m] = 0.1 * w.I_2m_tca1[m];
      }
    }
    /* the TCA values replace the evolved ones only now (perturbations2.c:8999-9020) */
    if (m <= 1) {
      w.I_1m[m] = w.I_1m_tca1[m];
      w.C_1m[m] = c1tca;
    }
    w.I_2m[m] = w.I_2m_tca1[m];
    if (s.has_pol) {
      w.E_2m[m] = w.E_2m_tca1[m];
      w.B_2m[m] = (m != 0 ? w.B_2m_tca1[m] : 0.0);
    }
  }
  /* perturb2_einstein (perturbations2.c:8484-8814), Newtonian gauge, phi_eq = huang */
  double a_sq = bg.a_sq, k_sq = t.k_sq;
  if (m == 0) {
    double rho_quadrupole = bg.rho_g * w.I_2m[0] + bg.rho_b * w.b_22m[0] + bg.rho_cdm * w.cdm_22m[0] + bg.rho_ur * gN(2, 0);
    double rho_mono_b = bg.rho_b * getb(c, y, 0, 0), rho_mono_c = bg.rho_cdm * getc(c, y, 0, 0);
    double phi = y(s.idx_phi);
    w.psi = phi - 0.6 * bg.a2_k2 * rho_quadrupole + (lin ? 0.0 : qs[s.iq_psi]);
    w.phi_prime = y(s.idx_phip);
    w.phi_pp = k_sq * ONE_THIRD * (w.psi - 2 * phi) - Hc * (3 * w.phi_prime) - 2 * w.psi * (Hc * Hc + bg.Hc_prime) -
               a_sq * 0.5 * (rho_mono_b + rho_mono_c) + (lin ? 0.0 : qs[s.iq_phi_prime_prime]);
  } else if (m == 1) {
    double rq1 = bg.rho_g * w.I_2m[1] + bg.rho_b * w.b_22m[1] + bg.rho_cdm * w.cdm_22m[1] + bg.rho_ur * gN(2, 1);
    w.omega_m1_prime = -2 * Hc * y(s.idx_omega) + (0.4 * SQRT_3) * t.inv_k * a_sq * rq1 + (lin ? 0.0 : qs[s.iq_omega_m1_prime]);
  } else {
    double rq2 = bg.rho_g * w.I_2m[2] + bg.rho_b * w.b_22m[2] + bg.rho_cdm * w.cdm_22m[2] + bg.rho_ur * gN(2, 2);
    w.gamma_m2_pp = -2 * Hc * y(s.idx_gammap) - k_sq * y(s.idx_gamma) - 0.4 * a_sq * rq2 +
                    (lin ? 0.0 : qs[s.iq_gamma_m2_prime_prime]);
  }
  if (rsa && m <= 1) rsa_moments(c, y, lin, w, m);
}

/* the whole workspace, one thread */
template <class Y, class C> __device__ void compute_ws(const C &c, int ap, const Y &y, int lin, WS &w) {
  for (int m = 0; m < 3; ++m) compute_ws_m(c, ap, y, lin, w, m);
}

/* the workspace into sh->ws, the three m parts on three threads of the team */
template <class Y, class C> __device__ void compute_ws_team(const C &c, int ap, const Y &y) {
  if (c.size >= 96) {
    /* lane 0 of warps 0, 1, 2: the three parts run on different schedulers */
    if ((c.rank & 31) == 0 && c.rank < 96) compute_ws_m(c, ap, y, 0, c.sh->ws, c.rank >> 5);
  } else {
    for (int m = c.rank; m < 3; m += c.size) compute_ws_m(c, ap, y, 0, c.sh->ws, m);
  }
}

/* ------------------------------------------------------------------ derivs rows */

/* every row except phi' (which needs two other rows, see row() below) */
template <class Y, class C>
__device__ double row_h(const C &c, int ap, int i, const Y &y, const WS &w, int lin, double tau) {
  const DevSpec &s = c.s;
  const Tri &t = c.sh->tri;
  const BgV &bg = c.sh->bg;
  int sp = c.eq_sp[i], l = c.eq_l[i], m = c.eq_m[i];
  double k = t.k, kd = bg.kappa_dot, Hc = bg.Hc;
  double mc = s.compute_m[0] ? -3 * w.phi_prime : 0.0, me = s.compute_m[0] ? k * w.psi : 0.0;
  double omp = w.omega_m1_prime, om = s.compute_m[1] ? y(s.idx_omega) : 0.0;
  double gp = s.compute_m[2] ? y(s.idx_gammap) : 0.0;
  int use_qs = !lin && s.has_qs;
  double d = 0.0;
  if (ap == AP_RSA && sp <= SP_N) return 0.0;
  switch (sp) {
  case SP_I: {
    if (ap == AP_TCA && l >= 1) return 0.0;
    if (ap == AP_NONE && l == s.l_max_g) {
      double cc = (l + 1 + m) * bg.inv_ktau;
      d = k * (s.cl_I[m] * getI(c, ap, y, l - 1, m) - cc * getI(c, ap, y, l, m)) - kd * getI(c, ap, y, l, m);
    } else if (l == 0) {
      d = -FOUR_THIRDS * (k * w.I_1m[0] / 4 + mc);
    } else if (l == 1) {
      d = k * (c.cmin(1, m, m) * w.I_00 - c.cplu(1, m, m) * w.I_2m[m]) + w.C_1m[m];
      if (m == 0) d += 4 * me;
      if (m == 1) d += -4 * omp;
    } else if (l == 2) {
      double Pi = 0.1 * (w.I_2m[m] - SQRT_6 * w.E_2m[m]);
      d = k * (c.cmin(2, m, m) * w.I_1m[m] - c.cplu(2, m, m) * getI(c, ap, y, 3, m)) - kd * (w.I_2m[m] - Pi);
      if (m == 2) d += 4 * gp;
    } else {
      d = k * (c.cmin(l, m, m) * getI(c, ap, y, l - 1, m) - c.cplu(l, m, m) * getI(c, ap, y, l + 1, m)) -
          kd * getI(c, ap, y, l, m);
    }
    if (use_qs) d += c.qs[s.iq_g + c.LM(l, m)];
    return d;
  }
  case SP_E: {
    if (ap != AP_NONE) return 0.0;
    if (l == s.l_max_pol) {
      double cc = (l + 3) * bg.inv_ktau;
      d = k * (s.cl_P[m] * getE(c, ap, y, l - 1, m) - cc * getE(c, ap, y, l, m) - s.cmix_P[m] * getB(c, ap, y, l, m)) -
          kd * getE(c, ap, y, l, m);
    } else if (l == 2) {
      double Pi = 0.1 * (w.I_2m[m] - SQRT_6 * w.E_2m[m]);
      d = k * (-c.dplu(2, m, m) * getE(c, ap, y, 3, m) - c.dzer(2, m, m) * w.B_2m[m]) - kd * (w.E_2m[m] + SQRT_6 * Pi);
    } else {
      d = k * (c.dmin(l, m, m) * getE(c, ap, y, l - 1, m) - c.dplu(l, m, m) * getE(c, ap, y, l + 1, m) -
               c.dzer(l, m, m) * getB(c, ap, y, l, m)) -
          kd * getE(c, ap, y, l, m);
    }
    if (use_qs) d += c.qs[s.iq_E + c.LM(l, m)];
    return d;
  }
  case SP_B: {
    if (ap != AP_NONE) return 0.0;
    if (l == s.l_max_pol) {
      double cc = (l + 3) * bg.inv_ktau;
      d = k * (s.cl_P[m] * getB(c, ap, y, l - 1, m) - cc * getB(c, ap, y, l, m) + s.cmix_P[m] * getE(c, ap, y, l, m)) -
          kd * getB(c, ap, y, l, m);
    } else {
      d = k * (c.dmin(l, m, m) * getB(c, ap, y, l - 1, m) - c.dplu(l, m, m) * getB(c, ap, y, l + 1, m) +
               c.dzer(l, m, m) * getE(c, ap, y, l, m)) -
          kd * getB(c, ap, y, l, m);
    }
    if (use_qs) d += c.qs[s.iq_B + c.LM(l, m)];
    return d;
  }
  case SP_N: {
    if (l == s.l_max_ur) {
      double cc = (l + 1 + m) * bg.inv_ktau;
      d = k * (s.cl_N[m] * getN(c, y, l - 1, m) - cc * getN(c, y, l, m));
    } else if (l == 0) {
      d = -FOUR_THIRDS * (k * w.N_1m[0] * 0.25 + mc);
    } else if (l == 1) {
      d = k * (c.cmin(1, m, m) * w.N_00 - c.cplu(1, m, m) * getN(c, y, 2, m));
      if (m == 0) d += 4 * me;
      if (m == 1) d += -4 * omp;
    } else {
      d = k * (c.cmin(l, m, m) * getN(c, y, l - 1, m) - c.cplu(l, m, m) * getN(c, y, l + 1, m));
      if (l == 2 && m == 2) d += 4 * gp;
    }
    if (use_qs) d += c.qs[s.iq_ur + c.LM(l, m)];
    return d;
  }
  case SP_B000:
    d = -(k * getb(c, y, 1, 0) * ONE_THIRD + mc) - Hc * w.b_200;
    if (use_qs) d += c.qs[s.iq_b000];
    return d;
  case SP_B11:
    d = -Hc * getb(c, y, 1, m) + k * (c.cmin(1, m, m) * w.b_200 - c.cplu(1, m, m) * w.b_22m[m]) - bg.r * w.C_1m[m];
    if (m == 0) d += 3 * me;
    if (m == 1) d += -3 * (omp + Hc * om);
    if (use_qs) d += c.qs[s.iq_b11[m]];
    return d;
  case SP_C000:
    d = -(k * getc(c, y, 1, 0) * ONE_THIRD + mc) - Hc * w.cdm_200;
    if (use_qs) d += c.qs[s.iq_c000];
    return d;
  case SP_C11:
    d = -Hc * getc(c, y, 1, m) + k * (c.cmin(1, m, m) * w.cdm_200 - c.cplu(1, m, m) * w.cdm_22m[m]);
    if (m == 0) d += 3 * me;
    if (m == 1) d += -3 * (omp + Hc * om);
    if (use_qs) d += c.qs[s.iq_c11[m]];
    return d;
  case SP_PHI:
    return w.phi_prime;
  case SP_OMEGA:
    return omp;
  case SP_GAMMA:
    return gp;
  case SP_GAMMAP:
    return w.gamma_m2_pp;
  }
  return 0.0;
}


/* psi' given the time derivatives of the photon and neutrino quadrupoles
   (perturb2_compute_psi_prime, perturbations2.c:10188-10383); in tight coupling
   the photon quadrupole derivative is the TCA one. */
template <class Y, class C>
__device__ double psi_prime_of(const C &c, int ap, const Y &y, const WS &w, int lin, double dI20, double dN20) {
  const DevSpec &s = c.s;
  const Tri &t = c.sh->tri;
  const BgV &bg = c.sh->bg;
  double k = t.k, kd = bg.kappa_dot, Hc = bg.Hc;
  int use_qs = !lin && s.has_qs;
  if (ap == AP_TCA)
    dI20 = 2 / 3. * k * w.I_1m_tca1[0] - kd * (w.I_2m_tca1[0] - w.Pi_tca1[0]) + (use_qs ? c.qs[s.iq_g + c.LM(2, 0)] : 0.0);
  double rqp = bg.rho_g * dI20 + bg.rho_ur * dN20;
  if (!lin) {
    rqp += bg.rho_b * 15 * t.k1_ten_k2[2] * c.qs[s.iq_vvp_b];
    rqp += bg.rho_cdm * 15 * t.k1_ten_k2[2] * c.qs[s.iq_vvp_cdm];
  }
  return w.phi_prime - 2 * Hc * (w.psi - y(s.idx_phi)) -
         0.6 * bg.a2_k2 * (rqp + Hc * bg.rho_b * w.b_22m[0] + Hc * bg.rho_cdm * w.cdm_22m[0]) +
         (lin ? 0.0 : c.qs[s.iq_psi_prime]);
}

/* Row i of dy = f(tau, y).  The phi' row is phi'' = (Einstein part) - Hc psi',
   where psi' needs the I_20 and N_20 rows. */
template <class Y, class C>
__device__ double row(const C &c, int ap, int i, const Y &y, const WS &w, int lin, double tau) {
  if (c.eq_sp[i] != SP_PHIP) return row_h(c, ap, i, y, w, lin, tau);
  /* in RSA the reference's dI(2,0) and dN(2,0) index the photon and neutrino
     blocks, which are empty then, at lm(2,0) = the size of the baryon block: both
     read the CDM density row (perturbations2.c:6853-6891, 10253, 10304) */
  double dI20 = ap == AP_TCA ? 0.0 : row_h(c, ap, ap == AP_RSA ? c.s.idx_c000 : c.idx_I[c.LM(2, 0)], y, w, lin, tau);
  double dN20 = row_h(c, ap, ap == AP_RSA ? c.s.idx_c000 : c.idx_N[c.LM(2, 0)], y, w, lin, tau);
  return w.phi_pp - c.sh->bg.Hc * psi_prime_of(c, ap, y, w, lin, dI20, dN20);
}

/* Row of a hierarchy moment with l >= 3 from its table entry (GenRow): the same
   free-streaming, Thomson and closure terms as row_h, along one code path for
   every species, l and m.  Zero where an approximation drops the moment (tight
   coupling: I and E, B; radiation streaming: all four). */
template <class Y, class C> __device__ __forceinline__ double gen_row(const C &c, int ap, const GenRow &r, const Y &y) {
  if (ap == AP_RSA || (ap == AP_TCA && r.kind != 3)) return 0.0;
  const BgV &bg = c.sh->bg;
  double yi = y(r.i);
  double d = c.sh->tri.k * (r.c1 * y(r.j1) + r.c2 * y(r.j2) + r.c3 * y(r.j3) - r.cd * bg.inv_ktau * yi);
  if (r.kind != 3) d -= bg.kappa_dot * yi;
  if (c.s.has_qs) d += c.qs[r.q];
  return d;
}

/* the table entry of chain row e through the read-only cache */
template <class C> __device__ inline GenRow load_gen(const C &c, int e) {
  const GenRow *g = c.ct.gen + e;
  GenRow r;
  r.c1 = __ldg(&g->c1); r.c2 = __ldg(&g->c2); r.c3 = __ldg(&g->c3); r.cd = __ldg(&g->cd);
  r.i = __ldg(&g->i); r.j1 = __ldg(&g->j1); r.j2 = __ldg(&g->j2); r.j3 = __ldg(&g->j3);
  r.q = __ldg(&g->q); r.kind = __ldg(&g->kind);
  return r;
}

/* dy = f(tau, y): block-wide; prepare(tau) must have run.  The core rows (row(),
   row_slot order) and the chain rows (GenRow table) share one index space over
   the team's threads.  Ends with a barrier. */
template <class C, class A, class B> __device__ void rhs(const C &c, int ap, double tau, A y, B dy) {
  const DevSpec &s = c.s;
  auto yv = yvec(y);
  compute_ws_team(c, ap, yv);
  c.sync();
  for (int e = c.rank; e < s.n_row_slots + s.n_gen; e += c.size) {
    if (e < s.n_row_slots) {
      int i = c.row_slot[e];
      if (i >= 0) dy[i] = row(c, ap, i, yv, c.sh->ws, 0, tau);
    } else if (ap == AP_RSA) {
      /* radiation streaming: the moments with l >= 3 are frozen, their rows zero */
      dy[__ldg(&c.ct.gen[e - s.n_row_slots].i)] = 0.0;
    } else {
      GenRow r = load_gen(c, e - s.n_row_slots);
      dy[r.i] = gen_row(c, ap, r, yv);
    }
  }
  c.sync();
}

/* One simplified-Newton right-hand side: rows of f(tau, y) as in rhs(), each
   thread turning its row straight into the residual del = h/(gamma) f - (psi +
   dif_{k+1}) and the solve vector in the iteration-matrix precision.  Ends with a
   barrier. */
template <typename T, class C, class A> __device__ void newton_rhs(const C &c, int ap, double tau, A y, double hinvGak) {
  const DevSpec &s = c.s;
  auto yv = yvec(y);
  compute_ws_team(c, ap, yv);
  c.sync();
  PH_MARK(c, PH_WS);
  auto x = c.template xsol<T>();
  for (int e = c.rank; e < s.n_row_slots + s.n_gen; e += c.size) {
    int i;
    double fi;
    if (e < s.n_row_slots) {
      i = c.row_slot[e];
      if (i < 0) continue;
      fi = row(c, ap, i, yv, c.sh->ws, 0, tau);
    } else if (ap == AP_RSA) {
      i = __ldg(&c.ct.gen[e - s.n_row_slots].i);
      fi = 0.0;
    } else {
      GenRow r = load_gen(c, e - s.n_row_slots);
      i = r.i;
      fi = gen_row(c, ap, r, yv);
    }
    x[i] = (T)(hinvGak * fi - (c.psiv[i] + c.difkp1[i]));
  }
  c.sync();
  PH_MARK(c, PH_ROWS);
}

/* ------------------------------------------------------------------ iteration matrix */

/* The iteration matrix M = I - h gamma J of an NDF step is block diagonal in m
   (azimuthal modes never couple).  Within an m block the state splits into a
   dense core (metric and matter variables and the moments with l <= 2, at most
   S2_MAXCORE entries) and up to three chains of moments with l >= 3: I, E
   (paired with B in blocks that have B) and N.  Free streaming couples a moment
   only to the same species at l - 1 and l + 1 (and E to B at the same l); the
   Thomson term and the closure stay within one l; only the l = 3 node of a chain
   couples to the core (to its l = 2 neighbours, and to psi' through the l = 2
   rows).  So every chain is block tridiagonal with 1 x 1 or 2 x 2 blocks, and
       M = [ C  F ]    C: core x core, T: the chains, F: the core rows on the
           [ E  T ]    chains' first nodes, E: the first nodes' rows on the core.
   The factorisation eliminates each chain from its last node upwards,
       Theta_last = D_last,   Theta_k = D_k - U_k Theta_(k+1)^-1 L_(k+1),
   with D, L, U the diagonal, lower and upper blocks of M, and inverts the core's
   Schur complement S = C - sum over chains of F Theta_0^-1 E by Gauss-Jordan
   elimination with partial pivoting.  A chain needs no pivoting: the coupling
   coefficients of l -> l + 1 and of l + 1 -> l are positive and enter M with
   opposite signs, so U_k L_(k+1) is a negative multiple of the identity (E and B
   share their coefficients), and the Thomson and E-B terms add a positive
   diagonal and a skew part; every Theta_k therefore keeps a positive definite
   symmetric part, at least that of the identity.
   The factors kept (layout in DevSpec ch_off / core_off): per chain node k
   Q_k = U_k Theta_(k+1)^-1, Theta_k^-1 and P_k = Theta_k^-1 L_k; per chain
   R = Theta_0^-1 E and F; the core's S^-1.  A solve is two sweeps along every
   chain around one core matrix-vector product:
       g_last = b_last,   g_k = b_k - Q_k g_(k+1),   h_k = Theta_k^-1 g_k,
       x_core = S^-1 (b_core - sum F h_0),
       x_0 = h_0 - R x_core,   x_k = h_k - P_k x_(k-1).
   Work and storage are O(n) per block (against O(n kl (kl + ku)) for a banded
   LU whose band must span the core), so the factors of every hierarchy class
   fit in shared memory.  Each sweep is a linear recurrence, i.e. a composition
   of affine maps, so a warp evaluates it as a scan (chain_back, chain_fwd). */

template <typename T> __device__ inline T tabs(T x) { return x < T(0) ? -x : x; }

/* position of J(i, j), i and j in block b with structure codes pi and pj (mx_pos),
   in the structured storage; -1 for an entry outside the structure */
template <class C> __device__ inline int mx_slot(const C &c, int b, int pi, int pj) {
  const DevSpec &s = c.s;
  int ci = (pi >> 8) - 1, cj = (pj >> 8) - 1, cn = s.core_n[b];
  if (ci < 0 && cj < 0) return s.core_off[b] + pi * cn + pj;
  if (ci < 0) {
    /* a core row on a chain column: the chain's first node only */
    int d = s.ch_d[b][cj], kj = pj & 127, aj = (pj >> 7) & 1;
    if (kj != 0) return -1;
    return s.ch_off[b][cj] + 3 * d * d * s.ch_len[b][cj] + d * cn + pi * d + aj;
  }
  int d = s.ch_d[b][ci], ki = pi & 127, ai = (pi >> 7) & 1;
  if (cj < 0) {
    /* a chain row on a core column: the chain's first node only */
    if (ki != 0) return -1;
    return s.ch_off[b][ci] + 3 * d * d * s.ch_len[b][ci] + ai * cn + pj;
  }
  int kj = pj & 127, aj = (pj >> 7) & 1;
  if (ci != cj || kj < ki - 1 || kj > ki + 1) return -1;
  int part = kj == ki ? 0 : (kj < ki ? 1 : 2);
  return s.ch_off[b][ci] + (3 * ki + part) * d * d + ai * d + aj;
}

/* Exact Jacobian of the affine system at tau (prepare(tau) must have run):
   J[:, j] = A e_j, one thread per column, scattered into the structured storage
   in the iteration-matrix precision.  Every row of the column's block is
   evaluated, so an entry outside the structure is detected (status
   SONG2_E_CONFIG) instead of being dropped.  Ends with a barrier. */
template <typename T, class C> __device__ __forceinline__ int jacobian(const C &c, int ap, double tau) {
  const DevSpec &s = c.s;
  auto J = c.template jacv<T>();
  for (int e = c.rank; e < s.lu_elems; e += c.size) J[e] = T(0);
  if (c.rank == 0) c.sh->mx_bad = 0;
  c.sync();
  for (int j = c.rank; j < s.n; j += c.size) {
    int b = 0;
    while (b + 1 < s.nblk && j >= s.blk_start[b + 1]) ++b;
    int b0 = s.blk_start[b], nb = s.blk_size[b];
    int pj = __ldg(c.ct.mx_pos + j);
    YUnit yu{j};
    WS w;
    compute_ws(c, ap, yu, 1, w);
    for (int i = b0; i < b0 + nb; ++i) {
      double v = row(c, ap, i, yu, w, 1, tau);
      if (v != 0.0) {
        int slot = mx_slot(c, b, __ldg(c.ct.mx_pos + i), pj);
        if (slot < 0) c.sh->mx_bad = 1;
        else J[slot] = (T)v;
      }
    }
  }
  c.sync();
  return c.sh->mx_bad ? SONG2_E_CONFIG : SONG2_OK;
}

/* d x d blocks, row major, d = 1 or 2 */
template <typename T, int D> __device__ inline void mx_mul(const T *a, const T *b, T *r) {
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      T acc = T(0);
#pragma unroll
      for (int k = 0; k < D; ++k) acc += a[i * D + k] * b[k * D + j];
      r[i * D + j] = acc;
    }
}
template <typename T, int D> __device__ inline bool mx_inv(const T *a, T *r) {
  if constexpr (D == 1) {
    r[0] = T(1) / a[0];
    return tabs(a[0]) > T(0);
  } else {
    T det = a[0] * a[3] - a[1] * a[2];
    T id = T(1) / det;
    r[0] = a[3] * id; r[1] = -a[1] * id; r[2] = -a[2] * id; r[3] = a[0] * id;
    return tabs(det) > T(0);
  }
}

/* one chain of block b, by one lane: Q_k, Theta_k^-1, P_k from the last node up,
   then R = Theta_0^-1 E and the scaled F.  False on a zero pivot. */
template <typename T, int D, class C, class VJ, class VF>
__device__ __forceinline__ bool chain_factor(const C &c, int b, int ch, T hg, const VJ &J, const VF &F) {
  const DevSpec &s = c.s;
  constexpr int D2 = D * D;
  int len = s.ch_len[b][ch], cn = s.core_n[b], base = s.ch_off[b][ch];
  T tn[D2], lnext[D2];
  bool ok = true;
  for (int k = len - 1; k >= 0; --k) {
    int o = base + 3 * D2 * k;
    T th[D2], ml[D2];
#pragma unroll
    for (int e = 0; e < D2; ++e) {
      th[e] = (e % (D + 1) == 0 ? T(1) : T(0)) - hg * J[o + e];
      ml[e] = -hg * J[o + D2 + e];
    }
    if (k < len - 1) {
      T mu[D2], q[D2], ql[D2];
#pragma unroll
      for (int e = 0; e < D2; ++e) mu[e] = -hg * J[o + 2 * D2 + e];
      mx_mul<T, D>(mu, tn, q);
      mx_mul<T, D>(q, lnext, ql);
#pragma unroll
      for (int e = 0; e < D2; ++e) {
        th[e] -= ql[e];
        F[o + e] = q[e];
      }
    } else {
#pragma unroll
      for (int e = 0; e < D2; ++e) F[o + e] = T(0);
    }
    T ti[D2], pk[D2];
    ok &= mx_inv<T, D>(th, ti);
    mx_mul<T, D>(ti, ml, pk);
#pragma unroll
    for (int e = 0; e < D2; ++e) {
      F[o + D2 + e] = ti[e];
      F[o + 2 * D2 + e] = pk[e];
      tn[e] = ti[e];
      lnext[e] = ml[e];
    }
  }
  int oe = base + 3 * D2 * len;
  for (int j = 0; j < cn; ++j)
#pragma unroll
    for (int a = 0; a < D; ++a) {
      T acc = T(0);
#pragma unroll
      for (int q = 0; q < D; ++q) acc += tn[a * D + q] * (-hg * J[oe + q * cn + j]);
      F[oe + a * cn + j] = acc;
    }
  for (int e = 0; e < cn * D; ++e) F[oe + D * cn + e] = -hg * J[oe + D * cn + e];
  return ok;
}

/* the core of block b, by a group of W lanes (after its chains): the Schur
   complement and its inverse, in place, by Gauss-Jordan elimination with partial
   pivoting (lane j updates columns j, j + W, ...).  False on a zero pivot. */
template <typename T, class C, class VJ, class VF>
__device__ __forceinline__ bool core_factor(const C &c, int b, T hg, const VJ &J, const VF &F, int lane, int W, unsigned mask,
                                            int nch) {
  const DevSpec &s = c.s;
  int cn = s.core_n[b], co = s.core_off[b];
  if (cn == 0) return true;
  for (int e = lane; e < cn * cn; e += W) {
    int i = e / cn, j = e % cn;
    T v = (i == j ? T(1) : T(0)) - hg * J[co + e];
    for (int ch = 0; ch < nch; ++ch) {
      int d = s.ch_d[b][ch], oe = s.ch_off[b][ch] + 3 * d * d * s.ch_len[b][ch];
      for (int a = 0; a < d; ++a) v -= F[oe + d * cn + i * d + a] * F[oe + a * cn + j];
    }
    F[co + e] = v;
  }
  __syncwarp(mask);
  bool ok = true;
  int perm[S2_MAXCORE];
  for (int p = 0; p < cn; ++p) {
    int r = p;
    T best = tabs((T)F[co + p * cn + p]);
    for (int i = p + 1; i < cn; ++i) {
      T v = tabs((T)F[co + i * cn + p]);
      if (v > best) { best = v; r = i; }
    }
    perm[p] = r;
    __syncwarp(mask);
    if (r != p)
      for (int j = lane; j < cn; j += W) {
        T t = F[co + p * cn + j];
        F[co + p * cn + j] = F[co + r * cn + j];
        F[co + r * cn + j] = t;
      }
    __syncwarp(mask);
    T colp[S2_MAXCORE];
    for (int i = 0; i < cn; ++i) colp[i] = F[co + i * cn + p];
    __syncwarp(mask);
    T piv = colp[p];
    if (!(tabs(piv) > T(0))) { ok = false; piv = T(1); }
    T pinv = T(1) / piv;
    for (int j = lane; j < cn; j += W) {
      T apj = (j == p ? T(1) : (T)F[co + p * cn + j]) * pinv;
      F[co + p * cn + j] = apj;
      for (int i = 0; i < cn; ++i)
        if (i != p) F[co + i * cn + j] = (j == p ? T(0) : (T)F[co + i * cn + j]) - apj * colp[i];
    }
    __syncwarp(mask);
  }
  /* undo the row interchanges on the inverse's columns, one row per lane */
  for (int i = lane; i < cn; i += W)
    for (int p = cn - 1; p >= 0; --p)
      if (perm[p] != p) {
        T t = F[co + i * cn + p];
        F[co + i * cn + p] = F[co + i * cn + perm[p]];
        F[co + i * cn + perm[p]] = t;
      }
  __syncwarp(mask);
  return ok;
}

/* run f(b, lane, W, mask) for every block: a warp per block (CTA teams), the team
   itself otherwise */
template <class C, class F> __device__ void per_block_group(const C &c, F f) {
  const DevSpec &s = c.s;
  if constexpr (C::STR) {
    for (int b = 0; b < s.nblk; ++b) f(b, c.rank, c.size, c.tmask);
  } else if (c.size == 32) {
    for (int b = 0; b < s.nblk; ++b) f(b, c.rank, 32, 0xffffffffu);
  } else {
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int b = warp; b < s.nblk; b += nw) f(b, lane, 32, 0xffffffffu);
  }
}

/* f1(b, ch) for every chain of node dimension 1 and f2(b, ch) for every chain of
   dimension 2: in a CTA team the scalar chains run on the lanes of warp 0 and the
   E/B chains on the lanes of warp 1, so that every warp follows one code path and
   the two kinds run side by side; smaller teams take the chains in turn. */
template <class C, class F1, class F2> __device__ void for_chains(const C &c, F1 f1, F2 f2) {
  const DevSpec &s = c.s;
  if constexpr (!C::STR) {
    if (c.size >= 64) {
      int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
      if (warp == 0 && lane < s.n_ch1) f1(s.ch1[lane] >> 4, s.ch1[lane] & 15);
      if (warp == 1 && lane < s.n_ch2) f2(s.ch2[lane] >> 4, s.ch2[lane] & 15);
      return;
    }
  }
  for (int t = c.rank; t < s.n_ch1 + s.n_ch2; t += c.size) {
    if (t < s.n_ch1) f1(s.ch1[t] >> 4, s.ch1[t] & 15);
    else f2(s.ch2[t - s.n_ch1] >> 4, s.ch2[t - s.n_ch1] & 15);
  }
}

/* M = I - hinvGak J factorised from the stored Jacobian: every chain on its own
   lane, then the core of every block.  Ends with a barrier; sets sh->lu_fail on a
   zero pivot.  One out-of-line call per factorisation: inlined into the NDF loop
   the chain and core eliminations raise its register spills, and as separate
   calls each would save and restore the caller's registers. */
template <typename T, class C> __device__ __noinline__ void form_and_factor(const C &c, double hinvGak) {
  const DevSpec &s = c.s;
  auto J = c.template jacv<T>();
  auto F = c.template lu<T>();
  T hg = (T)hinvGak;
  /* radiation streaming: the chains' rows are zero, so their blocks of M are the
     identity and their coupling to the cores vanishes; only the cores are factorised */
  const bool chains = c.sh->ap != AP_RSA;
  if (chains)
    for_chains(
        c, [&](int b, int ch) { if (!chain_factor<T, 1>(c, b, ch, hg, J, F)) c.sh->lu_fail = 1; },
        [&](int b, int ch) { if (!chain_factor<T, 2>(c, b, ch, hg, J, F)) c.sh->lu_fail = 1; });
  c.sync();
  PH_MARK(c, PH_FACT_CHAIN);
  per_block_group(c, [&](int b, int lane, int W, unsigned mask) {
    if (!core_factor<T>(c, b, hg, J, F, lane, W, mask, chains ? s.ch_n[b] : 0)) c.sh->lu_fail = 1;
  });
  c.sync();
}

/* An affine map z -> A z + B of d-vectors (d = 1 or 2): the sweeps of a chain are
   compositions of such maps, evaluated as a scan across the lanes of a group. */
template <typename T, int D> struct Aff {
  T A[D * D], B[D];
};
template <typename T, int D> __device__ inline Aff<T, D> aff_id() {
  Aff<T, D> m;
#pragma unroll
  for (int e = 0; e < D * D; ++e) m.A[e] = (e % (D + 1) == 0) ? T(1) : T(0);
#pragma unroll
  for (int a = 0; a < D; ++a) m.B[a] = T(0);
  return m;
}
/* f o g: z -> fA (gA z + gB) + fB */
template <typename T, int D> __device__ inline Aff<T, D> aff_after(const Aff<T, D> &f, const Aff<T, D> &g) {
  Aff<T, D> r;
#pragma unroll
  for (int i = 0; i < D; ++i) {
    T b = f.B[i];
#pragma unroll
    for (int k = 0; k < D; ++k) b += f.A[i * D + k] * g.B[k];
    r.B[i] = b;
#pragma unroll
    for (int j = 0; j < D; ++j) {
      T a = T(0);
#pragma unroll
      for (int k = 0; k < D; ++k) a += f.A[i * D + k] * g.A[k * D + j];
      r.A[i * D + j] = a;
    }
  }
  return r;
}
template <typename T, int D> __device__ inline Aff<T, D> aff_shfl(const Aff<T, D> &m, int delta, bool down, int W,
                                                                   unsigned mask) {
  Aff<T, D> r;
#pragma unroll
  for (int e = 0; e < D * D; ++e) r.A[e] = down ? __shfl_down_sync(mask, m.A[e], delta, W) : __shfl_up_sync(mask, m.A[e], delta, W);
#pragma unroll
  for (int a = 0; a < D; ++a) r.B[a] = down ? __shfl_down_sync(mask, m.B[a], delta, W) : __shfl_up_sync(mask, m.B[a], delta, W);
  return r;
}

/* Backward sweep of one chain by a group of W lanes (W a power of two): g_last =
   b_last, g_k = b_k - Q_k g_(k+1), and h_k = Theta_k^-1 g_k into the node entries of
   x.  g_k is the composition f_k o f_(k+1) o ... o f_last of the maps
   f_k(z) = b_k - Q_k z (Q_last = 0), so each lane composes its own run of
   P = ceil(len / W) nodes, a suffix scan across the lanes (log2 W shuffle steps)
   gives every lane the value entering its run, and the lane replays its nodes. */
template <typename T, int D, class C, class VF, class X>
__device__ void chain_back(const C &c, int b, int ch, const VF &F, const X &x, int lane, int W, unsigned mask) {
  const DevSpec &s = c.s;
  constexpr int D2 = D * D;
  int len = s.ch_len[b][ch], base = s.ch_off[b][ch];
  const short *ix = c.mx_s + s.ch_idx[b][ch];
  int P = (len + W - 1) / W, k0 = lane * P, k1 = min(len, k0 + P);
  Aff<T, D> m = aff_id<T, D>();
  for (int k = k1 - 1; k >= k0; --k) {
    Aff<T, D> f;
#pragma unroll
    for (int e = 0; e < D2; ++e) f.A[e] = -(T)F[base + 3 * D2 * k + e];
#pragma unroll
    for (int a = 0; a < D; ++a) f.B[a] = x[ix[k * D + a]];
    m = aff_after(f, m);
  }
  for (int off = 1; off < W; off <<= 1) {
    Aff<T, D> o = aff_shfl(m, off, true, W, mask);
    if (lane + off < W) m = aff_after(m, o);
  }
  T z[D];
#pragma unroll
  for (int a = 0; a < D; ++a) {
    z[a] = __shfl_down_sync(mask, m.B[a], 1, W);
    if (k1 >= len) z[a] = T(0);
  }
  for (int k = k1 - 1; k >= k0; --k) {
    int o = base + 3 * D2 * k;
    T g[D];
#pragma unroll
    for (int a = 0; a < D; ++a) {
      T v = x[ix[k * D + a]];
#pragma unroll
      for (int r = 0; r < D; ++r) v -= F[o + a * D + r] * z[r];
      g[a] = v;
    }
#pragma unroll
    for (int a = 0; a < D; ++a) {
      T h = T(0);
#pragma unroll
      for (int r = 0; r < D; ++r) h += F[o + D2 + a * D + r] * g[r];
      x[ix[k * D + a]] = h;
      z[a] = g[a];
    }
  }
}

/* Forward sweep of one chain by a group of W lanes: x_0 = h_0 - R x_core,
   x_k = h_k - P_k x_(k-1), a prefix scan of the maps z -> h_k - P_k z (node 0's map
   is the constant x_0), as in chain_back. */
template <typename T, int D, class C, class VF, class X>
__device__ void chain_fwd(const C &c, int b, int ch, const VF &F, const X &x, int lane, int W, unsigned mask) {
  const DevSpec &s = c.s;
  constexpr int D2 = D * D;
  int len = s.ch_len[b][ch], base = s.ch_off[b][ch], cn = s.core_n[b];
  const short *ix = c.mx_s + s.ch_idx[b][ch], *cx = c.mx_s + s.core_idx[b];
  int oe = base + 3 * D2 * len;
  int P = (len + W - 1) / W, k0 = lane * P, k1 = min(len, k0 + P);
  T x0[D];
  if (k0 == 0 && k1 > 0)
#pragma unroll
    for (int a = 0; a < D; ++a) {
      T v = x[ix[a]];
      for (int j = 0; j < cn; ++j) v -= F[oe + a * cn + j] * (T)x[cx[j]];
      x0[a] = v;
    }
  Aff<T, D> m = aff_id<T, D>();
  for (int k = k0; k < k1; ++k) {
    Aff<T, D> f;
    if (k == 0) {
#pragma unroll
      for (int e = 0; e < D2; ++e) f.A[e] = T(0);
#pragma unroll
      for (int a = 0; a < D; ++a) f.B[a] = x0[a];
    } else {
#pragma unroll
      for (int e = 0; e < D2; ++e) f.A[e] = -(T)F[base + 3 * D2 * k + 2 * D2 + e];
#pragma unroll
      for (int a = 0; a < D; ++a) f.B[a] = x[ix[k * D + a]];
    }
    m = aff_after(f, m);
  }
  for (int off = 1; off < W; off <<= 1) {
    Aff<T, D> o = aff_shfl(m, off, false, W, mask);
    if (lane >= off) m = aff_after(m, o);
  }
  T z[D];
#pragma unroll
  for (int a = 0; a < D; ++a) z[a] = __shfl_up_sync(mask, m.B[a], 1, W);
  for (int k = k0; k < k1; ++k) {
    T v[D];
    if (k == 0) {
#pragma unroll
      for (int a = 0; a < D; ++a) v[a] = x0[a];
    } else {
      int o = base + 3 * D2 * k + 2 * D2;
#pragma unroll
      for (int a = 0; a < D; ++a) {
        v[a] = x[ix[k * D + a]];
#pragma unroll
        for (int r = 0; r < D; ++r) v[a] -= F[o + a * D + r] * z[r];
      }
    }
#pragma unroll
    for (int a = 0; a < D; ++a) {
      x[ix[k * D + a]] = v[a];
      z[a] = v[a];
    }
  }
}

/* f(b, ch, lane, W, mask) for every chain, each chain by a whole group of lanes:
   in a CTA team the warps take the chains in turn, otherwise the team takes them
   one after the other */
template <class C, class F> __device__ void per_chain_group(const C &c, F f) {
  const DevSpec &s = c.s;
  int nc = s.n_ch1 + s.n_ch2;
  auto pick = [&](int t) { return t < s.n_ch1 ? s.ch1[t] : s.ch2[t - s.n_ch1]; };
  if constexpr (C::STR) {
    for (int t = 0; t < nc; ++t) f(pick(t) >> 4, pick(t) & 15, c.rank, c.size, c.tmask);
  } else if (c.size == 32) {
    for (int t = 0; t < nc; ++t) f(pick(t) >> 4, pick(t) & 15, c.rank, 32, 0xffffffffu);
  } else {
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int t = warp; t < nc; t += nw) f(pick(t) >> 4, pick(t) & 15, lane, 32, 0xffffffffu);
  }
}

/* the core of block b in M x = xsol: x_core = S^-1 (b_core - sum F h_0), by a group
   of W lanes, after the chains' backward sweeps */
template <typename T, class C> __device__ void core_solve(const C &c, int b, int lane, int W, unsigned mask, bool chains) {
  const DevSpec &s = c.s;
  auto F = c.template lu<T>();
  auto x = c.template xsol<T>();
  int nch = chains ? s.ch_n[b] : 0, cn = s.core_n[b];
  if (cn == 0) return;
  const short *cx = c.mx_s + s.core_idx[b];
  for (int i = lane; i < cn; i += W) {
    T r = x[cx[i]];
    for (int ch = 0; ch < nch; ++ch) {
      int d = s.ch_d[b][ch], oe = s.ch_off[b][ch] + 3 * d * d * s.ch_len[b][ch];
      const short *ix = c.mx_s + s.ch_idx[b][ch];
      for (int a = 0; a < d; ++a) r -= F[oe + d * cn + i * d + a] * (T)x[ix[a]];
    }
    x[cx[i]] = r;
  }
  __syncwarp(mask);
  T out[S2_MAXCORE];
  int cnt = 0;
  int co = s.core_off[b];
  for (int i = lane; i < cn; i += W) {
    T acc = T(0);
    for (int j = 0; j < cn; ++j) acc += F[co + i * cn + j] * (T)x[cx[j]];
    out[cnt++] = acc;
  }
  __syncwarp(mask);
  cnt = 0;
  for (int i = lane; i < cn; i += W) x[cx[i]] = out[cnt++];
}

/* xsol <- M^{-1} xsol (the right-hand side already in the solve vector): the
   backward sweeps of every chain, the cores, the forward sweeps, separated by
   barriers.  Ends with a barrier. */
template <typename T, class C> __device__ void lu_solve(const C &c) {
  const DevSpec &s = c.s;
  auto F = c.template lu<T>();
  auto x = c.template xsol<T>();
  /* radiation streaming: the chains' right-hand sides are zero and their blocks
     the identity, so their solution is zero and only the cores are solved */
  const bool chains = c.sh->ap != AP_RSA;
  if (chains) {
    per_chain_group(c, [&](int b, int ch, int lane, int W, unsigned mask) {
      if (s.ch_d[b][ch] == 1) chain_back<T, 1>(c, b, ch, F, x, lane, W, mask);
      else chain_back<T, 2>(c, b, ch, F, x, lane, W, mask);
    });
    c.sync();
  }
  PH_MARK(c, PH_SOLVE_BACK);
  per_block_group(c, [&](int b, int lane, int W, unsigned mask) { core_solve<T>(c, b, lane, W, mask, chains); });
  c.sync();
  PH_MARK(c, PH_SOLVE_CORE);
  if (chains) {
    per_chain_group(c, [&](int b, int ch, int lane, int W, unsigned mask) {
      if (s.ch_d[b][ch] == 1) chain_fwd<T, 1>(c, b, ch, F, x, lane, W, mask);
      else chain_fwd<T, 2>(c, b, ch, F, x, lane, W, mask);
    });
    c.sync();
  }
}

/* ------------------------------------------------------------------ reductions */

/* Max of non-negative doubles over the team.  The reduction runs on the bit
   patterns: for x >= 0 the IEEE-754 order equals the unsigned-integer order, and
   a NaN compares above +inf, so no FP64 instruction is spent on it. */
__device__ inline unsigned long long dbits(double v) { return (unsigned long long)__double_as_longlong(v); }

template <class C> __device__ double block_max_bits(const C &c, unsigned long long v) {
  if constexpr (C::STR) {
    for (int off = c.size >> 1; off > 0; off >>= 1) {
      unsigned long long o = __shfl_xor_sync(c.tmask, v, off);
      v = o > v ? o : v;
    }
  } else {
    for (int off = 16; off > 0; off >>= 1) {
      unsigned long long o = __shfl_xor_sync(0xffffffffu, v, off);
      v = o > v ? o : v;
    }
    if (c.size > 32) {
      int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
      __syncthreads();
      if (lane == 0) ((unsigned long long *)c.sh->red)[warp] = v;
      __syncthreads();
      int nw = (blockDim.x + 31) >> 5;
      v = 0;
      for (int i = 0; i < nw; ++i) {
        unsigned long long o = ((unsigned long long *)c.sh->red)[i];
        v = o > v ? o : v;
      }
    }
  }
  /* any NaN maps to +inf, so callers test a single "< inf" */
  if (v > 0x7ff0000000000000ull) v = 0x7ff0000000000000ull;
  return __longlong_as_double((long long)v);
}

/* N maxima of non-negative doubles over the team at once, through the same two
   barriers (the bit-pattern reduction of block_max_bits) */
template <int N, class C> __device__ void block_max_bits_n(const C &c, unsigned long long (&v)[N], double (&out)[N]) {
  if constexpr (C::STR) {
    for (int off = c.size >> 1; off > 0; off >>= 1)
#pragma unroll
      for (int q = 0; q < N; ++q) {
        unsigned long long o = __shfl_xor_sync(c.tmask, v[q], off);
        v[q] = o > v[q] ? o : v[q];
      }
  } else {
    for (int off = 16; off > 0; off >>= 1)
#pragma unroll
      for (int q = 0; q < N; ++q) {
        unsigned long long o = __shfl_xor_sync(0xffffffffu, v[q], off);
        v[q] = o > v[q] ? o : v[q];
      }
    if (c.size > 32) {
      static_assert(N * 8 <= 32, "reduction slots");
      int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
      unsigned long long *red = (unsigned long long *)c.sh->red;
      __syncthreads();
      if (lane == 0)
#pragma unroll
        for (int q = 0; q < N; ++q) red[q * 8 + warp] = v[q];
      __syncthreads();
      int nw = (blockDim.x + 31) >> 5;
#pragma unroll
      for (int q = 0; q < N; ++q) {
        v[q] = 0;
        for (int i = 0; i < nw; ++i) {
          unsigned long long o = red[q * 8 + i];
          v[q] = o > v[q] ? o : v[q];
        }
      }
    }
  }
#pragma unroll
  for (int q = 0; q < N; ++q) {
    if (v[q] > 0x7ff0000000000000ull) v[q] = 0x7ff0000000000000ull;
    out[q] = __longlong_as_double((long long)v[q]);
  }
}

/* running max of |x| in the bit domain (the sign bit is cleared, NaN stays above inf) */
__device__ inline void bmax(unsigned long long &acc, double x) {
  unsigned long long b = dbits(x) & 0x7fffffffffffffffull;
  acc = b > acc ? b : acc;
}


/* ------------------------------------------------------------------ outputs */

/* First-order collision terms over kappa' of the photon intensity (stored in the
   first-order table) and of the E polarisation (its linear collision term,
   -E_l - sqrt6/10 Pi delta_l2, Pi = I_2 - sqrt6 E_2), unrotated. */
template <class V> __device__ double fo_coll_I(const V &fo, const DevSpec &s, int l) { return fo[s.fo_CG + l]; }
template <class V> __device__ double fo_coll_E(const V &fo, const DevSpec &s, int l) {
  if (l < 2) return 0.0;
  double v = -fo[s.fo_E + l];
  if (l == 2) v -= SQRT_6 * 0.1 * (fo[SONG2_FO_I + 2] - SQRT_6 * fo[s.fo_E + 2]);
  return v;
}

/* delta-tilde part of the (l,m) source of field 0 (T), 1 (E) or 2 (B):
   -2 kappa' (delta*delta/2 + delta*collision), perturbations2.c:12339-12398 (T),
   12509-12561 (E), 12658-12710 (B). */
template <class C> __device__ __noinline__ double delta_tilde_source(const C &c, int field, int l, int m, double kappa_dot) {
  const DevSpec &s = c.s;
  auto fo1 = c.fo1, fo2 = c.fo2;
  int Q = field == 0 ? s.dt_qt : s.dt_qp;
  double dd = 0.0, dc = 0.0;
  for (int l1 = 0; l1 <= Q; ++l1)
    for (int l2 = abs(l1 - l); l2 <= min(l1 + l, Q); ++l2) {
      if (((l1 + l2 + l) & 1) != (field == 2 ? 1 : 0)) continue;
      for (int m1 = -l1; m1 <= l1; ++m1) {
        int m2 = m - m1;
        if (abs(m2) > l2) continue;
        double cpl = __ldg(c.p.dt_coup + dt_index(s, field, l, m, l1, m1, l2));
        double r11 = c.rot_1(l1, m1), r21 = c.rot_2(l1, m1), r12 = c.rot_1(l2, m2), r22 = c.rot_2(l2, m2);
        double I_1 = r11 * c.I1r(l1), I_2 = r21 * c.I2r(l1);
        if (field == 0) {
          double c_1 = r12 * fo_coll_I(fo1, s, l2), c_2 = r22 * fo_coll_I(fo2, s, l2);
          dd += cpl * 2 * I_1 * (r22 * c.I2r(l2));
          dc += cpl * 2 * 0.5 * (I_1 * c_2 + I_2 * c_1);
        } else {
          double E_1 = r12 * c.E1r(l2), E_2 = r22 * c.E2r(l2);
          double cI_1 = r11 * fo_coll_I(fo1, s, l1), cI_2 = r21 * fo_coll_I(fo2, s, l1);
          double cE_1 = r12 * fo_coll_E(fo1, s, l2), cE_2 = r22 * fo_coll_E(fo2, s, l2);
          dd += cpl * 2 * 0.5 * (I_1 * E_2 + I_2 * E_1);
          dc += cpl * 0.5 * (I_1 * cE_2 + cI_1 * E_2 + I_2 * cE_1 + cI_2 * E_1);
        }
      }
    }
  return -2 * kappa_dot * 0.5 * dd - 2 * kappa_dot * dc;
}

template <class C, class A, class B>
__device__ void store_sources(const C &c, int index_tau, double tau, A y, B dy) {
  const DevSpec &s = c.s;
  const Tri &t = c.sh->tri;
  auto yv = yvec(y);
  /* psi' from the phi' row: psi' = (phi_pp - dy[phi']) / Hc */
  if (c.rank == 0) {
    double psi_prime = 0.0;
    if (s.compute_m[0]) {
      int ap = c.sh->ap;
      double dI20 = ap == AP_TCA ? 0.0 : dy[ap == AP_RSA ? c.s.idx_c000 : c.idx_I[c.LM(2, 0)]];
      double dN20 = dy[ap == AP_RSA ? c.s.idx_c000 : c.idx_N[c.LM(2, 0)]];
      psi_prime = psi_prime_of(c, ap, yv, c.sh->ws, 0, dI20, dN20);
    }
    c.sh->psi_prime = psi_prime;
  }
  c.sync();
  const WS &w = c.sh->ws;
  const BgV &bg = c.sh->bg;
  auto fo1 = c.fo1, fo2 = c.fo2;
  double k1 = t.k1, k2 = t.k2, k = t.k;
  double psi_1 = fo1[SONG2_FO_PSI], psi_2 = fo2[SONG2_FO_PSI], phi_1 = fo1[SONG2_FO_PHI], phi_2 = fo2[SONG2_FO_PHI];
  double phi_prime_1 = fo1[SONG2_FO_PHI_P], phi_prime_2 = fo2[SONG2_FO_PHI_P];
  double psi_prime_1 = fo1[SONG2_FO_PSI_P], psi_prime_2 = fo2[SONG2_FO_PSI_P];
  double psi = w.psi, phi_prime = w.phi_prime, psi_prime = c.sh->psi_prime;
  if (s.compute_m[0] && s.los_exp_pot) {
    psi = psi - 2 * psi_1 * psi_2;
    phi_prime = phi_prime + 2 * (phi_1 * phi_prime_2 + phi_prime_1 * phi_2);
    psi_prime = psi_prime - 2 * (psi_1 * psi_prime_2 + psi_prime_1 * psi_2);
  }
  double omp = w.omega_m1_prime, gp = s.compute_m[2] ? y[s.idx_gammap] : 0.0;
  double kd = bg.kappa_dot;
  int64_t col = t.pair_off + (int64_t)index_tau * t.k3_size + t.i3;
  for (int tp = c.rank; tp < s.tp2_size; tp += c.size) {
    int kind = s.tp_kind[tp], l = s.tp_l[tp], m = s.tp_m[tp];
    double src = 0.0;
    if (!s.compute_m[m]) {
      /* a mode this triplet's hierarchy class does not evolve */
      c.p.sources[(int64_t)tp * s.per_type + col] = 0.0;
      continue;
    }
    if (kind == TP_T) {
      if (l == 0) {
        src += kd * w.I_00;
        if (s.los_pure_metric) src += 4 * phi_prime;
        else {
          src += (s.los_sw ? 1 : 0) * (4 * kd * psi);
          src += (s.los_isw ? 1 : 0) * (4 * (phi_prime + psi_prime));
        }
        if (s.los_quad_metric && !s.los_exp_pot) src += 8 * (phi_1 * phi_prime_2 + phi_2 * phi_prime_1);
      } else if (l == 1) {
        if (s.los_pure_scat) src += FOUR_THIRDS * kd * getb(c, yv, 1, m);
        if (s.los_pure_metric) {
          if (m == 0) src += 4 * k * psi;
          if (m == 1) src += -4 * omp;
        } else if (m == 1)
          src += (s.los_isw ? 1 : 0) * (-4 * omp);
        if (s.los_quad_metric) {
          if (!s.los_exp_pot) src += -4 * (t.k1_m[m + 1] * psi_1 * (psi_2 - phi_2) + t.k2_m[m + 1] * psi_2 * (psi_1 - phi_1));
          else src += -4 * (t.k1_m[m + 1] * psi_1 * (-psi_2 - phi_2) + t.k2_m[m + 1] * psi_2 * (-psi_1 - phi_1));
        }
      } else if (l == 2) {
        if (s.los_pure_scat) src += kd * 0.1 * (w.I_2m[m] - SQRT_6 * w.E_2m[m]);
        if (s.los_pure_metric && m == 2) src += 4 * gp;
      }
      if (s.los_quad_scat) src += c.qc[s.iq_g + c.LM(l, m)];
      if (s.los_time_delay)
        src -= c.I2r(l + 1) * c.S(CP22, l, m) * k2 * (phi_1 + psi_1) - c.I2r(l - 1) * c.S(CM22, l, m) * k2 * (phi_1 + psi_1) +
               c.I1r(l + 1) * c.S(CP11, l, m) * k1 * (phi_2 + psi_2) - c.I1r(l - 1) * c.S(CM11, l, m) * k1 * (phi_2 + psi_2);
      if (s.los_redshift)
        src -= -4 * phi_prime_1 * c.rot_2(l, m) * c.I2r(l) + c.I2r(l + 1) * 4 * c.S(CP12, l, m) * k1 * psi_1 -
               c.I2r(l - 1) * 4 * c.S(CM12, l, m) * k1 * psi_1 - 4 * phi_prime_2 * c.rot_1(l, m) * c.I1r(l) +
               c.I1r(l + 1) * 4 * c.S(CP21, l, m) * k2 * psi_2 - c.I1r(l - 1) * 4 * c.S(CM21, l, m) * k2 * psi_2;
      if (s.los_lensing)
        src -= c.I2r(l + 1) * (-(l + 2) * c.S(CP12, l, m)) * k1 * (phi_1 + psi_1) -
               c.I2r(l - 1) * ((l - 1) * c.S(CM12, l, m)) * k1 * (phi_1 + psi_1) +
               c.I1r(l + 1) * (-(l + 2) * c.S(CP21, l, m)) * k2 * (phi_2 + psi_2) -
               c.I1r(l - 1) * ((l - 1) * c.S(CM21, l, m)) * k2 * (phi_2 + psi_2);
      if (s.dtilde) src += delta_tilde_source(c, 0, l, m, kd);
    } else if (kind == TP_E) {
      if (l >= 2) {
        if (l == 2 && s.los_pure_scat) src += -SQRT_6 * kd * 0.1 * (w.I_2m[m] - SQRT_6 * w.E_2m[m]);
        if (s.los_quad_scat) src += c.qc[s.iq_E + c.LM(l, m)];
        if (s.los_time_delay)
          src -= c.E2r(l + 1) * c.S(DP22, l, m) * k2 * (phi_1 + psi_1) - c.E2r(l - 1) * c.S(DM22, l, m) * k2 * (phi_1 + psi_1) +
                 c.E1r(l + 1) * c.S(DP11, l, m) * k1 * (phi_2 + psi_2) - c.E1r(l - 1) * c.S(DM11, l, m) * k1 * (phi_2 + psi_2);
        if (s.los_redshift)
          src -= -4 * phi_prime_1 * c.rot_2(l, m) * c.E2r(l) + c.E2r(l + 1) * 4 * c.S(DP12, l, m) * k1 * psi_1 -
                 c.E2r(l - 1) * 4 * c.S(DM12, l, m) * k1 * psi_1 - 4 * phi_prime_2 * c.rot_1(l, m) * c.E1r(l) +
                 c.E1r(l + 1) * 4 * c.S(DP21, l, m) * k2 * psi_2 - c.E1r(l - 1) * 4 * c.S(DM21, l, m) * k2 * psi_2;
        if (s.los_lensing)
          src -= c.E2r(l + 1) * (-(l + 2) * c.S(DP12, l, m)) * k1 * (phi_1 + psi_1) -
                 c.E2r(l - 1) * ((l - 1) * c.S(DM12, l, m)) * k1 * (phi_1 + psi_1) +
                 c.E1r(l + 1) * (-(l + 2) * c.S(DP21, l, m)) * k2 * (phi_2 + psi_2) -
                 c.E1r(l - 1) * ((l - 1) * c.S(DM21, l, m)) * k2 * (phi_2 + psi_2);
        if (s.dtilde) src += delta_tilde_source(c, 1, l, m, kd);
      }
    } else if (kind == TP_B) {
      if (l >= 2 && m != 0) {
        if (s.los_quad_scat) src += c.qc[s.iq_B + c.LM(l, m)];
        if (s.los_time_delay)
          src -= -k2 * c.E2r(l) * c.S(DZ22, l, m) * (phi_1 + psi_1) - k1 * c.E1r(l) * c.S(DZ11, l, m) * (phi_2 + psi_2);
        if (s.los_redshift)
          src -= -c.E2r(l) * 4 * c.S(DZ12, l, m) * k1 * psi_1 - c.E1r(l) * 4 * c.S(DZ21, l, m) * k2 * psi_2;
        if (s.los_lensing)
          src -= -c.E2r(l) * (-c.S(DZ12, l, m)) * k1 * (phi_1 + psi_1) - c.E1r(l) * (-c.S(DZ21, l, m)) * k2 * (phi_2 + psi_2);
        if (s.dtilde) src += delta_tilde_source(c, 2, l, m, kd);
      }
    } else if (kind == TP_D) {
      if (s.compute_m[0]) {
        double v_dot_v_cdm = -t.k1_dot_k2 * fo1[SONG2_FO_V_CDM] * fo2[SONG2_FO_V_CDM];
        src = 0.5 * (getc(c, yv, 0, 0) - 2 * v_dot_v_cdm);
      }
      c.p.sources[(int64_t)tp * s.per_type + col] = src;
      continue;
    }
    c.p.sources[(int64_t)tp * s.per_type + col] = src * bg.exp_m_kappa;
  }
}

template <class C, class A, class B> __device__ void store_first_order(const C &c, int index_tau, A y, B dy) {
  const DevSpec &s = c.s;
  const Tri &t = c.sh->tri;
  int ap = c.sh->ap;
  auto yv = yvec(y);
  const WS &w = c.sh->ws;
  const BgV &bg = c.sh->bg;
  double k = t.k;
  double *o = c.p.fo_out + ((size_t)t.i1 * s.fo_tau_size + index_tau) * s.nfo;
  int L1 = s.fo_l_max + 1;
  for (int q = c.rank; q < s.nfo; q += c.size) {
    double v = 0.0;
    if (q < SONG2_FO_I) {
      switch (q) {
      case SONG2_FO_PHI: v = y[s.idx_phi]; break;
      case SONG2_FO_PSI: v = w.psi; break;
      case SONG2_FO_PHI_P: v = y[s.idx_phip]; break;
      case SONG2_FO_PSI_P: v = (w.phi_pp - dy[s.idx_phip]) / bg.Hc; break;
      case SONG2_FO_PHI_PP: v = dy[s.idx_phip]; break;
      case SONG2_FO_DELTA_G: v = w.I_00; break;
      case SONG2_FO_V_G: v = -w.I_1m[0] / (4 * k); break;
      case SONG2_FO_DELTA_B: v = y[s.idx_b000]; break;
      case SONG2_FO_V_B: v = -y[s.idx_b11[0]] / (3 * k); break;
      case SONG2_FO_DELTA_B_P: v = dy[s.idx_b000]; break;
      case SONG2_FO_V_B_P: v = -dy[s.idx_b11[0]] / (3 * k); break;
      case SONG2_FO_DELTA_CDM: v = y[s.idx_c000]; break;
      case SONG2_FO_V_CDM: v = -y[s.idx_c11[0]] / (3 * k); break;
      case SONG2_FO_V_CDM_P: v = -dy[s.idx_c11[0]] / (3 * k); break;
      case SONG2_FO_DELTA_UR: v = w.N_00; break;
      case SONG2_FO_V_UR: v = -w.N_1m[0] / (4 * k); break;
      case SONG2_FO_DIPOLE_B: v = y[s.idx_b11[0]]; break;
      case SONG2_FO_DIPOLE_CDM: v = y[s.idx_c11[0]]; break;
      }
    } else {
      int blk = (q - SONG2_FO_I) / L1, l = (q - SONG2_FO_I) % L1;
      if (blk == 0) v = (l == 0) ? w.I_00 : (l == 1) ? w.I_1m[0] : (l == 2) ? w.I_2m[0] : getI(c, ap, yv, l, 0);
      else if (blk == 1) v = (l < 2) ? 0.0 : (l == 2) ? w.E_2m[0] : getE(c, ap, yv, l, 0);
      else if (blk == 2) v = (l == 0) ? w.N_00 : (l == 1) ? w.N_1m[0] : getN(c, yv, l, 0);
      else
        v = (l == 0) ? 0.0 : (l == 1) ? w.C_1m[0] / bg.kappa_dot
          : (l == 2) ? -w.I_2m[0] + 0.1 * (w.I_2m[0] - SQRT_6 * w.E_2m[0]) : -getI(c, ap, yv, l, 0);
    }
    o[q] = v;
  }
}

/* ------------------------------------------------------------------ geometry */

/* sqrt((l-m)!/(l+m)!) P_l^m(x), Condon-Shortley phase, normalised recurrence;
   rescaled: divided by (1-x^2)^(m/2), by leaving that factor out of P_m^m (the
   form of plegendre_lm_rescaled, which stays finite as x -> 1) */
__device__ double legendre_norm(int l, int m, double x, int rescaled) {
  double sx = rescaled ? 1.0 : sqrt(fmax(0.0, 1.0 - x * x));
  double q = 1.0;
  for (int i = 1; i <= m; ++i) q *= -sqrt((2.0 * i - 1.0) / (2.0 * i)) * sx;
  if (l == m) return q;
  double q0 = q, q1 = x * sqrt(2.0 * m + 1.0) * q;
  for (int ll = m + 2; ll <= l; ++ll) {
    double q2 = ((2.0 * ll - 1.0) * x * q1 - sqrt((double)(ll - 1) * (ll - 1) - (double)m * m) * q0) /
                sqrt((double)ll * ll - (double)m * m);
    q0 = q1; q1 = q2;
  }
  return q1;
}

template <class C> __device__ int geometry(const C &c) {
  const DevSpec &s = c.s;
  Tri &t = c.sh->tri;
  int tid = c.rank, nt = c.size;
  if (tid == 0) {
    double k1 = t.k1, k2 = t.k2, k = t.k;
    t.k_sq = k * k;
    t.inv_k = 1.0 / k;
    t.inv_k_sq = t.inv_k * t.inv_k;
    t.lnk = log(k);
    t.cosk1k2 = (t.k_sq - k1 * k1 - k2 * k2) / (2 * k1 * k2);
    t.cosk1k = (k1 + k2 * t.cosk1k2) / k;
    t.cosk2k = (k2 + k1 * t.cosk1k2) / k;
    t.k1_dot_k2 = k1 * k2 * t.cosk1k2;
    /* perturbations2.c:5604-5652: with rescaling, rot(l,m) = rescaled P_lm (times
       (k1/k2)^m for k2) and rot(l,-m) = (-1)^m P_lm sin^m, i.e. (-1)^m rot(l,m) sin^2m */
    double s2 = fmax(0.0, 1.0 - t.cosk1k * t.cosk1k), f = 1.0;
    for (int m = 0; m < SONG2_MAX_M + 3; ++m) {
      t.mfac[m] = s.rescale ? f : 1.0;
      f *= s2;
    }
  }
  c.sync();
  if (fabs(t.cosk1k2) > 1 || fabs(t.cosk1k) > 1 || fabs(t.cosk2k) > 1) return 1;
  for (int e = tid; e < (s.Lq + 1) * (s.mq_max + 1); e += nt) {
    int l = e / (s.mq_max + 1), m = e % (s.mq_max + 1);
    if (m > l) continue;
    double r1 = legendre_norm(l, m, t.cosk1k, s.rescale), r2 = legendre_norm(l, m, t.cosk2k, s.rescale);
    if (m & 1) r2 = -r2;
    if (s.rescale)
      for (int i = 0; i < m; ++i) r2 *= t.k1 / t.k2;
    c.rot1[c.LMQ(l, m)] = r1;
    c.rot2[c.LMQ(l, m)] = r2;
  }
  c.sync();
  if (tid == 0) {
    double k1 = t.k1, k2 = t.k2;
    double k1_M1 = t.k1_m[0] = k1 * c.rot_1(1, -1), k1_0 = t.k1_m[1] = k1 * c.rot_1(1, 0), k1_P1 = t.k1_m[2] = k1 * c.rot_1(1, 1);
    double k2_M1 = t.k2_m[0] = k2 * c.rot_2(1, -1), k2_0 = t.k2_m[1] = k2 * c.rot_2(1, 0), k2_P1 = t.k2_m[2] = k2 * c.rot_2(1, 1);
    double kk = t.k1_dot_k2;
    t.k1_ten_k2[0] = SQRT_2 / SQRT_3 * k1_M1 * k2_M1;
    t.k1_ten_k2[1] = (k1_M1 * k2_0 + k2_M1 * k1_0) / SQRT_3;
    t.k1_ten_k2[2] = k1_0 * k2_0 - kk / 3.;
    t.k1_ten_k2[3] = (k1_P1 * k2_0 + k2_P1 * k1_0) / SQRT_3;
    t.k1_ten_k2[4] = SQRT_2 / SQRT_3 * k1_P1 * k2_P1;
    t.k1_ten_k1[0] = SQRT_2 / SQRT_3 * k1_M1 * k1_M1;
    t.k1_ten_k1[1] = (k1_M1 * k1_0 + k1_M1 * k1_0) / SQRT_3;
    t.k1_ten_k1[2] = k1_0 * k1_0 - k1 * k1 / 3.;
    t.k1_ten_k1[3] = (k1_P1 * k1_0 + k1_P1 * k1_0) / SQRT_3;
    t.k1_ten_k1[4] = SQRT_2 / SQRT_3 * k1_P1 * k1_P1;
    t.k2_ten_k2[0] = SQRT_2 / SQRT_3 * k2_M1 * k2_M1;
    t.k2_ten_k2[1] = (k2_M1 * k2_0 + k2_M1 * k2_0) / SQRT_3;
    t.k2_ten_k2[2] = k2_0 * k2_0 - k2 * k2 / 3.;
    t.k2_ten_k2[3] = (k2_P1 * k2_0 + k2_P1 * k2_0) / SQRT_3;
    t.k2_ten_k2[4] = SQRT_2 / SQRT_3 * k2_P1 * k2_P1;
  }
  /* summed couplings (perturbations2.c:5752-5845) for l <= L_big */
  for (int e = tid; e < (s.L_big + 1) * s.m_size; e += nt) {
    int l = e / s.m_size, im = e % s.m_size, m = s.m[im];
    if (m > l) continue;
    int lm = c.LM(l, m);
    double a[20];
    for (int X = 0; X < 20; ++X) a[X] = 0.0;
    for (int m2 = -1; m2 <= 1; ++m2) {
      int m1 = m - m2;
      double cm = __ldg(c.ct.cmin + lm * 3 + m - m1 + 1), cp = __ldg(c.ct.cplu + lm * 3 + m - m1 + 1);
      double dm = __ldg(c.ct.dmin + lm * 3 + m - m1 + 1), dp = __ldg(c.ct.dplu + lm * 3 + m - m1 + 1);
      double dz = __ldg(c.ct.dzer + lm * 3 + m - m1 + 1);
      double r11 = c.rot_1(1, m2), r21 = c.rot_2(1, m2);
      double r1m = c.rot_1(l - 1, m1), r2m = c.rot_2(l - 1, m1), r1p = c.rot_1(l + 1, m1), r2p = c.rot_2(l + 1, m1);
      double r10 = c.rot_1(l, m1), r20 = c.rot_2(l, m1);
      a[CM12] += r11 * r2m * cm; a[CM21] += r21 * r1m * cm; a[CP12] += r11 * r2p * cp; a[CP21] += r21 * r1p * cp;
      a[CM11] += r11 * r1m * cm; a[CM22] += r21 * r2m * cm; a[CP11] += r11 * r1p * cp; a[CP22] += r21 * r2p * cp;
      a[DM12] += r11 * r2m * dm; a[DM21] += r21 * r1m * dm; a[DP12] += r11 * r2p * dp; a[DP21] += r21 * r1p * dp;
      a[DM11] += r11 * r1m * dm; a[DM22] += r21 * r2m * dm; a[DP11] += r11 * r1p * dp; a[DP22] += r21 * r2p * dp;
      a[DZ12] += r11 * r20 * dz; a[DZ21] += r21 * r10 * dz; a[DZ11] += r11 * r10 * dz; a[DZ22] += r21 * r20 * dz;
    }
    for (int X = 0; X < 20; ++X) c.sc[X * s.n_lm + lm] = a[X];
  }
  c.sync();
  return 0;
}

/* start time (perturbations2.c:3388-3524) and TCA interval (perturbations2.c:4854-5403), thread 0 */
template <class C> __device__ int intervals(const C &c) {
  const DevSpec &s = c.s;
  Tri &t = c.sh->tri;
  double kmax = fmax(t.k, fmax(t.k1, t.k2));
  double tau_lower = exp(s.bg_lntau0), tau_upper = c.p.tau[0];
  if (s.mode_first_order) tau_upper = exp(s.fo_lntau0);
  double Hc, kd;
  bg_hk(c, tau_lower, Hc, kd);
  if (Hc / kd > s.start_h || kmax / Hc > s.start_k) return 1;
  double tau_mid = 0.5 * (tau_lower + tau_upper);
  for (int it = 0; it < 200 && (tau_upper - tau_lower) / tau_lower > s.tol_tau; ++it) {
    bg_hk(c, tau_mid, Hc, kd);
    if (Hc / kd > s.start_h || kmax / Hc > s.start_k) tau_upper = tau_mid;
    else tau_lower = tau_mid;
    tau_mid = 0.5 * (tau_lower + tau_upper);
  }
  t.tau_ini = tau_mid;
  t.tau_end = s.mode_first_order ? exp(s.fo_lntau0 + (s.fo_tau_size - 1) * s.fo_dlntau) : c.p.tau[s.tau_size - 1];
  if (s.mode_first_order) t.tau_end = exp(s.fo_lntau0 + (s.fo_tau_size - 1) * s.fo_dlntau);
  /* TCA trigger: tau_c/tau_h < trig_h and tau_c * max(k1,k2,k) < trig_k */
  auto tca_on = [&](double tau) {
    double h, kk;
    bg_hk(c, tau, h, kk);
    return s.tca_on && ((1.0 / kk) / (1.0 / h) < s.tca_h) && ((1.0 / kk) * kmax < s.tca_k);
  };
  /* RSA trigger (perturbations2.c:5309-5321): k tau above the trigger, after free streaming */
  auto rsa_on = [&](double tau) {
    return s.rsa && tau * t.k > s.rsa_k && tau > s.tau_fs;
  };
  int tca0 = tca_on(t.tau_ini);
  double t_tca = t.tau_ini;
  if (tca0) {
    if (tca_on(t.tau_end)) t_tca = t.tau_end;
    else {
      double lo = t.tau_ini, hi = t.tau_end;
      for (int it = 0; it < 200 && (hi - lo) / lo > s.tol_tau; ++it) {
        double mid = 0.5 * (lo + hi);
        if (tca_on(mid)) lo = mid; else hi = mid;
      }
      t_tca = 0.5 * (lo + hi);
    }
  }
  double t_rsa = t.tau_end;
  if (t_tca < t.tau_end && rsa_on(t.tau_end)) {
    if (rsa_on(t_tca)) t_rsa = t_tca;
    else {
      double lo = t_tca, hi = t.tau_end;
      for (int it = 0; it < 200 && (hi - lo) / lo > s.tol_tau; ++it) {
        double mid = 0.5 * (lo + hi);
        if (rsa_on(mid)) hi = mid; else lo = mid;
      }
      t_rsa = 0.5 * (lo + hi);
    }
  }
  int n = 0;
  t.ivb[0] = t.tau_ini;
  if (tca0) { t.ivk[n] = AP_TCA; t.ivb[++n] = t_tca; }
  if (t.ivb[n] < t_rsa) { t.ivk[n] = AP_NONE; t.ivb[++n] = t_rsa; }
  if (t_rsa < t.tau_end) { t.ivk[n] = AP_RSA; t.ivb[++n] = t.tau_end; }
  t.nint = n;
  return 0;
}

/* ------------------------------------------------------------------ initial conditions (thread 0) */

template <class C> __device__ void initial_conditions(const C &c, double tau) {
  const DevSpec &s = c.s;
  const Tri &t = c.sh->tri;
  const BgV &bg = c.sh->bg;
  auto y = c.y;
  for (int i = 0; i < s.n; ++i) y[i] = 0.0;
  if (s.ic == SONG2_IC_ZERO || !s.compute_m[0]) return;
  int ap = c.sh->ap;
  double k = t.k, k_sq = t.k_sq, Hc = bg.Hc, Hc_sq = Hc * Hc, a_sq = bg.a_sq;
  double rho_r = bg.rho_g + bg.rho_ur, frac_ur = bg.rho_ur / rho_r, frac_g = 1 - frac_ur;
  double rho_tot = Hc_sq / a_sq, Omega_m = (bg.rho_b + bg.rho_cdm) / rho_tot, Omega_r = rho_r / rho_tot;
  auto fo1 = c.fo1, fo2 = c.fo2, qs = c.qs;
  if (s.ic == SONG2_IC_AD) {
    double k1_0 = t.k1_m[1], k2_0 = t.k2_m[1];
    double delta_g_1 = fo1[SONG2_FO_DELTA_G], delta_g_2 = fo2[SONG2_FO_DELTA_G];
    double vpot_g_1 = fo1[SONG2_FO_V_G], vpot_g_2 = fo2[SONG2_FO_V_G];
    double delta_b_1 = fo1[SONG2_FO_DELTA_B], delta_b_2 = fo2[SONG2_FO_DELTA_B];
    double vpot_b_1 = fo1[SONG2_FO_V_B], vpot_b_2 = fo2[SONG2_FO_V_B];
    double delta_cdm_1 = fo1[SONG2_FO_DELTA_CDM], delta_cdm_2 = fo2[SONG2_FO_DELTA_CDM];
    double vpot_cdm_1 = fo1[SONG2_FO_V_CDM], vpot_cdm_2 = fo2[SONG2_FO_V_CDM];
    double delta_ur_1 = fo1[SONG2_FO_DELTA_UR], delta_ur_2 = fo2[SONG2_FO_DELTA_UR];
    double vpot_ur_1 = fo1[SONG2_FO_V_UR], vpot_ur_2 = fo2[SONG2_FO_V_UR];
    double phi_1 = fo1[SONG2_FO_PHI], phi_2 = fo2[SONG2_FO_PHI], psi_1 = fo1[SONG2_FO_PSI], psi_2 = fo2[SONG2_FO_PSI];
    double zeta = 2 * (3 / 5. * s.fnl);
    double A_quad = qs[s.iq_psi];
    double I_2_0_quad = 5 / 8. * (c.S(CM12, 2, 0) * c.I1r(1) * c.I2r(1) + c.S(CM21, 2, 0) * c.I2r(1) * c.I1r(1));
    double N_2_0_quad = 1 / 3. * (k / Hc_sq) * qs[s.iq_ur + c.LM(1, 0)] + 1 / (2 * Hc) * qs[s.iq_ur + c.LM(2, 0)] +
                        8 / 3. * (k_sq / Hc_sq) * psi_1 * psi_2;
    double quadrupole_quad = (frac_g * I_2_0_quad + frac_ur * N_2_0_quad) * 3 / 5. * (Hc_sq / k_sq);
    double B_quad = A_quad - quadrupole_quad;
    double frac_g_factor = 1 + 4 / 15. * (1 - frac_g);
    double psi = 1. / frac_g_factor * 2 / 3. * (-zeta + psi_1 * psi_2 - 2 * phi_1 * phi_2 + B_quad);
    double I_2_0 = I_2_0_quad;
    double N_2_0 = 2 / 3. * (k_sq / Hc_sq) * psi + N_2_0_quad;
    double phi = (1 + 2 / 5. * frac_ur) * psi - B_quad;
    double L_quad = qs[s.iq_phi_prime_longitudinal];
    double u0 = 2 * (k / Hc) * (psi - L_quad / Hc) - (-k1_0 * vpot_cdm_1) * (3 * Omega_m * delta_cdm_2 + 4 * Omega_r * delta_g_2) -
                (-k2_0 * vpot_cdm_2) * (3 * Omega_m * delta_cdm_1 + 4 * Omega_r * delta_g_1);
    u0 *= 1 / (3 * Omega_m + 4 * Omega_r);
    double I_1_0 = 4 * (u0 + delta_g_1 * (-k2_0 * vpot_g_2) + delta_g_2 * (-k1_0 * vpot_g_1));
    double N_1_0 = 4 * (u0 + delta_ur_1 * (-k2_0 * vpot_ur_2) + delta_ur_2 * (-k1_0 * vpot_ur_1));
    double b_1_1_0 = 3 * (u0 + delta_b_1 * (-k2_0 * vpot_b_2) + delta_b_2 * (-k1_0 * vpot_b_1));
    double cdm_1_1_0 = 3 * (u0 + delta_cdm_1 * (-k2_0 * vpot_cdm_2) + delta_cdm_2 * (-k1_0 * vpot_cdm_1));
    double I_0_0 = -2 * psi + 8 * psi_1 * psi_2;
    double b_0_0_0 = 3 * (I_0_0 / 4 - delta_g_1 * delta_g_2 / 16);
    y[s.idx_phi] = phi;
    y[c.idx_I[c.LM(0, 0)]] = I_0_0;
    if (!ap) {
      y[c.idx_I[c.LM(1, 0)]] = I_1_0;
      y[c.idx_I[c.LM(2, 0)]] = I_2_0;
    }
    y[s.idx_b000] = b_0_0_0;
    y[s.idx_b11[0]] = b_1_1_0;
    y[s.idx_c000] = b_0_0_0;
    y[s.idx_c11[0]] = cdm_1_1_0;
    y[c.idx_N[c.LM(0, 0)]] = I_0_0;
    y[c.idx_N[c.LM(1, 0)]] = N_1_0;
    y[c.idx_N[c.LM(2, 0)]] = N_2_0;
    double rho_monopole = bg.rho_g * I_0_0 + bg.rho_b * b_0_0_0 + bg.rho_cdm * b_0_0_0 + bg.rho_ur * I_0_0;
    y[s.idx_phip] = -Hc * psi - k_sq / (3 * Hc) * phi - a_sq * rho_monopole / (2 * Hc) + qs[s.iq_phi_prime_poisson];
  } else if (s.ic == SONG2_IC_AD_FIRST_ORDER) {
    double c_zeta = 0.5 * (2 * (-(3 / 5. * s.fnl)));
    double psi = 20 * c_zeta / (15 + 4 * frac_ur);
    y[s.idx_phi] = (1 + 2 / 5. * frac_ur) * psi;
    double u0 = 0.5 * k * tau * psi;
    double I_0_0 = -2 * psi;
    y[c.idx_I[c.LM(0, 0)]] = I_0_0;
    if (!ap) y[c.idx_I[c.LM(1, 0)]] = 4 * u0;
    y[s.idx_b000] = 0.75 * I_0_0;
    y[s.idx_b11[0]] = 3 * u0;
    y[s.idx_c000] = 0.75 * I_0_0;
    y[s.idx_c11[0]] = 3 * u0;
    y[c.idx_N[c.LM(0, 0)]] = I_0_0;
    y[c.idx_N[c.LM(1, 0)]] = 4 * u0;
    /* I_20 = 10 shear, consistent with the second-order initial conditions */
    y[c.idx_N[c.LM(2, 0)]] = 10 * (1 / 15. * k * k * tau * tau * psi);
    y[s.idx_phip] = 0.0;
  }
}

/* ------------------------------------------------------------------ NDF15 */

/* x^p for the step-size and order heuristics, in FP32: the choice needs a few
   significant digits, and an FP64 pow costs hundreds of cycles of the SM's FP64
   pipe on GB300.  x = 0 gives 0, x = inf gives inf, as pow does for p > 0. */
__device__ inline double pow_ctl(double x, double p) { return (double)exp2f((float)p * log2f((float)x)); }

__constant__ double c_G[5] = {1.0, 1.5, 11.0 / 6.0, 25.0 / 12.0, 137.0 / 60.0};
__constant__ double c_alpha[5] = {-0.1850, -1.0 / 9.0, -0.0823, -0.0415, 0.0};
/* U(i, j) = (-1)^(i+1) binom(j+1, i+1) (zero below the diagonal) */
__constant__ double c_U[5][5] = {{-1, -2, -3, -4, -5}, {0, 1, 3, 6, 10}, {0, 0, -1, -4, -10}, {0, 0, 0, 1, 5}, {0, 0, 0, 0, -1}};

/* dif[:,0..k-1] <- dif * (R(r) U): thread 0 forms R U, every thread updates its own components */
template <class C> __device__ void rescale_dif(const C &c, int k, double r) {
  double (*RU)[5] = c.sh->RU, (*Rm)[5] = c.sh->Rm;
  /* R(r) entry (i, j) = prod_{p=1..i+1} ((p-1) - (j+1) r) / p, one entry per thread */
  for (int e = c.rank; e < k * k; e += c.size) {
    int i = e / k, j = e % k;
    double prod = 1.0;
    for (int p = 1; p <= i + 1; ++p) prod *= ((p - 1) - (j + 1) * r) / p;
    Rm[i][j] = prod;
  }
  c.sync();
  /* RU = R U with U(i, j) = (-1)^(i+1) binom(j+1, i+1) for j >= i */
  for (int e = c.rank; e < k * k; e += c.size) {
    int i = e / k, j = e % k;
    double sm = 0;
    for (int p = 0; p <= j; ++p) sm += Rm[i][p] * c_U[p][j];
    RU[i][j] = sm;
  }
  c.sync();
  int n = c.s.n;
  for (int e = c.rank; e < n; e += c.size) {
    double tmp[5];
    for (int j = 0; j < k; ++j) {
      double sm = 0;
      for (int i = 0; i < k; ++i) sm += c.dif[i * n + e] * RU[i][j];
      tmp[j] = sm;
    }
    for (int j = 0; j < k; ++j) c.dif[j * n + e] = tmp[j];
  }
  c.sync();
}

template <typename T, class C>
__device__ int refactor(const C &c, double hinvGak, song2_triplet_stats &st) {
  if (c.rank == 0) c.sh->lu_fail = 0;
  c.sync();
  form_and_factor<T>(c, hinvGak);
  st.n_lu++;
  return c.sh->lu_fail ? SONG2_E_SINGULAR : SONG2_OK;
}

/* output of one sampling time: y interpolated in c.yout.  As in the reference,
   dy comes from derivs (tabulated quadratic sources, perturbations2.c:7702-7718)
   and the source functions from quadratic sources and workspace recomputed at
   tau (perturb2_sources, perturbations2.c:11956-12030). */
template <class C> __device__ void do_output(const C &c, int jout, double to) {
  int ap = c.sh->ap;
  prepare_table(c, to, ap);
  rhs(c, ap, to, c.yout, c.dyout);
  PH_MARK(c, PH_OUT_RHS);
  prepare(c, to, 1);
  compute_ws_team(c, ap, yvec(c.yout));
  c.sync();
  PH_MARK(c, PH_OUT_QS);
  if (c.s.mode_first_order) store_first_order(c, jout, c.yout, c.dyout);
  else store_sources(c, jout, to, c.yout, c.dyout);
  c.sync();
  PH_MARK(c, PH_OUT_STORE);
}

template <class C> __device__ inline double tout_at(const C &c, int j) {
  return c.s.mode_first_order ? exp(c.s.fo_lntau0 + j * c.s.fo_dlntau) : c.p.tau[j];
}

template <typename T, class C>
__device__ __forceinline__ int ndf15(const C &c, double t0, double t1, int &jout, int include_t0, song2_triplet_stats &st) {
  const DevSpec &s = c.s;
  int n = s.n, tid = c.rank, nt = c.size;
  int nout = s.mode_first_order ? s.fo_tau_size : s.tau_size;
  int ap = c.sh->ap;
  double rtol = s.rtol, threshold = s.threshold;
  const double eps = 2.220446049250313e-16;
  const int maxk = 5, maxit = 4;
  double invGa[5], erconst[5];
  for (int i = 0; i < 5; ++i) {
    invGa[i] = 1.0 / (c_G[i] * (1.0 - c_alpha[i]));
    erconst[i] = c_alpha[i] * c_G[i] + 1.0 / (i + 2);
  }
  auto y = c.y, f = c.f, ynew = c.ynew, difkp1 = c.difkp1, psiv = c.psiv, del = c.del, invwt = c.invwt;
  auto dif = c.dif;
  double t = t0, hmax = 0.1 * fabs(t1 - t0);
  if (include_t0)
    while (jout < nout && tout_at(c, jout) <= t0) {
      if (tout_at(c, jout) == t0) {
        for (int i = tid; i < n; i += nt) c.yout[i] = y[i];
        c.sync();
        do_output(c, jout, t0);
      }
      ++jout;
    }
  prepare_table(c, t, ap);
  rhs(c, ap, t, y, f);
  st.n_rhs++;
  if (jacobian<T>(c, ap, t)) return SONG2_E_CONFIG;
  st.n_jac++;
  int Jcurrent = 1;
  double hmin = 16 * eps * fabs(t);
  double absh = fmin(hmax, fabs(t1 - t0));
  unsigned long long vb = 0;
  for (int i = tid; i < n; i += nt) bmax(vb, f[i] / fmax(fabs(y[i]), threshold));
  double rh = 1.25 * block_max_bits(c, vb) / sqrt(rtol);
  if (absh * rh > 1) absh = 1.0 / rh;
  absh = fmax(absh, hmin);
  double h = absh;
  int k = 1;
  for (int e = tid; e < 7 * n; e += nt) dif[e] = 0.0;
  c.sync();
  for (int i = tid; i < n; i += nt) dif[i] = h * f[i];
  double hinvGak = h * invGa[k - 1];
  int nconhk = 0;
  if (refactor<T>(c, hinvGak, st)) return SONG2_E_SINGULAR;
  PH_MARK(c, PH_START);
  int havrate = 0;
  double rate = 0, abshlast = absh;
  int klast = k, done = 0, attempts = 0;
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
      rescale_dif(c, k, absh / abshlast);
      PH_MARK(c, PH_RESCALE);
      hinvGak = h * invGa[k - 1];
      nconhk = 0;
      if (refactor<T>(c, hinvGak, st)) return SONG2_E_SINGULAR;
      PH_MARK(c, PH_FACT);
      havrate = 0;
    }
    int nofailed = 1;
    double err = 0, tnew = t, errnrm = 0, ymax = 0;
    for (;;) {
      int gotynew = 0;
      while (!gotynew) {
        if (++attempts > s.max_steps) return SONG2_E_MAXSTEPS;
        /* predictor, its error weights and norm in one pass */
        unsigned long long vm = 0;
        for (int i = tid; i < n; i += nt) {
          double ps = 0, yi = y[i], pr = yi;
          for (int j = 0; j < k; ++j) {
            double dj = dif[(size_t)j * n + i];
            ps += dj * c_G[j];
            pr += dj;
          }
          psiv[i] = ps * invGa[k - 1];
          ynew[i] = pr;
          difkp1[i] = 0.0;
          /* error weight 1/max(|y|, |y_pred|, threshold): an FP32 reciprocal (the
             norms it scales need no more than single precision) */
          double iw = (double)__frcp_rn((float)fmax(fmax(fabs(yi), fabs(pr)), threshold));
          invwt[i] = iw;
          bmax(vm, pr * iw);
        }
        tnew = t + h;
        if (done) tnew = t1;
        h = tnew - t;
        double minnrm = 100 * eps * block_max_bits(c, vm);
        double oldnrm = 0;
        PH_MARK(c, PH_PRED);
        prepare_table(c, tnew, ap);
        PH_MARK(c, PH_PREP);
        for (int iter = 1; iter <= maxit; ++iter) {
          newton_rhs<T>(c, ap, tnew, ynew, hinvGak);
          st.n_rhs++;
          lu_solve<T>(c);
          PH_MARK(c, PH_SOLVE);
          /* the Newton norm, and with it the norms of the local error estimate and
             of the new state, should this iteration be the last */
          unsigned long long vv[3] = {0, 0, 0};
          auto xs = c.template xsol<T>();
          for (int i = tid; i < n; i += nt) {
            double d = (double)xs[i], w = invwt[i];
            double dk = difkp1[i] + d, yn = ynew[i] + d;
            bmax(vv[0], d * w);
            bmax(vv[1], dk * w);
            bmax(vv[2], yn);
            difkp1[i] = dk;
            ynew[i] = yn;
          }
          double nrm[3];
          block_max_bits_n<3>(c, vv, nrm);
          double newnrm = nrm[0];
          errnrm = nrm[1];
          ymax = nrm[2];
          PH_MARK(c, PH_NUPD);
          if (!(newnrm < INFINITY)) break;
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
        PH_MARK(c, PH_NUPD);
        if (!gotynew) {
          st.n_newton_fail++;
          if (absh <= hmin) return SONG2_E_NEWTON;
          if (Jcurrent) {
            double abshold = absh;
            absh = fmax(0.3 * absh, hmin);
            h = absh;
            done = 0;
            rescale_dif(c, k, absh / abshold);
            abshlast = absh;
            hinvGak = h * invGa[k - 1];
            nconhk = 0;
          } else {
            prepare(c, t, 0);
            if (jacobian<T>(c, ap, t)) return SONG2_E_CONFIG;
            st.n_jac++;
            Jcurrent = 1;
          }
          PH_MARK(c, PH_JAC);
          if (refactor<T>(c, hinvGak, st)) return SONG2_E_SINGULAR;
          PH_MARK(c, PH_FACT);
          havrate = 0;
        }
      }
      err = errnrm * erconst[k - 1];
      if (!(ymax < 1e300)) return SONG2_E_NAN;
      if (err > rtol) {
        st.n_rejected++;
        if (absh <= hmin) return SONG2_E_HMIN;
        double abshl = absh;
        if (nofailed) {
          nofailed = 0;
          double errkm1 = 0;
          if (k > 1) {
            unsigned long long vk = 0;
            for (int i = tid; i < n; i += nt) bmax(vk, (dif[(size_t)(k - 1) * n + i] + difkp1[i]) * invwt[i]);
            errkm1 = block_max_bits(c, vk) * erconst[k - 2];
          }
          /* the FP64 powers are evaluated side by side and shared */
          for (int q = tid; q < 2; q += nt) {
            if (q == 0) c.sh->ctl[0] = absh * fmax(0.1, 0.833 * pow_ctl(rtol / err, 1.0 / (k + 1)));
            else if (k > 1) c.sh->ctl[1] = absh * fmax(0.1, 0.769 * pow_ctl(rtol / errkm1, 1.0 / k));
          }
          c.sync();
          double hopt = c.sh->ctl[0];
          if (k > 1) {
            double hkm1 = c.sh->ctl[1];
            if (hkm1 > hopt) {
              hopt = fmin(absh, hkm1);
              k = k - 1;
            }
          }
          c.sync();
          absh = fmax(hmin, hopt);
        } else {
          absh = fmax(hmin, 0.5 * absh);
        }
        h = absh;
        if (absh < abshl) done = 0;
        PH_MARK(c, PH_ERR);
        rescale_dif(c, k, absh / abshl);
        PH_MARK(c, PH_RESCALE);
        abshlast = absh;
        klast = k;
        hinvGak = h * invGa[k - 1];
        nconhk = 0;
        if (refactor<T>(c, hinvGak, st)) return SONG2_E_SINGULAR;
        PH_MARK(c, PH_FACT);
        havrate = 0;
      } else
        break;
    }
    PH_MARK(c, PH_ERR);
    /* accepted step */
    st.n_steps++;
    for (int i = tid; i < n; i += nt) {
      double dk = dif[(size_t)k * n + i];
      dif[(size_t)(k + 1) * n + i] = difkp1[i] - dk;
      dif[(size_t)k * n + i] = difkp1[i];
      for (int j = k - 1; j >= 0; --j) dif[(size_t)j * n + i] += dif[(size_t)(j + 1) * n + i];
    }
    c.sync();
    PH_MARK(c, PH_ACCEPT);
    while (jout < nout && tout_at(c, jout) <= tnew) {
      double to = tout_at(c, jout);
      if (to > t || (include_t0 && to == t)) {
        double sv = (to - tnew) / h;
        for (int i = tid; i < n; i += nt) {
          double acc = ynew[i], term = 1.0;
          if (to != tnew)
            for (int j = 0; j < k; ++j) {
              term *= (sv + j) / (j + 1);
              acc += dif[(size_t)j * n + i] * term;
            }
          c.yout[i] = acc;
        }
        c.sync();
        do_output(c, jout, to);
        st.sources_calls++;
      }
      ++jout;
    }
    klast = k;
    abshlast = absh;
    nconhk = (nconhk + 1 < maxk + 2) ? nconhk + 1 : maxk + 2;
    if (nconhk >= k + 2) {
      unsigned long long vk = 0, vp = 0;
      for (int i = tid; i < n; i += nt) {
        if (k > 1) bmax(vk, dif[(size_t)(k - 1) * n + i] * invwt[i]);
        if (k < maxk) bmax(vp, dif[(size_t)(k + 1) * n + i] * invwt[i]);
      }
      unsigned long long vkp[2] = {vk, vp};
      double ekp[2];
      block_max_bits_n<2>(c, vkp, ekp);
      double errkm1 = ekp[0], errkp1 = ekp[1];
      /* the three candidate step sizes, side by side */
      for (int q = tid; q < 3; q += nt) {
        double temp, hq = 0.0;
        if (q == 0) {
          temp = 1.2 * pow_ctl(err / rtol, 1.0 / (k + 1));
          hq = (temp > 0.1) ? absh / temp : 10 * absh;
        } else if (q == 1 && k > 1) {
          temp = 1.3 * pow_ctl(errkm1 * erconst[k - 2] / rtol, 1.0 / k);
          hq = (temp > 0.1) ? absh / temp : 10 * absh;
        } else if (q == 2 && k < maxk) {
          temp = 1.4 * pow_ctl(errkp1 * erconst[k] / rtol, 1.0 / (k + 2));
          hq = (temp > 0.1) ? absh / temp : 10 * absh;
        }
        c.sh->ctl[q] = hq;
      }
      c.sync();
      double hopt = c.sh->ctl[0];
      int kopt = k;
      if (k > 1 && c.sh->ctl[1] > hopt) { hopt = c.sh->ctl[1]; kopt = k - 1; }
      if (k < maxk && c.sh->ctl[2] > hopt) { hopt = c.sh->ctl[2]; kopt = k + 1; }
      c.sync();
      if (hopt > absh) {
        absh = hopt;
        if (k != kopt) k = kopt;
      }
    }
    t = tnew;
    /* the new state becomes the current one: the two buffers trade places */
    {
      auto tmp = y;
      y = ynew;
      ynew = tmp;
    }
    c.sync();
    PH_MARK(c, PH_CTRL);
    Jcurrent = 0;
  }
  /* the next interval and the caller find the state in c.y */
  if (y.p != c.y.p) {
    for (int i = tid; i < n; i += nt) c.y[i] = y[i];
    c.sync();
  }
  return SONG2_OK;
}

/* ------------------------------------------------------------------ one triplet */

template <typename T, class C> __device__ __forceinline__ int solve_triplet(const C &c, song2_triplet_stats &st) {
  const DevSpec &s = c.s;
  int tid = c.rank;
  if (geometry(c)) return SONG2_E_CONFIG;
  if (tid == 0) c.sh->lu_fail = intervals(c);
  c.sync();
  if (c.sh->lu_fail) return SONG2_E_CONFIG;
  Tri &t = c.sh->tri;
  PH_MARK(c, PH_SETUP);
  build_qs_table(c);
  PH_MARK(c, PH_QTAB);
  int jout = 0;
  for (int iv = 0; iv < t.nint; ++iv) {
    double ta = t.ivb[iv], tb = t.ivb[iv + 1];
    if (iv == 0) {
      if (tid == 0) c.sh->ap = t.ivk[0];
      c.sync();
      prepare(c, ta, 1);
      if (tid == 0) initial_conditions(c, ta);
      c.sync();
    } else if (t.ivk[iv] == AP_RSA) {
      /* switching the RSA on drops the massless hierarchies: nothing to remap
         (perturbations2.c:7295-7300); their entries stay in y, unevolved */
      if (tid == 0) c.sh->ap = AP_RSA;
      c.sync();
    } else {
      /* TCA -> full remap (perturbations2.c:7233-7285): the frozen moments take the
         TCA values at the switching time, evaluated as derivs does; everything
         else carries over */
      prepare_table(c, ta, 1);
      if (tid == 0) {
        auto yv = yvec(c.y);
        compute_ws(c, 1, yv, 0, c.sh->ws);
        WS &w = c.sh->ws;
        for (int im = 0; im <= s.index_m_max[1]; ++im) c.y[c.idx_I[c.LM(1, s.m[im])]] = w.I_1m_tca1[s.m[im]];
        for (int im = 0; im <= s.index_m_max[2]; ++im) {
          int m = s.m[im];
          c.y[c.idx_I[c.LM(2, m)]] = w.I_2m_tca1[m];
          if (s.has_pol) {
            c.y[c.idx_E[c.LM(2, m)]] = w.E_2m_tca1[m];
            if (m != 0) c.y[c.idx_B[c.LM(2, m)]] = w.B_2m_tca1[m];
          }
        }
        c.sh->ap = 0;
      }
      c.sync();
    }
    PH_MARK(c, PH_IC);
    int stc = ndf15<T>(c, ta, tb, jout, iv == 0, st);
    if (stc != SONG2_OK) return stc;
  }
  int nout = s.mode_first_order ? s.fo_tau_size : s.tau_size;
  if (st.sources_calls != nout) return SONG2_E_CONFIG;
  return SONG2_OK;
}

/* set up the team's triplet from its work item (rank 0) */
template <class C> __device__ void begin_item(const C &c, int item) {
  const DevPtrs &p = c.p;
  WorkItem wi = p.items[item];
  if (c.rank == 0) {
    Tri &t = c.sh->tri;
    t.i1 = wi.i1; t.i2 = wi.i2; t.i3 = wi.i3; t.pair = wi.pair; t.item = item;
    t.k1 = p.k[wi.i1];
    t.k2 = p.k[wi.i2];
    t.k3_size = p.k3_size[wi.pair];
    t.k = p.k3[p.k3_off[wi.pair] + wi.i3];
    t.pair_off = p.pair_off[wi.pair];
  }
  c.sync();
}

template <typename T, class C> __device__ __forceinline__ void run_item(const C &c, int item) {
  PH_RESET(c);
  begin_item(c, item);
  song2_triplet_stats st;
  st.status = 0; st.n_steps = 0; st.n_rejected = 0; st.n_rhs = 0; st.n_jac = 0; st.n_lu = 0; st.n_newton_fail = 0;
  st.sources_calls = 0;
  st.retried = 0;
  int stc = solve_triplet<T>(c, st);
  st.status = stc;
  if (c.rank == 0) c.p.stats[c.p.stats_by_ref ? c.p.items[item].ref : item] = st;
  PH_ITEM_END(c);
  c.sync();
}

/* CTA or warp per triplet: persistent, one item at a time from the queue.  With
   hierarchy classes (uneven batches, CTA teams only) the item's class spec is
   copied into shared memory and the team's context is rebuilt for it.  MINB is the
   number of CTAs per SM the register allocation must allow (2 for the launch group
   of small hierarchy classes, whose shared-memory plans fit two CTAs per SM). */
template <typename T, int MODE, int CLASSES, int MINB = 1>
__global__ void __launch_bounds__(256, MINB) evolver_kernel(const __grid_constant__ DevSpec s, const __grid_constant__ DevPtrs p) {
  extern __shared__ __align__(16) char smem[];
  __shared__ int s_item[8];
  const int prec = sizeof(T) == sizeof(float) ? SONG2_PREC_MIXED : SONG2_PREC_FP64;
  if constexpr (!CLASSES) {
    KX<MODE> c(s, p, p.tabs, smem, prec);
    int slot = MODE == MODE_WARP ? (threadIdx.x >> 5) : 0;
    c.load_tables();
    c.sync();
    for (int guard = 0; guard < s.n_items + 1; ++guard) {
      if (c.rank == 0) s_item[slot] = atomicAdd(p.queue, 1);
      c.sync();
      int item = s_item[slot];
      c.sync();
      if (item >= s.n_items) break;
      run_item<T>(c, item);
    }
  } else {
    DevSpec *cs = (DevSpec *)smem;
    char *rest = smem + al(sizeof(DevSpec));
    for (int guard = 0; guard < s.n_items + 1; ++guard) {
      if (threadIdx.x == 0) s_item[0] = atomicAdd(p.queue, 1);
      __syncthreads();
      int item = s_item[0];
      __syncthreads();
      if (item >= s.n_items) break;
      int cls = p.items[item].cls;
      static_assert(sizeof(DevSpec) % sizeof(long long) == 0, "DevSpec copy granularity");
      const long long *src = (const long long *)(p.class_spec + cls);
      long long *dst = (long long *)cs;
      for (int e = threadIdx.x; e < (int)(sizeof(DevSpec) / sizeof(long long)); e += blockDim.x) dst[e] = src[e];
      __syncthreads();
      KX<MODE> c(*cs, p, p.class_tabs[cls], rest, prec);
      c.load_tables();
      c.sync();
      run_item<T>(c, item);
    }
  }
}

/* G lanes per triplet: each warp takes the next 32/G items of the cost-sorted
   queue at once, so that its teams advance through similar triplets side by side. */
template <typename T>
__global__ void __launch_bounds__(128) team_kernel(const __grid_constant__ DevSpec s, const __grid_constant__ DevPtrs p) {
  extern __shared__ __align__(16) char smem[];
  KX<MODE_TEAM> c(s, p, p.tabs, smem, sizeof(T) == sizeof(float) ? SONG2_PREC_MIXED : SONG2_PREC_FP64);
  c.load_tables();
  __syncthreads();
  int lane = threadIdx.x & 31, tiw = lane / s.team_lanes;
  for (int guard = 0; guard < s.n_items + 1; ++guard) {
    int base = 0;
    if (lane == 0) base = atomicAdd(p.queue, c.nt);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= s.n_items) break;
    int item = base + tiw;
    if (item < s.n_items) run_item<T>(c, item);
    __syncwarp();
  }
}

} // namespace

#endif
