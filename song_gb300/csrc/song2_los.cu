// song2_los.cu - line-of-sight integration of the second-order sources on the
// device: the projection-function tables of SONG's bessel2 module and the
// transfer functions of its transfer2 module.
//
// Tables (bessel2_init, bessel2.c:75-497), built once per handle:
//   j_l1(x)      one thread per x node: Miller's downward recurrence over every l
//                of the extended l1 list, stored from the l1's x_min on
//                (bessel2_j_for_l1, :1669-1800);
//   J_Llm(x)     one block row per (J, L, l, m): the 3j-weighted sum of j_l1
//                (bessel2_J_Llm, :1460-1600), then one thread per row finds the
//                first non-negligible x by the reference's bisection
//                (bessel2_J_for_Llm, :1041-1458); spline second derivatives per
//                row for cubic interpolation (:423-477).
// Transfers (transfer2_init loop, transfer2.c:283-556), persistent CTAs over
// the (pair, k) units in pair-major order so that concurrent CTAs read nearby x
// of the same J rows:
//   the pair's sources interpolated to k in k3 (:2612-2780) into shared memory;
//   the integration grid in time (:2366-2610), built interval by interval with
//   a block scan, and the time interpolation weights (:2783-2926);
//   one warp per transfer type (T/E/B, l, m), its lanes over the time grid:
//   sum_L J(x) S with x = k (tau0 - tau), the trapezoid measure, the factors of
//   transfer2_compute (:1861-2138).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "song2.h"
#include "song2_los.h"
#include "song2_los_view.h"

#define CKL(x)                                                                                     \
  do {                                                                                             \
    cudaError_t e_ = (x);                                                                          \
    if (e_ != cudaSuccess) {                                                                       \
      snprintf(err, SONG2_ERRLEN, "%s failed: %s (%s:%d)", #x, cudaGetErrorString(e_), __FILE__, \
               __LINE__);                                                                          \
      return 1;                                                                                    \
    }                                                                                              \
  } while (0)

namespace {

constexpr int NJ = 3;             // J_TT, J_EE, J_EB
constexpr int MAXC = 24;          // l1 terms of one J row (2 L_max + 1)
constexpr int MAXTERM = 32;       // (J, L) contributions of one transfer type
constexpr int LOS_THREADS = 256;
constexpr int LOS_WARPS = LOS_THREADS / 32;
constexpr int GRID_SMEM_MAX = 2048;  // integration grids up to this size live in shared memory

// one (J row, source type, sign) contribution of a transfer type
struct Term {
  int row;      // J row
  int tp;       // source type (index into the shared source rows)
  int xmin;     // first non-negligible x index of the row
  int mix;      // 0: direct, 1: mixing (accumulated apart, as the reference)
};

struct LosDev {
  // x grid
  int x_size;
  double x_max, x_step;
  // tables
  const double *J, *ddJ;
  const int *Jxmin;
  // spec
  int tau_size, k_size;
  const double *tau;          // source time sampling
  const double *k3;           // sources' k3 grids, pair after pair
  const int *k3_off, *k3_n;   // per pair
  const long long *src_off;   // per pair: offset within one source type
  long long per_type;
  const double *ddk;          // spline second derivatives in k3 (cubic), layout of the sources
  // units
  long long n_units;
  const int *unit_pair;
  const double *unit_k;
  const int *unit_left;
  const double *unit_b;
  // source rows used: tp index in the flat sources of each shared row
  int n_rows_src;
  const int *src_tp;
  // transfer types
  int n_tt;
  const int *tt_l;
  const double *tt_msign;     // sign of the mixing contribution (-1 for E->B)
  const int *tt_nterm;
  const int *tt_ndir;         // direct terms (they come first)
  const int *tt_xmin;         // smallest x_min of the type's terms
  const Term *terms;          // [n_tt][MAXTERM]
  // sampling options
  int tau_sampling, time_cubic, k3_cubic, bessel_cubic;
  double tau_linstep, tau0;
  int grid_cap;               // capacity of one CTA's integration grid
  int grid_in_smem;
  double *grid_scratch;       // per CTA when not in shared memory
  int *queue;
  int *status;
};

// ------------------------------------------------------------- tables

// j_l1(x) for every l1 of the list (ascending), one thread per x node
__global__ void __launch_bounds__(128) jl_kernel(int x_size, double x_max, int n_l1, const int *__restrict__ l1,
                                                 const int *__restrict__ jxmin, double *__restrict__ jtab) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= x_size) return;
  double x = s2los_x_of(i, x_size, x_max);
  int lmax = l1[n_l1 - 1];
  if (x == 0.0) {
    for (int r = 0; r < n_l1; ++r) jtab[(size_t)r * x_size + i] = (l1[r] == 0 && i >= jxmin[r]) ? 1.0 : 0.0;
    return;
  }
  int top = s2los_miller_start(x, lmax);
  double inv = 1.0 / x;
  double fp = 0.0, f = 1.0;
  int scale = 0;
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
  fp = 0.0;
  f = 1.0;
  scale = 0;
  int r = n_l1 - 1;
  for (int l = top; l >= 0 && r >= 0; --l) {
    if (l == l1[r]) {
      double v = ldexp(f * m_norm, e_norm - S2LOS_SCALE_BITS * (final_scale - scale));
      jtab[(size_t)r * x_size + i] = (i >= jxmin[r]) ? v : 0.0;
      --r;
    }
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

// J rows: J[row][x] = scale_row * sum_t coef[row][t] j_l1(row,t)(x)
__global__ void __launch_bounds__(256) J_kernel(int x_size, int n_rows, const int *__restrict__ nterm,
                                                const double *__restrict__ coef, const int *__restrict__ jrow,
                                                const double *__restrict__ rscale, const double *__restrict__ jtab,
                                                double *__restrict__ J) {
  int row = blockIdx.y;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= n_rows || i >= x_size) return;
  int n = nterm[row];
  double s = 0.0;
  for (int t = 0; t < n; ++t) s += coef[(size_t)row * MAXC + t] * jtab[(size_t)jrow[(size_t)row * MAXC + t] * x_size + i];
  J[(size_t)row * x_size + i] = s * rscale[row];
}

// first non-negligible x of every row (bessel2_J_for_Llm's bisection on |J| >= J_cut)
// mode: 0 negligible everywhere, 1 from x = 0 (L == l), 2 bisection from index `up`
__global__ void Jxmin_kernel(int x_size, int n_rows, const int *__restrict__ mode, const int *__restrict__ up0,
                             const double *__restrict__ up_x, double x_max, double J_cut,
                             const double *__restrict__ J, int *__restrict__ xmin, int *__restrict__ status) {
  int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= n_rows) return;
  const double *Jr = J + (size_t)row * x_size;
  int md = mode[row];
  if (md == 0) {
    xmin[row] = x_size - 1;
    return;
  }
  if (md == 1) {
    xmin[row] = 0;
    return;
  }
  int down = 0, up = up0[row];
  if (fabs(Jr[up]) < J_cut) {
    xmin[row] = x_size - 1;
    if (up_x[row] < x_max) atomicExch(status, 1);  // the reference stops: wrong initial guess
    return;
  }
  for (int it = 0; it < 64 && down != up - 1; ++it) {
    int mid = (up + down) / 2;
    if (fabs(Jr[mid]) >= J_cut) up = mid;
    else down = mid;
  }
  xmin[row] = down;
}

// Cubic-spline second derivatives of one row (natural, or the estimated end
// derivatives for l = 2), over the x nodes from the row's x_min on; u is the
// recurrence's scratch row.
__device__ void spline_row(const double *__restrict__ y, int n, int est, double x_size_m1, double x_max, int x0,
                           double *__restrict__ y2, double *__restrict__ u) {
  auto X = [&](int i) { return 0.0 + (double)(x0 + i) * (x_max - 0.0) / x_size_m1; };
  if (n < 3) {
    for (int i = 0; i < n; ++i) y2[i] = 0.0;
    return;
  }
  if (est) {
    double x0_ = X(0), x1 = X(1), x2 = X(2);
    double dy = ((x2 - x0_) * (x2 - x0_) * (y[1] - y[0]) - (x1 - x0_) * (x1 - x0_) * (y[2] - y[0])) /
                ((x2 - x0_) * (x1 - x0_) * (x2 - x1));
    y2[0] = -0.5;
    u[0] = (3. / (x1 - x0_)) * ((y[1] - y[0]) / (x1 - x0_) - dy);
  } else {
    y2[0] = 0.0;
    u[0] = 0.0;
  }
  for (int i = 1; i < n - 1; ++i) {
    double xm = X(i - 1), xi = X(i), xp = X(i + 1);
    double sig = (xi - xm) / (xp - xm);
    double p = sig * y2[i - 1] + 2.0;
    y2[i] = (sig - 1.0) / p;
    u[i] = (y[i + 1] - y[i]) / (xp - xi) - (y[i] - y[i - 1]) / (xi - xm);
    u[i] = (6.0 * u[i] / (xp - xm) - sig * u[i - 1]) / p;
  }
  double qn, un;
  if (est) {
    double a = X(n - 3), b = X(n - 2), c = X(n - 1);
    double dy = ((a - c) * (a - c) * (y[n - 2] - y[n - 1]) - (b - c) * (b - c) * (y[n - 3] - y[n - 1])) /
                ((a - c) * (b - c) * (a - b));
    qn = 0.5;
    un = (3. / (c - b)) * (dy - (y[n - 1] - y[n - 2]) / (c - b));
  } else {
    qn = un = 0.0;
  }
  y2[n - 1] = (un - qn * u[n - 2]) / (qn * y2[n - 2] + 1.0);
  for (int k = n - 2; k >= 0; --k) y2[k] = y2[k] * y2[k + 1] + u[k];
}

__global__ void ddJ_kernel(int x_size, double x_max, int n_rows, const int *__restrict__ xmin,
                           const int *__restrict__ est, const double *__restrict__ J, double *__restrict__ ddJ,
                           double *__restrict__ scratch) {
  int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= n_rows) return;
  int x0 = xmin[row];
  int n = x_size - x0;
  spline_row(J + (size_t)row * x_size + x0, n, est[row], (double)(x_size - 1), x_max, x0,
             ddJ + (size_t)row * x_size + x0, scratch + (size_t)row * x_size);
}

// Spline second derivatives of the sources in k3 with estimated end derivatives
// (transfer2_interpolate_sources_in_k, cubic: array_spline_table_columns over
// the pair's k3 grid for every time), one thread per (source row, pair, tau).
__device__ void spline_gen(const double *__restrict__ x, const double *__restrict__ y, int stride, int n,
                           double *__restrict__ y2, double *__restrict__ u) {
  // y[i * stride], y2[i * stride]; the estimated end derivatives of a quadratic
  double dy = ((x[2] - x[0]) * (x[2] - x[0]) * (y[stride] - y[0]) - (x[1] - x[0]) * (x[1] - x[0]) * (y[2 * stride] - y[0])) /
              ((x[2] - x[0]) * (x[1] - x[0]) * (x[2] - x[1]));
  y2[0] = -0.5;
  u[0] = (3. / (x[1] - x[0])) * ((y[stride] - y[0]) / (x[1] - x[0]) - dy);
  for (int i = 1; i < n - 1; ++i) {
    double sig = (x[i] - x[i - 1]) / (x[i + 1] - x[i - 1]);
    double p = sig * y2[(i - 1) * stride] + 2.0;
    y2[i * stride] = (sig - 1.0) / p;
    double ui = (y[(i + 1) * stride] - y[i * stride]) / (x[i + 1] - x[i]) -
                (y[i * stride] - y[(i - 1) * stride]) / (x[i] - x[i - 1]);
    u[i] = (6.0 * ui / (x[i + 1] - x[i - 1]) - sig * u[i - 1]) / p;
  }
  double a = x[n - 3], b = x[n - 2], c = x[n - 1];
  double ya = y[(n - 3) * stride], yb = y[(n - 2) * stride], yc = y[(n - 1) * stride];
  double dyl = ((a - c) * (a - c) * (yb - yc) - (b - c) * (b - c) * (ya - yc)) / ((a - c) * (b - c) * (a - b));
  double qn = 0.5, un = (3. / (c - b)) * (dyl - (yc - yb) / (c - b));
  y2[(n - 1) * stride] = (un - qn * u[n - 2]) / (qn * y2[(n - 2) * stride] + 1.0);
  for (int k = n - 2; k >= 0; --k) y2[k * stride] = y2[k * stride] * y2[(k + 1) * stride] + u[k];
}

constexpr int MAXK3 = 256;

__global__ void ddk_kernel(int n_src, const int *__restrict__ src_tp, int n_pairs, int tau_size,
                           const double *__restrict__ k3, const int *__restrict__ k3_off, const int *__restrict__ k3_n,
                           const long long *__restrict__ src_off, long long per_type, const double *__restrict__ S,
                           double *__restrict__ ddk, int *__restrict__ status) {
  long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long total = (long long)n_src * n_pairs * tau_size;
  if (id >= total) return;
  int t = (int)(id % tau_size);
  long long r = id / tau_size;
  int p = (int)(r % n_pairs);
  int s = (int)(r / n_pairs);
  int n = k3_n[p];
  if (n > MAXK3) {
    atomicExch(status, 2);
    return;
  }
  double u[MAXK3];
  size_t base = (size_t)src_tp[s] * per_type + src_off[p] + (size_t)t * n;
  spline_gen(k3 + k3_off[p], S + base, 1, n, ddk + base, u);
}

// --------------------------------------------------- line of sight

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// exclusive scan of one value per thread (block-wide), returns the total
__device__ int block_exclusive_scan(int v, int *sh_warp, int &excl) {
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int incl = v;
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) sh_warp[w] = incl;
  __syncthreads();
  if (w == 0) {
    int t = (lane < LOS_WARPS) ? sh_warp[lane] : 0;
    int ti = t;
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, ti, o);
      if (lane >= o) ti += y;
    }
    if (lane < LOS_WARPS) sh_warp[lane] = ti - t;
    if (lane == LOS_WARPS - 1) sh_warp[LOS_WARPS] = ti;
  }
  __syncthreads();
  excl = sh_warp[w] + incl - v;
  int total = sh_warp[LOS_WARPS];
  __syncthreads();
  return total;
}

struct GridPtrs {
  double *tau, *dtau, *aJ, *a, *b, *h;
  int *ix, *left;
};

__device__ __forceinline__ GridPtrs grid_ptrs(double *base, int cap) {
  GridPtrs g;
  g.tau = base;
  g.dtau = base + cap;
  g.aJ = base + 2 * cap;
  g.a = base + 3 * cap;
  g.b = base + 4 * cap;
  g.h = base + 5 * cap;
  g.ix = reinterpret_cast<int *>(base + 6 * cap);
  g.left = g.ix + cap;
  return g;
}

constexpr int GRID_DOUBLES_PER_POINT = 7;
__host__ __device__ __forceinline__ int grid_doubles(int cap) { return GRID_DOUBLES_PER_POINT * cap; }

// INTERP_T: the integration grid is not the source sampling (time interpolation);
// CUBIC_J: cubic interpolation of the projection functions.  Both are template
// parameters so that the inner loop carries no runtime branch on them.
template <bool INTERP_T, bool CUBIC_J>
__global__ void __launch_bounds__(LOS_THREADS, 3) los_kernel(LosDev d, const double *__restrict__ S,
                                                          double *__restrict__ T) {
  extern __shared__ double sm[];
  __shared__ long long s_unit;
  __shared__ int s_scan[LOS_WARPS + 1];
  __shared__ int s_G;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int ts = d.tau_size;
  // shared layout: source rows [n_rows_src][ts]; with cubic time interpolation
  // their spline second derivatives and one recurrence scratch row per warp;
  // then the integration grid (or a global scratch slot of this CTA)
  const bool tcub = d.time_cubic && d.tau_sampling != SONG2_TAU_SAMPLING_SOURCES;
  double *Srow = sm;
  double *Sdd = Srow + (size_t)d.n_rows_src * ts;
  double *Su = Sdd + (size_t)d.n_rows_src * ts;
  double *gbase = d.time_cubic ? Su + (size_t)LOS_WARPS * ts : Sdd;
  if (!d.grid_in_smem) gbase = d.grid_scratch + (size_t)blockIdx.x * grid_doubles(d.grid_cap);
  GridPtrs g = grid_ptrs(gbase, d.grid_cap);

  for (;;) {
    if (tid == 0) s_unit = atomicAdd((unsigned long long *)d.queue, 1ull);
    __syncthreads();
    long long u = s_unit;
    __syncthreads();
    if (u >= d.n_units) break;
    const int p = d.unit_pair[u];
    const double k = d.unit_k[u];
    const int kl = d.unit_left[u];
    const double kb = d.unit_b[u], ka = 1.0 - kb;
    const int k3n = d.k3_n[p];
    const double *k3p = d.k3 + d.k3_off[p];
    const double kh = k3p[kl + 1] - k3p[kl];

    // 1. sources at k, every source row and time node
    for (int e = tid; e < d.n_rows_src * ts; e += LOS_THREADS) {
      int s = e / ts, t = e - s * ts;
      size_t base = (size_t)d.src_tp[s] * d.per_type + d.src_off[p] + (size_t)t * k3n + kl;
      double v = ka * S[base] + kb * S[base + 1];
      if (d.k3_cubic) v += ((ka * ka * ka - ka) * d.ddk[base] + (kb * kb * kb - kb) * d.ddk[base + 1]) * kh * kh / 6.0;
      Srow[e] = v;
    }
    __syncthreads();

    // 2. integration grid
    int G;
    if (d.tau_sampling == SONG2_TAU_SAMPLING_SOURCES) {
      G = ts;
      for (int i = tid; i < G; i += LOS_THREADS) {
        g.tau[i] = d.tau[i];
        g.left[i] = i;
      }
    } else {
      double step = (d.tau_sampling == SONG2_TAU_SAMPLING_CUSTOM) ? 2 * 3.141592653589793 / k * d.tau_linstep
                                                                  : d.x_step / k;
      // interval i = (tau_i, tau_{i+1}): points inserted by repeated steps from tau_i
      int total = 1;
      for (int i0 = 0; i0 < ts - 1; i0 += LOS_THREADS) {
        int i = i0 + tid, n = 0;
        if (i < ts - 1) {
          double t = d.tau[i];
          while (d.tau[i + 1] - t > step && n < d.grid_cap) {
            t += step;
            ++n;
          }
        }
        int excl;
        int chunk = block_exclusive_scan(i < ts - 1 ? n + 1 : 0, s_scan, excl);
        if (i < ts - 1) {
          int pos = total + excl;
          double t = d.tau[i];
          for (int j = 0; j < n; ++j) {
            t += step;
            if (pos + j < d.grid_cap) {
              g.tau[pos + j] = t;
              g.left[pos + j] = i + 1;  // the reference keeps the index of the next source time
            }
          }
          if (pos + n < d.grid_cap) {
            g.tau[pos + n] = d.tau[i + 1];
            g.left[pos + n] = i + 1;
          }
        }
        total += chunk;
      }
      if (tid == 0) {
        g.tau[0] = d.tau[0];
        g.left[0] = 0;
        s_G = total;
        if (total > d.grid_cap) atomicExch(d.status, 3);
      }
      __syncthreads();
      G = min(s_G, d.grid_cap);
      for (int i = tid; i < G; i += LOS_THREADS)
        if (g.left[i] == ts - 1) g.left[i] = ts - 2;
    }
    __syncthreads();
    // per grid point: trapezoid measure, x index and weight, time weights
    for (int i = tid; i < G; i += LOS_THREADS) {
      double ti = g.tau[i];
      double dt = (i == 0) ? g.tau[1] - g.tau[0] : (i == G - 1) ? g.tau[G - 1] - g.tau[G - 2] : g.tau[i + 1] - g.tau[i - 1];
      g.dtau[i] = dt;
      double x = k * (d.tau0 - ti);
      int ix = (int)(x / d.x_step);
      ix = max(0, min(ix, d.x_size - 2));  // in range by the host's check of k tau0 against x_max
      g.ix[i] = ix;
      g.aJ[i] = (s2los_x_of(ix + 1, d.x_size, d.x_max) - x) / d.x_step;
      if (d.tau_sampling != SONG2_TAU_SAMPLING_SOURCES) {
        int l = g.left[i];
        double h = d.tau[l + 1] - d.tau[l];
        double b = (ti - d.tau[l]) / h;
        g.b[i] = b;
        g.a[i] = 1.0 - b;
        g.h[i] = h;
      }
    }
    __syncthreads();
    // time spline of every source row, with estimated end derivatives
    // (transfer2_interpolate_sources_in_time, cubic): one row per warp, lane 0
    // runs the recurrence in its warp's scratch row
    if (tcub) {
      for (int s = warp; s < d.n_rows_src; s += LOS_WARPS)
        if (lane == 0) spline_gen(d.tau, Srow + (size_t)s * ts, 1, ts, Sdd + (size_t)s * ts, Su + (size_t)warp * ts);
      __syncthreads();
    }

    // 3. the integrals, one warp per transfer type, its lanes over the grid
    // points.  x = k (tau0 - tau) falls along the grid, so the points where any
    // term of the type can be non-negligible (ix >= the smallest x_min of its
    // terms) are a prefix of the grid, found by bisection; the rest add nothing.
    for (int o = warp; o < d.n_tt; o += LOS_WARPS) {
      const Term *tm = d.terms + (size_t)o * MAXTERM;
      const int nt = d.tt_nterm[o], nd = d.tt_ndir[o];
      const int xlo = d.tt_xmin[o];
      int P = 0;
      if (nt > 0 && g.ix[0] >= xlo) {
        int lo = 0, hi = G;  // g.ix[lo] >= xlo, and g.ix[hi] < xlo (hi == G: none)
        while (hi - lo > 1) {
          int mid = (lo + hi) >> 1;
          if (g.ix[mid] >= xlo) lo = mid;
          else hi = mid;
        }
        P = hi;
      }
      double dir = 0.0, mix = 0.0;
      for (int i = lane; i < P; i += 32) {
        const int ix = g.ix[i];
        const double aJ = g.aJ[i], bJ = 1 - aJ;
        int l = 0;
        double ta = 0.0, tb = 0.0, th = 0.0;
        if constexpr (INTERP_T) {
          l = g.left[i];
          ta = g.a[i];
          tb = g.b[i];
          th = g.h[i];
        }
        auto term = [&](const Term &t) -> double {
          const double *Jr = d.J + (size_t)t.row * d.x_size + ix;
          double Jv;
          if constexpr (!CUBIC_J) {
            Jv = aJ * __ldg(Jr) + bJ * __ldg(Jr + 1);
          } else {
            const double *dd = d.ddJ + (size_t)t.row * d.x_size + ix;
            Jv = (aJ * __ldg(Jr) + bJ * (__ldg(Jr + 1) - aJ * ((aJ + 1.) * __ldg(dd) + (2. - aJ) * __ldg(dd + 1)) *
                                                            d.x_step * d.x_step / 6.0));
          }
          const double *Sr = Srow + (size_t)t.tp * ts;
          double Sv;
          if constexpr (!INTERP_T) {
            Sv = Sr[i];
          } else {
            Sv = ta * Sr[l] + tb * Sr[l + 1];
            if (tcub) {
              const double *Sd = Sdd + (size_t)t.tp * ts;
              Sv += ((ta * ta * ta - ta) * Sd[l] + (tb * tb * tb - tb) * Sd[l + 1]) * th * th / 6.0;
            }
          }
          return Jv * Sv;
        };
        double sd = 0.0, sx = 0.0;
        for (int c = 0; c < nd; ++c) {
          const Term t = tm[c];
          if (ix >= t.xmin) sd += term(t);
        }
        for (int c = nd; c < nt; ++c) {
          const Term t = tm[c];
          if (ix >= t.xmin) sx += term(t);
        }
        dir += sd * g.dtau[i];
        mix += sx * g.dtau[i];
      }
      dir = warp_sum(dir);
      mix = warp_sum(mix);
      if (lane == 0) {
        // transfer2_integrate's 1/2 on each contribution, then transfer2_compute
        double direct = dir * 0.5, mixing = mix * 0.5;
        double tr = (d.tt_msign[o] < 0) ? direct - mixing : direct + mixing;
        tr /= 4.;
        tr /= (2. * d.tt_l[o] + 1);
        tr /= 2.;
        T[(size_t)o * d.n_units + u] = tr;
      }
    }
    __syncthreads();
  }
}

typedef void (*LosKernel)(LosDev, const double *, double *);

LosKernel los_kernel_for(bool interp_t, bool cubic_j) {
  if (interp_t) return cubic_j ? los_kernel<true, true> : los_kernel<true, false>;
  return cubic_j ? los_kernel<false, true> : los_kernel<false, false>;
}

}  // namespace

// ------------------------------------------------------------- host side

struct song2_los {
  song2_spec spec;
  song2_los_spec los;
  std::vector<int> l;
  std::vector<double> k, k3, tau;
  std::vector<int> k3_size;
  int x_size = 0, L_size = 0, m_size = 0, n_rows = 0, n_l1 = 0, n_tt = 0, n_pairs = 0, n_rows_src = 0;
  long long n_units = 0, per_type = 0;
  std::vector<int> l1;
  std::vector<int> jxmin, unit_size;  // host copies for the bispectrum integrals
  std::vector<double> unit_k;
  const double *d_unit_k = nullptr;
  double *d_ddj = nullptr;            // j_l1 spline table (cubic Bessel interpolation in the bispectrum)
  std::vector<void *> allocs;
  double *d_jtab = nullptr, *d_J = nullptr, *d_ddJ = nullptr, *d_ddk = nullptr, *d_grid = nullptr;
  int *d_Jxmin = nullptr, *d_status = nullptr, *d_queue = nullptr;
  LosDev dev{};
  size_t smem = 0;
  int grid = 0;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  float last_ms = 0.f, tables_ms = 0.f;
  LosKernel kernel = nullptr;
};

template <class T>
static int dev_upload(song2_los *h, const std::vector<T> &v, const T **out, char *err) {
  void *p = nullptr;
  size_t n = std::max<size_t>(1, v.size()) * sizeof(T);
  CKL(cudaMalloc(&p, n));
  h->allocs.push_back(p);
  if (!v.empty()) CKL(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  *out = (const T *)p;
  return 0;
}

static int dev_alloc(song2_los *h, size_t bytes, void **out, char *err) {
  CKL(cudaMalloc(out, std::max<size_t>(1, bytes)));
  h->allocs.push_back(*out);
  return 0;
}

// lm offset of (L, index_m) inside one source type block (l major, m <= l)
static int lm_offset(const song2_spec &s, int L, int im) {
  int n = 0;
  for (int l = 0; l < L; ++l)
    for (int i = 0; i < s.m_size; ++i)
      if (s.m[i] <= l) ++n;
  return n + im;
}

extern "C" int song2_los_create(const song2_spec *spec, const song2_los_spec *los, song2_los **out, char *err) {
  *out = nullptr;
  if (!spec || !los || !los->l || los->l_size < 1) {
    snprintf(err, SONG2_ERRLEN, "line-of-sight spec needs a multipole list");
    return 1;
  }
  if (!(los->tau0 > los->tau_rec) || !(los->tau_rec > 0) || !(los->x_step > 0) || !(los->x_max > los->x_step)) {
    snprintf(err, SONG2_ERRLEN, "line-of-sight spec: tau0=%g tau_rec=%g x_step=%g x_max=%g", los->tau0, los->tau_rec,
             los->x_step, los->x_max);
    return 1;
  }
  if (!spec->has_source_T && !spec->has_source_E && !spec->has_source_B) {
    snprintf(err, SONG2_ERRLEN, "no photon source types in the spec");
    return 1;
  }
  for (int i = 0; i < los->l_size; ++i)
    if (los->l[i] < 0 || (i && los->l[i] <= los->l[i - 1])) {
      snprintf(err, SONG2_ERRLEN, "multipole list must be ascending and non-negative");
      return 1;
    }
  song2_los *h = new song2_los();
  h->spec = *spec;
  h->los = *los;
  h->l.assign(los->l, los->l + los->l_size);
  h->los.l = h->l.data();
  const song2_spec &s = h->spec;
  h->k.assign(spec->k, spec->k + spec->k_size);
  h->k3_size.assign(spec->k3_size, spec->k3_size + (size_t)spec->k_size * spec->k_size);
  h->tau.assign(spec->tau, spec->tau + spec->tau_size);
  h->n_pairs = spec->k_size * (spec->k_size + 1) / 2;
  size_t nk3 = 0;
  for (int i1 = 0; i1 < spec->k_size; ++i1)
    for (int i2 = 0; i2 <= i1; ++i2) nk3 += spec->k3_size[i1 * spec->k_size + i2];
  h->k3.assign(spec->k3, spec->k3 + nk3);
  h->spec.k = h->k.data();
  h->spec.k3 = h->k3.data();
  h->spec.k3_size = h->k3_size.data();
  h->spec.tau = h->tau.data();
  auto fail = [&](void) {
    song2_los_destroy(h);
    return 1;
  };
  if (s.tau_size < 3) {
    snprintf(err, SONG2_ERRLEN, "line of sight needs at least 3 source times");
    return fail();
  }

  // ---- sizes
  const double x_max = h->los.x_max, x_step = h->los.x_step;
  h->x_size = s2los_x_size(x_max, x_step);
  int m_max = 0;
  for (int i = 0; i < s.m_size; ++i) m_max = std::max(m_max, s.m[i]);
  int l_los = 0;
  if (s.has_source_T) l_los = std::max(l_los, s.l_max_los_t);
  if (s.has_source_E || s.has_source_B) l_los = std::max(l_los, s.l_max_los_p);
  int L_max = std::max(l_los, m_max);  // pbs2->L_max (input2.c:2016)
  h->L_size = L_max + 1;
  h->m_size = s.m_size;
  const int l_size = h->los.l_size;
  h->n_rows = NJ * h->L_size * l_size * h->m_size;
  if (2 * L_max + 1 > MAXC) {
    snprintf(err, SONG2_ERRLEN, "L_max=%d too large for the projection rows", L_max);
    return fail();
  }

  // ---- extended l1 list (bessel2_get_l1_list, bessel2.c:832-958)
  {
    int Lx = L_max + m_max;
    int l1_top = h->l.back() + Lx;
    for (int l1 = 0; l1 <= l1_top; ++l1) {
      bool keep = false;
      for (int v : h->l)
        if (l1 >= v - Lx && l1 <= v + Lx) keep = true;
      if (keep) h->l1.push_back(l1);
    }
    h->n_l1 = (int)h->l1.size();
  }
  std::vector<int> l1_index(h->l1.back() + 1, -1);
  for (int r = 0; r < h->n_l1; ++r) l1_index[h->l1[r]] = r;
  std::vector<int> jxmin(h->n_l1);
  for (int r = 0; r < h->n_l1; ++r) jxmin[r] = s2los_bessel_xmin(h->l1[r], &h->los, h->x_size, x_max);
  h->jxmin = jxmin;

  // ---- projection rows (bessel2_J_for_Llm)
  const bool needT = s.has_source_T, needP = s.has_source_E || s.has_source_B;
  std::vector<int> nterm(h->n_rows, 0), jrow((size_t)h->n_rows * MAXC, 0), mode(h->n_rows, 0), up0(h->n_rows, 0),
      est(h->n_rows, 0);
  std::vector<double> coef((size_t)h->n_rows * MAXC, 0.0), rscale(h->n_rows, 0.0), upx(h->n_rows, 0.0);
  std::vector<double> f1(MAXC), f2(MAXC);
  for (int J = 0; J < NJ; ++J)
    for (int L = 0; L < h->L_size; ++L)
      for (int il = 0; il < l_size; ++il)
        for (int im = 0; im < h->m_size; ++im) {
          int row = ((J * h->L_size + L) * l_size + il) * h->m_size + im;
          int l = h->l[il], m = s.m[im];
          int S = (J == 0) ? 0 : 2;
          bool needed = (J == 0) ? needT : (needP && (J == 1 || m_max > 0));
          bool allowed = m <= std::min(L, l);
          bool spin = (S > l) || (S > L);
          bool eb0 = (J == 2) && (m == 0);
          est[row] = (l == 2);
          if (!needed || !allowed || spin || eb0) continue;  // negligible everywhere
          int lo1, hi1, lo2, hi2;
          if (song2_wigner3j_row(L, l, S, -S, &lo1, &hi1, f1.data(), MAXC) ||
              song2_wigner3j_row(L, l, -m, m, &lo2, &hi2, f2.data(), MAXC)) {
            snprintf(err, SONG2_ERRLEN, "3j row failed for (L,l,m)=(%d,%d,%d)", L, l, m);
            return fail();
          }
          int n = 0;
          for (int l1 = lo1; l1 <= hi1; ++l1) {
            double a = f1[l1 - lo1];
            if (a == 0.0) continue;
            double b = (l1 >= lo2 && l1 <= hi2) ? f2[l1 - lo2] : 0.0;
            bool even = ((l - l1 - L) % 2 == 0);
            double pref;
            if (J != 2) {
              if (!even) continue;
              pref = (((l - l1 - L) / 2) % 2 == 0) ? 1.0 : -1.0;
            } else {
              if (even) continue;
              pref = (((l - l1 - L - 1) / 2) % 2 == 0) ? 1.0 : -1.0;
            }
            int r1 = (l1 < (int)l1_index.size()) ? l1_index[l1] : -1;
            if (r1 < 0) {
              snprintf(err, SONG2_ERRLEN, "l1=%d missing from the extended list", l1);
              return fail();
            }
            coef[(size_t)row * MAXC + n] = pref * (2 * l1 + 1) * a * b;
            jrow[(size_t)row * MAXC + n] = r1;
            ++n;
          }
          nterm[row] = n;
          rscale[row] = (double)((m % 2 == 0 ? 1 : -1) * (2 * l + 1));
          if (L == l) {
            mode[row] = 1;
          } else {
            mode[row] = 2;
            double xu = lo1 + 0.5;
            if (xu >= x_max) {
              up0[row] = h->x_size - 1;
              upx[row] = x_max;
            } else {
              int i = 0;
              while (s2los_x_of(i, h->x_size, x_max) < xu) ++i;
              up0[row] = i;
              upx[row] = s2los_x_of(i, h->x_size, x_max);
            }
          }
        }

  // ---- transfer types and their (J, L) terms; shared source rows
  std::vector<int> tp_of((size_t)3 * h->L_size * h->m_size, -1);  // [type][L][im] -> shared row
  std::vector<int> src_tp;
  int base = 0;
  const int has[3] = {s.has_source_T, s.has_source_E, s.has_source_B};
  const int lmax_t[3] = {s.l_max_los_t, s.l_max_los_p, s.l_max_los_p};
  for (int t = 0; t < 3; ++t) {
    if (!has[t]) continue;
    for (int L = 0; L <= lmax_t[t] && L < h->L_size; ++L)
      for (int im = 0; im < h->m_size; ++im)
        if (s.m[im] <= L) {
          tp_of[((size_t)t * h->L_size + L) * h->m_size + im] = (int)src_tp.size();
          src_tp.push_back(base + lm_offset(s, L, im));
        }
    base += lm_offset(s, lmax_t[t] + 1, 0);
  }
  h->n_rows_src = (int)src_tp.size();
  h->n_tt = song2_transfer_types(&h->spec, &h->los, nullptr, nullptr, nullptr);
  std::vector<int> tt_type(h->n_tt), tt_l(h->n_tt), tt_m(h->n_tt), tt_nterm(h->n_tt, 0);
  std::vector<double> tt_msign(h->n_tt, 1.0);
  std::vector<int> tt_ndir(h->n_tt, 0);
  song2_transfer_types(&h->spec, &h->los, tt_type.data(), tt_l.data(), tt_m.data());
  std::vector<Term> terms((size_t)h->n_tt * MAXTERM);
  for (int o = 0; o < h->n_tt; ++o) {
    int il = (int)(std::lower_bound(h->l.begin(), h->l.end(), tt_l[o]) - h->l.begin());
    int im = 0;
    while (s.m[im] != tt_m[o]) ++im;
    int m = tt_m[o], l = tt_l[o];
    // (J, source type, sign, mixing) per output type (transfer2_compute)
    int nj = 0;
    int Js[2], St[2], Mx[2];
    double Sg[2];
    if (tt_type[o] == SONG2_TT_T) {
      Js[0] = 0; St[0] = 0; Sg[0] = 1; Mx[0] = 0; nj = 1;
    } else if (tt_type[o] == SONG2_TT_E) {
      Js[0] = 1; St[0] = 1; Sg[0] = 1; Mx[0] = 0; nj = 1;
      if (m != 0 && has[2]) { Js[1] = 2; St[1] = 2; Sg[1] = 1; Mx[1] = 1; nj = 2; }
    } else {
      Js[0] = 1; St[0] = 2; Sg[0] = 1; Mx[0] = 0; nj = 1;
      if (has[1]) { Js[1] = 2; St[1] = 1; Sg[1] = -1; Mx[1] = 1; nj = 2; }
    }
    int Lmax_o = (tt_type[o] == SONG2_TT_T) ? s.l_max_los_t : s.l_max_los_p;
    int n = 0;
    for (int q = 0; q < nj; ++q)
      for (int L = 0; L <= Lmax_o; ++L) {
        if (m > std::min(L, l)) continue;
        int tp = tp_of[((size_t)St[q] * h->L_size + L) * h->m_size + im];
        if (tp < 0) continue;
        if (n >= MAXTERM) {
          snprintf(err, SONG2_ERRLEN, "too many projection terms for one transfer type");
          return fail();
        }
        Term &t = terms[(size_t)o * MAXTERM + n++];
        t.row = ((Js[q] * h->L_size + L) * l_size + il) * h->m_size + im;
        t.tp = tp;
        t.xmin = 0;  // filled from the device x_min table below
        t.mix = Mx[q];
        if (Mx[q]) tt_msign[o] = Sg[q];
        else tt_ndir[o]++;
      }
    tt_nterm[o] = n;
  }

  // ---- transfer k grids and the k3 interpolation of each unit
  std::vector<int> ksz(h->n_pairs), kps(h->n_pairs), kpn(h->n_pairs);
  long long nu = song2_transfer_k_grids(&h->spec, &h->los, ksz.data(), kps.data(), kpn.data(), nullptr, err);
  if (nu < 0) return fail();
  std::vector<double> unit_k(nu);
  song2_transfer_k_grids(&h->spec, &h->los, nullptr, nullptr, nullptr, unit_k.data(), err);
  h->n_units = nu;
  std::vector<int> unit_pair(nu), unit_left(nu), k3off(h->n_pairs), k3n(h->n_pairs);
  std::vector<double> unit_b(nu);
  std::vector<long long> src_off(h->n_pairs);
  {
    long long u = 0, soff = 0;
    int p = 0, koff = 0;
    for (int i1 = 0; i1 < s.k_size; ++i1)
      for (int i2 = 0; i2 <= i1; ++i2, ++p) {
        int n3 = s.k3_size[i1 * s.k_size + i2];
        const double *kp = h->k3.data() + koff;
        k3off[p] = koff;
        k3n[p] = n3;
        src_off[p] = soff;
        // monotone search of transfer2_interpolate_sources_in_k over the physical points
        int ik = 0;
        int first = kps[p], last = kps[p] + kpn[p] - 1;
        std::vector<int> lf(ksz[p]);
        std::vector<double> bf(ksz[p]);
        for (int it = first; it <= last; ++it) {
          double kt = unit_k[u + it];
          while (ik + 1 < n3 && kp[ik + 1] < kt) ++ik;
          if (ik + 1 >= n3) ik = n3 - 2;
          double hh = kp[ik + 1] - kp[ik];
          lf[it] = ik;
          bf[it] = (kt - kp[ik]) / hh;
        }
        for (int it = 0; it < ksz[p]; ++it) {
          int src = it < first ? first : (it > last ? last : it);  // flat extrapolation
          unit_pair[u + it] = p;
          unit_left[u + it] = lf[src];
          unit_b[u + it] = bf[src];
        }
        u += ksz[p];
        koff += n3;
        soff += (long long)s.tau_size * n3;
      }
    h->per_type = soff;
  }

  // ---- device tables
  cudaEventCreate(&h->e0);
  cudaEventCreate(&h->e1);
  const int *d_l1, *d_jxmin, *d_nterm, *d_jrow, *d_mode, *d_up0, *d_est;
  const double *d_coef, *d_rscale, *d_upx;
  if (dev_upload(h, h->l1, &d_l1, err) || dev_upload(h, jxmin, &d_jxmin, err) || dev_upload(h, nterm, &d_nterm, err) ||
      dev_upload(h, jrow, &d_jrow, err) || dev_upload(h, mode, &d_mode, err) || dev_upload(h, up0, &d_up0, err) ||
      dev_upload(h, est, &d_est, err) || dev_upload(h, coef, &d_coef, err) || dev_upload(h, rscale, &d_rscale, err) ||
      dev_upload(h, upx, &d_upx, err))
    return fail();
  void *tmp;
  if (dev_alloc(h, sizeof(double) * (size_t)h->n_l1 * h->x_size, &tmp, err)) return fail();
  h->d_jtab = (double *)tmp;
  if (dev_alloc(h, sizeof(double) * (size_t)h->n_rows * h->x_size, &tmp, err)) return fail();
  h->d_J = (double *)tmp;
  if (dev_alloc(h, sizeof(int) * h->n_rows, &tmp, err)) return fail();
  h->d_Jxmin = (int *)tmp;
  if (dev_alloc(h, sizeof(int) * 4, &tmp, err)) return fail();
  h->d_status = (int *)tmp;
  if (dev_alloc(h, sizeof(unsigned long long), &tmp, err)) return fail();
  h->d_queue = (int *)tmp;
  CKL(cudaMemset(h->d_status, 0, sizeof(int) * 4));
  CKL(cudaEventRecord(h->e0, 0));
  jl_kernel<<<(h->x_size + 127) / 128, 128>>>(h->x_size, x_max, h->n_l1, d_l1, d_jxmin, h->d_jtab);
  {
    dim3 gJ((h->x_size + 255) / 256, h->n_rows);
    J_kernel<<<gJ, 256>>>(h->x_size, h->n_rows, d_nterm, d_coef, d_jrow, d_rscale, h->d_jtab, h->d_J);
  }
  Jxmin_kernel<<<(h->n_rows + 127) / 128, 128>>>(h->x_size, h->n_rows, d_mode, d_up0, d_upx, x_max, h->los.J_cut,
                                                 h->d_J, h->d_Jxmin, h->d_status);
  if (h->los.bessel_interpolation == SONG2_INTERP_CUBIC) {
    if (dev_alloc(h, sizeof(double) * (size_t)h->n_rows * h->x_size, &tmp, err)) return fail();
    h->d_ddJ = (double *)tmp;
    double *scratch;
    CKL(cudaMalloc((void **)&scratch, sizeof(double) * (size_t)h->n_rows * h->x_size));
    ddJ_kernel<<<(h->n_rows + 63) / 64, 64>>>(h->x_size, x_max, h->n_rows, h->d_Jxmin, d_est, h->d_J, h->d_ddJ,
                                              scratch);
    cudaError_t e = cudaDeviceSynchronize();
    cudaFree(scratch);
    CKL(e);
  }
  CKL(cudaEventRecord(h->e1, 0));
  CKL(cudaEventSynchronize(h->e1));
  CKL(cudaGetLastError());
  CKL(cudaEventElapsedTime(&h->tables_ms, h->e0, h->e1));
  int st[4];
  CKL(cudaMemcpy(st, h->d_status, sizeof(st), cudaMemcpyDeviceToHost));
  if (st[0]) {
    snprintf(err, SONG2_ERRLEN, "projection function negligible at its first peak (bessel2.c:1355-1366)");
    return fail();
  }
  // x_min of each term
  std::vector<int> Jxmin(h->n_rows);
  CKL(cudaMemcpy(Jxmin.data(), h->d_Jxmin, sizeof(int) * h->n_rows, cudaMemcpyDeviceToHost));
  // drop the terms whose projection row is negligible at every x (x index
  // x_size - 1 is never reached), keeping the direct terms first, and record
  // each type's smallest x_min
  std::vector<int> tt_xmin(h->n_tt, h->x_size);
  for (int o = 0; o < h->n_tt; ++o) {
    Term *to = terms.data() + (size_t)o * MAXTERM;
    int n = 0, nd = 0;
    for (int c = 0; c < tt_nterm[o]; ++c) {
      Term t = to[c];
      t.xmin = Jxmin[t.row];
      if (t.xmin >= h->x_size - 1) continue;
      if (!t.mix) ++nd;
      to[n++] = t;
      tt_xmin[o] = std::min(tt_xmin[o], t.xmin);
    }
    tt_nterm[o] = n;
    tt_ndir[o] = nd;
  }

  // ---- every x = k (tau0 - tau) inside the projection tables
  {
    double kmax = 0;
    for (double v : unit_k) kmax = std::max(kmax, v);
    if (h->tau.back() > h->los.tau0 || h->tau.front() <= 0) {
      snprintf(err, SONG2_ERRLEN, "source times must lie in (0, tau0=%g]", h->los.tau0);
      return fail();
    }
    double xm = kmax * (h->los.tau0 - h->tau.front());
    if ((int)(xm / x_step) > h->x_size - 2) {
      snprintf(err, SONG2_ERRLEN, "x_max=%g does not cover k (tau0 - tau) = %g; increase x_max", x_max, xm);
      return fail();
    }
  }

  // ---- integration grid capacity
  int cap = s.tau_size;
  if (h->los.tau_sampling != SONG2_TAU_SAMPLING_SOURCES) {
    double kmax = 0;
    for (double v : unit_k) kmax = std::max(kmax, v);
    double step = (h->los.tau_sampling == SONG2_TAU_SAMPLING_CUSTOM) ? 2 * 3.141592653589793 / kmax * h->los.tau_linstep
                                                                     : x_step / kmax;
    double span = h->tau.back() - h->tau.front();
    double c = 2.0 * s.tau_size + span / step + 4;
    if (c > 5e6) {
      snprintf(err, SONG2_ERRLEN, "integration grid of %g points per k is too large", c);
      return fail();
    }
    cap = (int)c;
  }

  // ---- device description of the integral
  LosDev &d = h->dev;
  d.x_size = h->x_size;
  d.x_max = x_max;
  d.x_step = x_step;
  d.J = h->d_J;
  d.ddJ = h->d_ddJ;
  d.Jxmin = h->d_Jxmin;
  d.tau_size = s.tau_size;
  d.k_size = s.k_size;
  const double *p_tau, *p_k3, *p_unit_k, *p_unit_b;
  const int *p_k3off, *p_k3n, *p_unit_pair, *p_unit_left, *p_src_tp, *p_tt_l, *p_tt_nterm;
  const double *p_tt_msign;
  const int *p_tt_ndir, *p_tt_xmin;
  const long long *p_src_off;
  const Term *p_terms;
  if (dev_upload(h, h->tau, &p_tau, err) || dev_upload(h, h->k3, &p_k3, err) || dev_upload(h, k3off, &p_k3off, err) ||
      dev_upload(h, k3n, &p_k3n, err) || dev_upload(h, src_off, &p_src_off, err) ||
      dev_upload(h, unit_k, &p_unit_k, err) || dev_upload(h, unit_b, &p_unit_b, err) ||
      dev_upload(h, unit_pair, &p_unit_pair, err) || dev_upload(h, unit_left, &p_unit_left, err) ||
      dev_upload(h, src_tp, &p_src_tp, err) || dev_upload(h, tt_l, &p_tt_l, err) ||
      dev_upload(h, tt_nterm, &p_tt_nterm, err) || dev_upload(h, terms, &p_terms, err) ||
      dev_upload(h, tt_msign, &p_tt_msign, err) || dev_upload(h, tt_ndir, &p_tt_ndir, err) ||
      dev_upload(h, tt_xmin, &p_tt_xmin, err))
    return fail();
  h->unit_k = unit_k;
  h->unit_size = ksz;
  h->d_unit_k = p_unit_k;
  d.tau = p_tau;
  d.k3 = p_k3;
  d.k3_off = p_k3off;
  d.k3_n = p_k3n;
  d.src_off = p_src_off;
  d.per_type = h->per_type;
  d.n_units = h->n_units;
  d.unit_pair = p_unit_pair;
  d.unit_k = p_unit_k;
  d.unit_left = p_unit_left;
  d.unit_b = p_unit_b;
  d.n_rows_src = h->n_rows_src;
  d.src_tp = p_src_tp;
  d.n_tt = h->n_tt;
  d.tt_l = p_tt_l;
  d.tt_msign = p_tt_msign;
  d.tt_ndir = p_tt_ndir;
  d.tt_xmin = p_tt_xmin;
  d.tt_nterm = p_tt_nterm;
  d.terms = p_terms;
  d.tau_sampling = h->los.tau_sampling;
  d.time_cubic = h->los.time_interpolation == SONG2_INTERP_CUBIC;
  d.k3_cubic = h->los.k3_interpolation == SONG2_INTERP_CUBIC;
  d.bessel_cubic = h->los.bessel_interpolation == SONG2_INTERP_CUBIC;
  d.tau_linstep = h->los.tau_linstep;
  d.tau0 = h->los.tau0;
  d.grid_cap = cap;
  d.queue = h->d_queue;
  d.status = h->d_status;
  int dev_id = 0, n_sm = 0;
  size_t smem_optin = 0;
  cudaGetDevice(&dev_id);
  cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev_id);
  {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev_id);
    smem_optin = (size_t)v;
  }
  size_t s_src = sizeof(double) * ((size_t)h->n_rows_src * s.tau_size * (d.time_cubic ? 2 : 1) +
                                    (d.time_cubic ? (size_t)LOS_WARPS * s.tau_size : 0));
  size_t s_grid = sizeof(double) * (size_t)grid_doubles(cap);
  d.grid_in_smem = (cap <= GRID_SMEM_MAX) && (s_src + s_grid + 1024 <= smem_optin);
  h->smem = s_src + (d.grid_in_smem ? s_grid : 0);
  if (h->smem + 1024 > smem_optin) {
    snprintf(err, SONG2_ERRLEN, "source rows of one k (%zu bytes) exceed shared memory", s_src);
    return fail();
  }
  h->kernel = los_kernel_for(d.tau_sampling != SONG2_TAU_SAMPLING_SOURCES, d.bessel_cubic);
  CKL(cudaFuncSetAttribute(h->kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)h->smem));
  int per_sm = 0;
  CKL(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, h->kernel, LOS_THREADS, h->smem));
  if (per_sm < 1) {
    snprintf(err, SONG2_ERRLEN, "line-of-sight kernel does not fit on an SM");
    return fail();
  }
  h->grid = (int)std::min<long long>((long long)per_sm * n_sm, std::max<long long>(1, h->n_units));
  if (!d.grid_in_smem) {
    if (dev_alloc(h, sizeof(double) * (size_t)grid_doubles(cap) * h->grid, &tmp, err)) return fail();
    d.grid_scratch = (double *)tmp;
  }
  if (d.k3_cubic) {
    size_t n = (size_t)song2_tp2_size(&h->spec) * h->per_type;
    if (dev_alloc(h, sizeof(double) * n, &tmp, err)) return fail();
    h->d_ddk = (double *)tmp;
    d.ddk = h->d_ddk;
  }
  *out = h;
  return 0;
}

int s2los_view(song2_los *h, S2LosView *v, char *err) {
  if (h->los.bessel_interpolation == SONG2_INTERP_CUBIC && !h->d_ddj) {
    // natural spline of each j_l1 row from its x_min on (bessel2.c:437-456)
    void *tmp;
    if (dev_alloc(h, sizeof(double) * (size_t)h->n_l1 * h->x_size, &tmp, err)) return 1;
    h->d_ddj = (double *)tmp;
    CKL(cudaMemset(h->d_ddj, 0, sizeof(double) * (size_t)h->n_l1 * h->x_size));
    const int *d_xmin, *d_est;
    std::vector<int> zeros(h->n_l1, 0);
    if (dev_upload(h, h->jxmin, &d_xmin, err) || dev_upload(h, zeros, &d_est, err)) return 1;
    double *scratch;
    CKL(cudaMalloc((void **)&scratch, sizeof(double) * (size_t)h->n_l1 * h->x_size));
    ddJ_kernel<<<(h->n_l1 + 63) / 64, 64>>>(h->x_size, h->los.x_max, h->n_l1, d_xmin, d_est, h->d_jtab, h->d_ddj,
                                            scratch);
    cudaError_t e = cudaDeviceSynchronize();
    cudaFree(scratch);
    CKL(e);
  }
  v->spec = &h->spec;
  v->los = &h->los;
  v->l_size = h->los.l_size;
  v->l = h->l.data();
  v->x_size = h->x_size;
  v->x_max = h->los.x_max;
  v->x_step = h->los.x_step;
  v->n_l1 = h->n_l1;
  v->l1 = h->l1.data();
  v->jxmin = h->jxmin.data();
  v->jtab_dev = h->d_jtab;
  v->ddj_dev = h->d_ddj;
  v->n_pairs = h->n_pairs;
  v->n_units = h->n_units;
  v->unit_size = h->unit_size.data();
  v->unit_k = h->unit_k.data();
  v->unit_k_dev = h->d_unit_k;
  v->n_tt = h->n_tt;
  return 0;
}

extern "C" void song2_los_destroy(song2_los *h) {
  if (!h) return;
  for (void *p : h->allocs) cudaFree(p);
  if (h->e0) cudaEventDestroy(h->e0);
  if (h->e1) cudaEventDestroy(h->e1);
  delete h;
}

extern "C" int64_t song2_los_transfer_size(const song2_los *h) { return (int64_t)h->n_tt * h->n_units; }

extern "C" float song2_los_last_ms(const song2_los *h) { return h->last_ms; }
extern "C" float song2_los_tables_ms(const song2_los *h) { return h->tables_ms; }

extern "C" int song2_los_run(song2_los *h, const double *sources_dev, double *transfer_dev, void *stream, char *err) {
  cudaStream_t st = (cudaStream_t)stream;
  CKL(cudaEventRecord(h->e0, st));
  CKL(cudaMemsetAsync(h->d_queue, 0, sizeof(unsigned long long), st));
  CKL(cudaMemsetAsync(h->d_status, 0, sizeof(int) * 4, st));
  if (h->dev.k3_cubic) {
    long long total = (long long)h->n_rows_src * h->n_pairs * h->spec.tau_size;
    ddk_kernel<<<(unsigned)((total + 127) / 128), 128, 0, st>>>(h->n_rows_src, h->dev.src_tp, h->n_pairs,
                                                                 h->spec.tau_size, h->dev.k3, h->dev.k3_off,
                                                                 h->dev.k3_n, h->dev.src_off, h->per_type,
                                                                 sources_dev, h->d_ddk, h->d_status);
  }
  h->kernel<<<h->grid, LOS_THREADS, h->smem, st>>>(h->dev, sources_dev, transfer_dev);
  CKL(cudaGetLastError());
  CKL(cudaEventRecord(h->e1, st));
  CKL(cudaEventSynchronize(h->e1));
  CKL(cudaEventElapsedTime(&h->last_ms, h->e0, h->e1));
  int stt[4];
  CKL(cudaMemcpy(stt, h->d_status, sizeof(stt), cudaMemcpyDeviceToHost));
  if (stt[0] == 2) {
    snprintf(err, SONG2_ERRLEN, "k3 grid longer than %d points for the cubic k3 interpolation", MAXK3);
    return 1;
  }
  if (stt[0] == 3) {
    snprintf(err, SONG2_ERRLEN, "integration grid exceeded its capacity of %d points", h->dev.grid_cap);
    return 1;
  }
  return 0;
}

extern "C" void song2_los_table_sizes(const song2_los *h, int *x_size, int *n_l1, int *L_size, int *m_size,
                                      int *n_rows) {
  if (x_size) *x_size = h->x_size;
  if (n_l1) *n_l1 = h->n_l1;
  if (L_size) *L_size = h->L_size;
  if (m_size) *m_size = h->m_size;
  if (n_rows) *n_rows = h->n_rows;
}

extern "C" int song2_los_tables(song2_los *h, int *l1, double *j_l1, double *J, int *J_xmin, char *err) {
  if (l1) memcpy(l1, h->l1.data(), sizeof(int) * h->n_l1);
  if (j_l1) CKL(cudaMemcpy(j_l1, h->d_jtab, sizeof(double) * (size_t)h->n_l1 * h->x_size, cudaMemcpyDeviceToHost));
  if (J) CKL(cudaMemcpy(J, h->d_J, sizeof(double) * (size_t)h->n_rows * h->x_size, cudaMemcpyDeviceToHost));
  if (J_xmin) CKL(cudaMemcpy(J_xmin, h->d_Jxmin, sizeof(int) * h->n_rows, cudaMemcpyDeviceToHost));
  return 0;
}

extern "C" int song2_gpu_transfer(const song2_spec *spec, const song2_los_spec *los, const double *sources_flat,
                                  double *transfer_flat, char *err) {
  song2_los *h = nullptr;
  if (song2_los_create(spec, los, &h, err)) return 1;
  size_t n_src = (size_t)song2_tp2_size(spec) * h->per_type;
  size_t n_out = (size_t)song2_los_transfer_size(h);
  double *d_src = nullptr, *d_out = nullptr;
  int rc = 0;
  if (cudaMalloc((void **)&d_src, sizeof(double) * std::max<size_t>(1, n_src)) != cudaSuccess ||
      cudaMalloc((void **)&d_out, sizeof(double) * std::max<size_t>(1, n_out)) != cudaSuccess) {
    snprintf(err, SONG2_ERRLEN, "device allocation failed for the sources and transfers");
    rc = 1;
  }
  if (!rc && cudaMemcpy(d_src, sources_flat, sizeof(double) * n_src, cudaMemcpyHostToDevice) != cudaSuccess) {
    snprintf(err, SONG2_ERRLEN, "upload of the sources failed");
    rc = 1;
  }
  if (!rc) rc = song2_los_run(h, d_src, d_out, nullptr, err);
  if (!rc && cudaMemcpy(transfer_flat, d_out, sizeof(double) * n_out, cudaMemcpyDeviceToHost) != cudaSuccess) {
    snprintf(err, SONG2_ERRLEN, "download of the transfers failed");
    rc = 1;
  }
  cudaFree(d_src);
  cudaFree(d_out);
  song2_los_destroy(h);
  return rc;
}
