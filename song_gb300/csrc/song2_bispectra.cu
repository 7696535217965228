// song2_bispectra.cu - the intrinsic bispectrum of the second-order transfer
// functions on the GPU (bispectra2_intrinsic_init and its integrals,
// bispectra2.c:300-3030).
//
// The reference integrates k3, then k2, k1 and r one after the other, each
// k1/k2 step interpolating the previous integral from the smooth grid of the
// sources onto the first-order transfer grid q and convolving it there with a
// Bessel function and a first-order transfer function.  The interpolation (a
// linear or cubic spline in k) is linear in the values it interpolates, so the
// q sums are moved in front of it: for every (l, r) the product
//   c(q) = dq q^4 j_L(r q) T1_l(q) P(q)
// is folded once into weights over the k grid (C for k2, D for k1 with the r
// measure), and the k2 and k1 integrals become small dot products over the k
// grid.  The result equals the reference's up to rounding; the cost of the
// k2 step drops from l3 r k1 (q + l2 q) to l3 r k1 l2 k.
//
// Kernels:
//   coef_kernel   C[Y][r][l2][k] and D[Z, M3, offset_L1][l1][r][k], once per
//                 handle (they depend only on the first-order inputs);
//                 split_rows_kernel scales their rows by powers of two and
//                 splits them into double-float (hi + lo floats);
//   k3_kernel     I3[l3][r][pair] = 2 c_M3 * 1/2 sum dk3 k3^2 j_L3(r k3) T2,
//                 one thread per (l3, pair, r), FP64;
//   k2_kernel     I2[l3][l2][r][k1] = sum_k C[r][l2][k] I3sym[l3][r][k1][k],
//                 one block per (l3, r), double-float dot products;
//   geo_kernel    the geometrical factor of every (l3, l2, l1) triangle and L1
//                 offset for one (M3, L3 offset);
//   k1r_kernel    sum_r sum_k D[l1][r][k] I2[l3][l2][r][k] for every l1 of the
//                 (l3, l2) triangles of two l2, every Z and L1 offset, times
//                 the geometrical factors, accumulated into the unsymmetrised
//                 bispectrum; double-float dot products;
//   sym_kernel    the sum over the position of the second-order field.
// Double-float keeps about 46 bits: GB300's FP32 pipe has 64 times the rate of
// its FP64 pipe, and these contractions are the bulk of the work.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "song2.h"
#include "song2_los.h"
#include "song2_los_view.h"

#define CKB(x)                                                                                     \
  do {                                                                                             \
    cudaError_t e_ = (x);                                                                          \
    if (e_ != cudaSuccess) {                                                                       \
      snprintf(err, SONG2_ERRLEN, "%s:%d %s: %s", __FILE__, __LINE__, #x, cudaGetErrorString(e_)); \
      return 1;                                                                                    \
    }                                                                                              \
  } while (0)

namespace {

constexpr int BI_THREADS = 256;
constexpr int BI_WARPS = BI_THREADS / 32;
constexpr int BI_MAX_K = 128;  // k grid size held in shared memory by k2_kernel
constexpr double BI_PI = 3.141592653589793238462643383279502884;

// field parity: T and E even, B odd
int field_parity(int f) { return f == SONG2_TT_B ? 1 : 0; }

// ------------------------------------------------------------ 3j and 6j
// From a table of ln n! (filled on the host in long double).

__device__ __forceinline__ bool triangle(int a, int b, int c) { return c >= abs(a - b) && c <= a + b; }

// (j1 j2 j3; 0 0 0), closed form
__device__ double w3j000(int j1, int j2, int j3, const double *__restrict__ lf) {
  if (!triangle(j1, j2, j3)) return 0.0;
  int J = j1 + j2 + j3;
  if (J & 1) return 0.0;
  int g = J / 2;
  double v = exp(0.5 * (lf[J - 2 * j1] + lf[J - 2 * j2] + lf[J - 2 * j3] - lf[J + 1]) + lf[g] - lf[g - j1] -
                 lf[g - j2] - lf[g - j3]);
  return (g & 1) ? -v : v;
}

// (j1 j2 j3; m1 m2 m3), Racah's sum (few terms when one j is small)
__device__ double w3j(int j1, int j2, int j3, int m1, int m2, int m3, const double *__restrict__ lf) {
  if (m1 + m2 + m3 != 0 || !triangle(j1, j2, j3) || abs(m1) > j1 || abs(m2) > j2 || abs(m3) > j3) return 0.0;
  if (m1 == 0 && m2 == 0) return w3j000(j1, j2, j3, lf);
  double pre = 0.5 * (lf[j1 + j2 - j3] + lf[j1 - j2 + j3] + lf[-j1 + j2 + j3] - lf[j1 + j2 + j3 + 1] + lf[j1 + m1] +
                      lf[j1 - m1] + lf[j2 + m2] + lf[j2 - m2] + lf[j3 + m3] + lf[j3 - m3]);
  int kmin = max(0, max(j2 - j3 - m1, j1 - j3 + m2));
  int kmax = min(j1 + j2 - j3, min(j1 - m1, j2 + m2));
  double s = 0.0;
  for (int k = kmin; k <= kmax; ++k) {
    double t = exp(pre - (lf[k] + lf[j3 - j2 + k + m1] + lf[j3 - j1 + k - m2] + lf[j1 + j2 - j3 - k] +
                          lf[j1 - k - m1] + lf[j2 - k + m2]));
    s += (k & 1) ? -t : t;
  }
  return ((j1 - j2 - m3) & 1) ? -s : s;
}

__device__ __forceinline__ double ldelta(int a, int b, int c, const double *__restrict__ lf) {
  return lf[a + b - c] + lf[a - b + c] + lf[-a + b + c] - lf[a + b + c + 1];
}

// {a b c; d e f}, Racah's sum
__device__ double w6j(int a, int b, int c, int d, int e, int f, const double *__restrict__ lf) {
  if (!triangle(a, b, c) || !triangle(a, e, f) || !triangle(d, b, f) || !triangle(d, e, c)) return 0.0;
  double ld = 0.5 * (ldelta(a, b, c, lf) + ldelta(a, e, f, lf) + ldelta(d, b, f, lf) + ldelta(d, e, c, lf));
  int tmin = max(max(a + b + c, a + e + f), max(d + b + f, d + e + c));
  int tmax = min(a + b + d + e, min(b + c + e + f, c + a + f + d));
  double s = 0.0;
  for (int t = tmin; t <= tmax; ++t) {
    double v = exp(ld + lf[t + 1] -
                   (lf[t - a - b - c] + lf[t - a - e - f] + lf[t - d - b - f] + lf[t - d - e - c] +
                    lf[a + b + d + e - t] + lf[b + c + e + f - t] + lf[c + a + f + d - t]));
    s += (t & 1) ? -v : v;
  }
  return s;
}

// ------------------------------------------------------------ Bessel j_L(x)
// bessel2_convolution's interpolation (bessel2.c:565-590): the row's table
// starts at its x_min node, steps of x_step from there.
struct JTab {
  const double *tab, *dd;
  const int *xmin;     // per row: first stored x index
  const double *xmin_u;  // per row: its x (the lin_space node) over x_step
  int x_size;
  double x_max, x_step, inv_step;
  int cubic;
  int *status;
};

// j_L(k r) with rs = r / x_step: u = (k r - x_min) / x_step as one fma
__device__ __forceinline__ double jl_at(const JTab &t, int row, double k, double rs) {
  // index and weight of bessel2_convolution, (xm + x_step (ix + 1) - x) / x_step,
  // written as ix + 1 - u
  const double u = fma(k, rs, -__ldg(&t.xmin_u[row]));
  if (u < 0.0) return 0.0;
  const int x0 = __ldg(&t.xmin[row]);
  int ix = (int)u;
  if (x0 + ix + 1 >= t.x_size) {  // outside the table: record and drop the term
    atomicOr(t.status, 1);
    return 0.0;
  }
  double a = (double)(ix + 1) - u;
  const double *r = t.tab + (size_t)row * t.x_size + x0 + ix;
  if (!t.cubic) {
    const double j1 = __ldg(r + 1);
    return fma(a, __ldg(r) - j1, j1);
  }
  const double *q = t.dd + (size_t)row * t.x_size + x0 + ix;
  return a * __ldg(r) +
         (1. - a) * (__ldg(r + 1) - a * ((a + 1.) * __ldg(q) + (2. - a) * __ldg(q + 1)) * t.x_step * t.x_step / 6.0);
}

// ------------------------------------------------------------ coefficients
// For every (l, r): out[k] = rfac(r) window(k) sum_q c(q) W(q, k), with
// c(q) = qw(q) j_L(r q) T1_l(q) and W the interpolation weights of the k grid.
// One thread per k interval sums the q of its interval (deterministic order).
struct CoefArgs {
  JTab jt;
  int l_size, r_size, k_size, q_size, cubic;
  const int *row_of_l;   // [l_size] Bessel row of the order used for each l (-1: zero)
  const double *T1;      // [l_size][q_size]
  const double *q, *qw;  // q, dq q^4 P(q)
  const double *qa, *qb; // linear weights of q in its interval
  const int *qbeg;       // [k_size]: first q of each interval (interval k_size - 1 empty)
  const double *hk;      // [k_size - 1] interval widths
  const double *S;       // [k_size][k_size] spline operator M = S y (cubic)
  const double *window;  // [k_size] 1/k^2
  const double *r;
  const double *rfac;    // [r_size]
  int l_major;           // 0: out[r][l][k] (C), 1: out[l][r][k] (D)
  double *out;
};

__global__ void __launch_bounds__(128) coef_kernel(CoefArgs a) {
  extern __shared__ double sh[];
  double *A = sh, *B = sh + a.k_size, *SA = sh + 2 * a.k_size, *SB = sh + 3 * a.k_size;
  const int il = blockIdx.x / a.r_size, ir = blockIdx.x % a.r_size;
  double *out = a.out + (a.l_major ? ((size_t)il * a.r_size + ir) : ((size_t)ir * a.l_size + il)) * a.k_size;
  const int row = a.row_of_l[il];
  if (row < 0) {
    for (int k = threadIdx.x; k < a.k_size; k += blockDim.x) out[k] = 0.0;
    return;
  }
  const double rs = a.r[ir] * a.jt.inv_step;
  const double *T = a.T1 + (size_t)il * a.q_size;
  for (int i = threadIdx.x; i < a.k_size; i += blockDim.x) {
    double sa = 0, sb = 0, ssa = 0, ssb = 0;
    if (i < a.k_size - 1) {
      double h2 = a.hk[i] * a.hk[i] / 6.0;
      for (int iq = a.qbeg[i]; iq < a.qbeg[i + 1]; ++iq) {
        double g = T[iq];
        if (g == 0.0) continue;
        double c = a.qw[iq] * jl_at(a.jt, row, a.q[iq], rs) * g;
        double wa = a.qa[iq], wb = a.qb[iq];
        sa += c * wa;
        sb += c * wb;
        if (a.cubic) {
          ssa += c * (wa * wa * wa - wa) * h2;
          ssb += c * (wb * wb * wb - wb) * h2;
        }
      }
    }
    A[i] = sa;
    B[i] = sb;
    SA[i] = ssa;
    SB[i] = ssb;
  }
  __syncthreads();
  const double rf = a.rfac[ir];
  for (int j = threadIdx.x; j < a.k_size; j += blockDim.x) {
    double v = A[j] + (j > 0 ? B[j - 1] : 0.0);
    if (a.cubic)
      for (int i = 0; i < a.k_size - 1; ++i) v += SA[i] * a.S[i * a.k_size + j] + SB[i] * a.S[(i + 1) * a.k_size + j];
    out[j] = v * a.window[j] * rf;
  }
}

// ------------------------------------------------------------ k3 integral
struct K3Args {
  JTab jt;
  int l_size, r_size, n_pairs, M3, offset_L3;
  double coef;                // c_M3
  const int *l;               // [l_size]
  const int *row_of_L;        // Bessel row of every order up to the table's top
  const int *tt;              // transfer type of (X, l3, M3) at tt[il3 * tt_stride], -1 if none
  int tt_stride;
  const double *r;
  const double *unit_k, *unit_w;  // k and k^2 dk of every transfer k unit
  const long long *unit_off;  // [n_pairs]
  const int *unit_n;
  const double *T2;
  long long n_units;
  double *I3;                 // [l3][r][pair]
};

__global__ void __launch_bounds__(BI_THREADS) k3_kernel(K3Args a) {
  // one thread per (l3, pair, r), r fastest
  const unsigned t = blockIdx.x * BI_THREADS + threadIdx.x;
  if (t >= (unsigned)(a.l_size * a.n_pairs * a.r_size)) return;
  const int ir = (int)(t % (unsigned)a.r_size);
  const unsigned w = t / (unsigned)a.r_size;
  const int il3 = (int)(w / (unsigned)a.n_pairs), p = (int)(w % (unsigned)a.n_pairs);
  const int l3 = a.l[il3];
  const int L3 = abs(l3 - a.M3) + a.offset_L3;
  double *out = a.I3 + ((size_t)il3 * a.r_size + ir) * a.n_pairs + p;
  const int tt = a.tt[il3 * a.tt_stride];
  if (a.M3 > l3 || L3 > l3 + a.M3 || tt < 0) {
    *out = 0.0;
    return;
  }
  const int row = a.row_of_L[L3];
  const long long u0 = a.unit_off[p];
  const int n = a.unit_n[p];
  const double *T = a.T2 + (size_t)tt * a.n_units + u0;
  const double *kk = a.unit_k + u0, *wk = a.unit_w + u0;
  const double rs = a.r[ir] * a.jt.inv_step;
  double s = 0.0;
  for (int i = 0; i < n; ++i) {
    double f = __ldg(&T[i]);
    if (f == 0.0) continue;
    double j = jl_at(a.jt, row, __ldg(&kk[i]), rs);
    s = fma(__ldg(&wk[i]) * f, j, s);
  }
  double v = 0.5 * s;
  if (a.M3 != 0) v *= a.coef;
  *out = v * 2.0;
}

// ------------------------------------------------------------ k2 integral
// Double-float arithmetic on the FP32 pipe (GB300's FP64 pipe is 64 times
// narrower): a value is hi + lo with |lo| <= ulp(hi)/2; the product of two is
// formed without error in its leading part (fmaf) and added to the running sum
// by Knuth's two-sum, so a dot product keeps about 46 bits.
__device__ __forceinline__ float2 df_split(double x) {
  const float h = __double2float_rn(x);
  return make_float2(h, __double2float_rn(x - (double)h));
}

__device__ __forceinline__ void df_fma(float2 d, float2 g, float &hi, float &lo) {
  const float p = d.x * g.x;
  float e = fmaf(d.x, g.x, -p);
  e = fmaf(d.x, g.y, e);
  e = fmaf(d.y, g.x, e);
  const float s = hi + p;
  const float v = s - hi;
  lo += ((hi - (s - v)) + (p - v)) + e;
  hi = s;
}

struct K2Args {
  int l_size, r_size, k_size, n_pairs, M3;
  const int *l;
  const double *k;
  const double *I3;  // [l3][r][pair]
  const float2 *C;   // [r][l2][k] as double-float, each (r, l2) row scaled by 2^-Ce
  const int *Ce;     // [r][l2]
  double *I2;        // [l3][l2][r][k1]
};

__global__ void __launch_bounds__(BI_THREADS) k2_kernel(K2Args a) {
  extern __shared__ double F[];  // [k1][k] doubles, then the same as double-float
  __shared__ int fe[BI_MAX_K];
  const int il3 = blockIdx.x / a.r_size, ir = blockIdx.x % a.r_size;
  const int K = a.k_size;
  if (a.M3 > a.l[il3]) {
    for (int i = threadIdx.x; i < a.l_size * K; i += blockDim.x) {
      int il2 = i / K, k1 = i % K;
      a.I2[(((size_t)il3 * a.l_size + il2) * a.r_size + ir) * K + k1] = 0.0;
    }
    return;
  }
  float2 *F2 = (float2 *)(F + K * K);
  const double *I = a.I3 + ((size_t)il3 * a.r_size + ir) * a.n_pairs;
  for (int i = threadIdx.x; i < K * K; i += blockDim.x) {
    int k1 = i / K, k2 = i % K;
    double v;
    if (k1 > k2) {
      v = I[k1 * (k1 + 1) / 2 + k2];
    } else {
      // T(k2, k1, k3) = (-1)^m T(k1, k2, k3) with the rescaling (k1/k2)^m
      // (bispectra2.c:1476-1500)
      double f = 1.0, x = -a.k[k1] / a.k[k2];
      for (int m = 0; m < a.M3; ++m) f *= x;
      v = I[k2 * (k2 + 1) / 2 + k1] * f;
    }
    F[i] = v;
  }
  __syncthreads();
  // each k1 row scaled to a largest magnitude in [0.5, 1), split into double-float
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int k1 = warp; k1 < K; k1 += BI_WARPS) {
    double m = 0.0;
    for (int j = lane; j < K; j += 32) m = fmax(m, fabs(F[k1 * K + j]));
    for (int w = 16; w; w >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, w));
    int e = 0;
    if (m > 0.0) frexp(m, &e);
    if (lane == 0) fe[k1] = e;
    for (int j = lane; j < K; j += 32) F2[k1 * K + j] = df_split(ldexp(F[k1 * K + j], -e));
  }
  __syncthreads();
  for (int i = threadIdx.x; i < a.l_size * K; i += blockDim.x) {
    int il2 = i / K, k1 = i % K;
    const size_t row = (size_t)ir * a.l_size + il2;
    const float2 *c = a.C + row * K;
    const float2 *f = F2 + k1 * K;
    float hi = 0.f, lo = 0.f;
    for (int j = 0; j < K; ++j) df_fma(__ldg(&c[j]), f[j], hi, lo);
    a.I2[(((size_t)il3 * a.l_size + il2) * a.r_size + ir) * K + k1] =
        ldexp((double)hi + (double)lo, __ldg(&a.Ce[row]) + fe[k1]);
  }
}

// ------------------------------------------------------------ k1 and r integrals, geometry
// One block per (l3, l2) for one (X, M3, offset_L3, Y): the k2 integrals of the
// pair over (r, k) staged in shared memory once, then, warp by warp, every
// (offset_L1, l1) of the triangle with both D tables of its Z fields.
constexpr int BI_MAX_Z = 3;
struct K1Args {
  int l_size, r_size, k_size, M3, offset_L3, parity, m_max, bf;
  int g2;                        // l2 values per block
  const double *geo;             // [o][packed triangle entry]: geometrical factor of (M3, L3, L1 offset 2o)
  long long n_tri;
  const int *l;
  const int *tri_min, *tri_max;  // [l_size][l_size] index range of the third multipole
  const long long *tri_off;      // [l_size][l_size] offset in the packed triangle arrays
  const double *I2;              // [l3][l2][r][k]
  const float2 *D[BI_MAX_Z];     // per Z: offset_L1 slabs [o][l1][r][k] as double-float (hi, lo), o = offset_L1 / 2
  const int *De[BI_MAX_Z];       // per Z: [o][l1] power-of-two exponent of each scaled row
  const double *lf;              // ln n!
  double *U[BI_MAX_Z];           // per Z: unsymmetrised bispectrum of (X, Y, Z), packed
};

// bispectra2_intrinsic_geometrical_factors (bispectra2.c:2456-2880): the
// factor of one (l3, l2, l1) and (M3, L3, L1); it does not depend on Z
__device__ __noinline__ double geometry_factor(int M3, int offset_L3, int parity, const double *__restrict__ lf,
                                               int l3, int l2, int l1, int L3, int L1) {
  const bool even = parity == 0;
  double f_l3L3 = w3j(L3, M3, l3, 0, -M3, M3, lf);
  double summed = f_l3L3;
  if (M3 != 0) summed = even ? f_l3L3 + ((offset_L3 & 1) ? -f_l3L3 : f_l3L3)
                              : f_l3L3 - ((offset_L3 & 1) ? -f_l3L3 : f_l3L3);
  double f_l1l2l3 = w3j000(l1, l2, l3, lf);
  double f_L1l2L3 = w3j000(L1, l2, L3, lf);
  double f_l1L1M3 = w3j000(L1, l1, M3, lf);
  double f_6j = w6j(L1, L3, l2, l3, l1, M3, lf);
  bool even_conf = ((l1 + l2 + l3) % 2 == 0);
  double prefactor = even ? 8.0 / (BI_PI * BI_PI * BI_PI) * (2 * L1 + 1.) * (2 * L3 + 1.)
                          : -0.5 / (4 * BI_PI * BI_PI * BI_PI * BI_PI) * (2 * L1 + 1.) * (2 * L3 + 1.) *
                                (2 * l1 + 1) * (2 * l2 + 1);
  double geometry = summed * f_l1L1M3 * f_L1l2L3 * f_6j;
  if (even && even_conf) geometry /= f_l1l2l3;
  int exponent = even ? l3 + L3 - l1 - L1 : l3 + L3 - l1 - L1 - 1;
  double sign = ((exponent / 2) % 2 == 0) ? 1.0 : -1.0;
  return sign * prefactor * geometry;
}

// The geometrical factor of every packed (l3, l2, l1) triangle entry and even
// offset of L1, for one (M3, offset_L3): one thread per value.
struct GeoArgs {
  int l_size, M3, offset_L3, parity, m_max, n_off;
  long long n_tri;
  const int *l;
  const int *ta, *tb, *tc;  // [n_tri] index of l3, l2, l1 of each entry
  const double *lf;
  double *geo;              // [n_off][n_tri]
};

__global__ void geo_kernel(GeoArgs a) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= a.n_tri * a.n_off) return;
  const int o = (int)(t / a.n_tri);
  const long long e = t % a.n_tri;
  const int l3 = a.l[a.ta[e]], l2 = a.l[a.tb[e]], l1 = a.l[a.tc[e]], M3 = a.M3;
  const int L3 = abs(l3 - M3) + a.offset_L3, L1 = abs(l1 - M3) + 2 * o;
  double v = 0.0;
  if (M3 <= l3 && L3 <= l3 + M3 && L1 <= l1 + M3 && triangle(L1, l2, L3))
    v = (a.parity == 0 && a.m_max == 0) ? 8.0 / (BI_PI * BI_PI * BI_PI)
                                        : geometry_factor(M3, a.offset_L3, a.parity, a.lf, l3, l2, l1, L3, L1);
  a.geo[t] = v;
}

constexpr int BI_MAX_G2 = 2;  // l2 values per block sharing the D loads

__global__ void __launch_bounds__(BI_THREADS, 2) k1r_kernel(K1Args a) {
  extern __shared__ float2 G2[];  // [g][r][k], each (l3, l2) row scaled by 2^-e
  __shared__ double red[BI_WARPS];
  __shared__ int ge[BI_MAX_G2];
  const int n_grp = (a.l_size + a.g2 - 1) / a.g2;
  const int il3 = blockIdx.x / n_grp, il2_0 = (blockIdx.x % n_grp) * a.g2;
  const int l3 = a.l[il3], M3 = a.M3;
  if (M3 > l3) return;
  const int L3 = abs(l3 - M3) + a.offset_L3;
  if (L3 > l3 + M3) return;
  const int ng = min(a.g2, a.l_size - il2_0);
  const int RK = a.r_size * a.k_size;
  int t0[BI_MAX_G2], t1[BI_MAX_G2], l2v[BI_MAX_G2], lo = a.l_size, hi = -1;
#pragma unroll
  for (int g = 0; g < BI_MAX_G2; ++g) {
    t0[g] = 0;
    t1[g] = -1;
    l2v[g] = 0;
    if (g < ng) {
      t0[g] = a.tri_min[il3 * a.l_size + il2_0 + g];
      t1[g] = a.tri_max[il3 * a.l_size + il2_0 + g];
      l2v[g] = a.l[il2_0 + g];
      if (t1[g] >= t0[g]) {
        lo = min(lo, t0[g]);
        hi = max(hi, t1[g]);
      }
    }
  }
  if (hi < lo) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // stage the k2 integrals, each row scaled to a largest magnitude in [0.5, 1)
  for (int g = 0; g < ng; ++g) {
    const double *src = a.I2 + ((size_t)il3 * a.l_size + il2_0 + g) * RK;
    double m = 0.0;
    for (int i = threadIdx.x; i < RK; i += blockDim.x) m = fmax(m, fabs(src[i]));
    for (int w = 16; w; w >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, w));
    if (lane == 0) red[warp] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
      double mm = 0.0;
      for (int w = 0; w < BI_WARPS; ++w) mm = fmax(mm, red[w]);
      int e = 0;
      if (mm > 0.0) frexp(mm, &e);
      ge[g] = e;
    }
    __syncthreads();
    const int e = ge[g];
    for (int i = threadIdx.x; i < RK; i += blockDim.x) G2[g * RK + i] = df_split(ldexp(src[i], -e));
    __syncthreads();
  }
  const int n_off = M3 + 1;  // even offsets 0, 2, ..., 2 M3
  const size_t slab = (size_t)a.l_size * RK;
  const bool m0 = a.parity == 0 && a.m_max == 0;
  // one warp per l1: its offsets of L1 in turn, so that each output has one writer
  for (int il1 = lo + warp; il1 <= hi; il1 += BI_WARPS) {
    const int l1 = a.l[il1];
    double acc[BI_MAX_Z][BI_MAX_G2];
#pragma unroll
    for (int z = 0; z < BI_MAX_Z; ++z)
#pragma unroll
      for (int g = 0; g < BI_MAX_G2; ++g) acc[z][g] = 0.0;
    for (int o = 0; o < n_off; ++o) {
      const int L1 = abs(l1 - M3) + 2 * o;
      if (L1 > l1 + M3) continue;
      bool on[BI_MAX_G2];
      bool any = false;
#pragma unroll
      for (int g = 0; g < BI_MAX_G2; ++g) {
        on[g] = g < ng && il1 >= t0[g] && il1 <= t1[g] && triangle(L1, l2v[g], L3);
        any = any || on[g];
      }
      if (!any) continue;
      float sh[BI_MAX_Z][BI_MAX_G2], sl[BI_MAX_Z][BI_MAX_G2];
#pragma unroll
      for (int z = 0; z < BI_MAX_Z; ++z)
#pragma unroll
        for (int g = 0; g < BI_MAX_G2; ++g) sh[z][g] = sl[z][g] = 0.0f;
      const size_t off = o * slab + (size_t)il1 * RK;
#pragma unroll 2
      for (int i = lane; i < RK; i += 32) {
        float2 d[BI_MAX_Z];
#pragma unroll
        for (int z = 0; z < BI_MAX_Z; ++z) d[z] = (z < a.bf) ? __ldg(&a.D[z][off + i]) : make_float2(0.f, 0.f);
#pragma unroll
        for (int g = 0; g < BI_MAX_G2; ++g)
          if (on[g]) {
            const float2 gi = G2[g * RK + i];
#pragma unroll
            for (int z = 0; z < BI_MAX_Z; ++z)
              if (z < a.bf) df_fma(d[z], gi, sh[z][g], sl[z][g]);
          }
      }
      double s[BI_MAX_Z][BI_MAX_G2];
#pragma unroll
      for (int z = 0; z < BI_MAX_Z; ++z)
#pragma unroll
        for (int g = 0; g < BI_MAX_G2; ++g) {
          double v = (double)sh[z][g] + (double)sl[z][g];
#pragma unroll
          for (int w = 16; w; w >>= 1) v += __shfl_xor_sync(0xffffffffu, v, w);
          s[z][g] = v;
        }
      if (lane == 0) {
#pragma unroll
        for (int g = 0; g < BI_MAX_G2; ++g)
          if (on[g]) {
            const double f =
                a.geo[o * a.n_tri + a.tri_off[il3 * a.l_size + il2_0 + g] + (il1 - t0[g])];
#pragma unroll
            for (int z = 0; z < BI_MAX_Z; ++z)
              if (z < a.bf) acc[z][g] += f * ldexp(s[z][g], a.De[z][o * a.l_size + il1] + ge[g]);
          }
      }
    }
    if (lane == 0) {
#pragma unroll
      for (int g = 0; g < BI_MAX_G2; ++g)
        if (g < ng && il1 >= t0[g] && il1 <= t1[g]) {
          const long long base = a.tri_off[il3 * a.l_size + il2_0 + g] + (il1 - t0[g]);
#pragma unroll
          for (int z = 0; z < BI_MAX_Z; ++z)
            if (z < a.bf) {
              double *dst = a.U[z] + base;
              *dst = m0 ? acc[z][g] : *dst + acc[z][g];
            }
        }
    }
  }
}

// D rows (l1 of one (Z, offset) slab) scaled to a largest magnitude in
// [0.5, 1) and split into double-float; one block per row.
__global__ void split_rows_kernel(const double *__restrict__ D, int rows, int RK, float2 *__restrict__ D2,
                                  int *__restrict__ De) {
  __shared__ double red[BI_WARPS];
  __shared__ int e_s;
  const int row = blockIdx.x;
  if (row >= rows) return;
  const double *src = D + (size_t)row * RK;
  double m = 0.0;
  for (int i = threadIdx.x; i < RK; i += blockDim.x) m = fmax(m, fabs(src[i]));
  for (int w = 16; w; w >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, w));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double mm = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) mm = fmax(mm, red[w]);
    int e = 0;
    if (mm > 0.0) frexp(mm, &e);
    e_s = e;
    De[row] = e;
  }
  __syncthreads();
  const int e = e_s;
  for (int i = threadIdx.x; i < RK; i += blockDim.x) D2[(size_t)row * RK + i] = df_split(ldexp(src[i], -e));
}

// ------------------------------------------------------------ symmetrisation
struct SymArgs {
  int bf, l_size;
  long long n_conf, n_tri;
  const int *c1, *c2, *c3;
  const int *tri_min;
  const long long *tri_off;
  const double *U;
  double *out;
};

__device__ __forceinline__ double u_at(const SymArgs &a, int X, int Y, int Z, int i, int j, int k) {
  size_t base = ((size_t)(X * a.bf + Y) * a.bf + Z) * a.n_tri;
  int t = i * a.l_size + j;
  return a.U[base + a.tri_off[t] + (k - a.tri_min[t])];
}

__global__ void sym_kernel(SymArgs a) {
  long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long n = (long long)a.bf * a.bf * a.bf * a.n_conf;
  if (idx >= n) return;
  long long c = idx % a.n_conf;
  int xyz = (int)(idx / a.n_conf);
  int Z = xyz % a.bf, Y = (xyz / a.bf) % a.bf, X = xyz / (a.bf * a.bf);
  int i1 = a.c1[c], i2 = a.c2[c], i3 = a.c3[c];
  a.out[idx] = u_at(a, X, Y, Z, i1, i2, i3) + u_at(a, Y, X, Z, i2, i1, i3) + u_at(a, Z, Y, X, i3, i2, i1);
}

}  // namespace

// ------------------------------------------------------------ host

// triangle index range of the third multipole for (index_a, index_b): the
// first l >= |la - lb| and the last l <= la + lb
static void tri_range(const int *l, int n, int ia, int ib, int *lo, int *hi) {
  int a = l[ia], b = l[ib];
  int mn = std::abs(a - b), mx = a + b;
  int i = 0;
  while (i < n && l[i] < mn) ++i;
  int j = n - 1;
  while (j >= 0 && l[j] > mx) --j;
  *lo = i;
  *hi = j;
}

extern "C" int64_t song2_bispectra_configs(int l_size, const int *l, int *i1, int *i2, int *i3) {
  int64_t n = 0;
  for (int a = 0; a < l_size; ++a)
    for (int b = 0; b <= a; ++b) {
      int lo, hi;
      tri_range(l, l_size, a, b, &lo, &hi);
      hi = std::min(hi, b);
      for (int c = lo; c <= hi; ++c) {
        if (i1) i1[n] = a;
        if (i2) i2[n] = b;
        if (i3) i3[n] = c;
        ++n;
      }
    }
  return n;
}

// cubic spline second derivatives with the end derivatives of the parabolas
// through the first and last three points (CLASS's estimated derivative)
static void spline_est(const double *x, const double *y, int n, double *y2) {
  std::vector<double> u(n);
  double dy = ((x[2] - x[0]) * (x[2] - x[0]) * (y[1] - y[0]) - (x[1] - x[0]) * (x[1] - x[0]) * (y[2] - y[0])) /
              ((x[2] - x[0]) * (x[1] - x[0]) * (x[2] - x[1]));
  y2[0] = -0.5;
  u[0] = (3. / (x[1] - x[0])) * ((y[1] - y[0]) / (x[1] - x[0]) - dy);
  for (int i = 1; i < n - 1; ++i) {
    double sig = (x[i] - x[i - 1]) / (x[i + 1] - x[i - 1]);
    double p = sig * y2[i - 1] + 2.0;
    y2[i] = (sig - 1.0) / p;
    u[i] = (y[i + 1] - y[i]) / (x[i + 1] - x[i]) - (y[i] - y[i - 1]) / (x[i] - x[i - 1]);
    u[i] = (6.0 * u[i] / (x[i + 1] - x[i - 1]) - sig * u[i - 1]) / p;
  }
  double a = x[n - 3], b = x[n - 2], c = x[n - 1];
  double dyn = ((a - c) * (a - c) * (y[n - 2] - y[n - 1]) - (b - c) * (b - c) * (y[n - 3] - y[n - 1])) /
               ((a - c) * (b - c) * (a - b));
  double qn = 0.5, un = (3. / (c - b)) * (dyn - (y[n - 1] - y[n - 2]) / (c - b));
  y2[n - 1] = (un - qn * u[n - 2]) / (qn * y2[n - 2] + 1.0);
  for (int k = n - 2; k >= 0; --k) y2[k] = y2[k] * y2[k + 1] + u[k];
}

// trapezoidal measure: x[1]-x[0], x[i+1]-x[i-1], x[n-1]-x[n-2]
static void trapezoid(const double *x, int n, double *d) {
  if (n == 1) {
    d[0] = 0.0;
    return;
  }
  d[0] = x[1] - x[0];
  for (int i = 1; i < n - 1; ++i) d[i] = x[i + 1] - x[i - 1];
  d[n - 1] = x[n - 1] - x[n - 2];
}

struct song2_bispectra {
  song2_los *los = nullptr;
  S2LosView v{};
  int bf = 0, bfs[3] = {0, 0, 0}, parity = 0, m_max = 0, m_size = 0, g2 = 1;
  std::vector<int> m;
  int l_size = 0, r_size = 0, k_size = 0, q_size = 0;
  long long n_tri = 0, n_conf = 0;
  std::vector<int> tri_min, tri_max;
  std::vector<long long> tri_off;
  std::vector<int> tt;  // [bf][l_size][m_size]
  std::vector<double> k;
  std::vector<void *> allocs;
  // device
  JTab jt{};
  const int *d_l = nullptr, *d_row_of_L = nullptr, *d_tri_min = nullptr, *d_tri_max = nullptr;
  const int *d_unit_n = nullptr, *d_c1 = nullptr, *d_c2 = nullptr, *d_c3 = nullptr, *d_tt = nullptr;
  const int *d_ta = nullptr, *d_tb = nullptr, *d_tc = nullptr;
  double *d_geo = nullptr;  // [offset_L1 / 2][packed triangle entry]
  const long long *d_tri_off = nullptr, *d_unit_off = nullptr;
  const double *d_r = nullptr, *d_k = nullptr, *d_unit_w = nullptr, *d_lf = nullptr;
  double *d_C = nullptr;  // [bf][r][l][k]
  double *d_D = nullptr;  // [bf][(im, offset_L1/2)][l][r][k]
  float2 *d_D2 = nullptr; // the same, scaled per row, as double-float
  float2 *d_C2 = nullptr; // C scaled per (Y, r, l2) row, as double-float
  int *d_Ce = nullptr;
  int *d_De = nullptr;    // [bf][(im, offset_L1/2)][l]: the rows' exponents
  std::vector<long long> d_slot;  // D slot of (im, offset_L1) pairs: index im * (m_max + 1) + offset_L1 / 2
  long long n_dslots = 0;
  double *d_I3 = nullptr, *d_I2 = nullptr, *d_U = nullptr;
  int *d_status = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  float last_ms = 0.f;
};

template <class T>
static int bup(song2_bispectra *h, const std::vector<T> &v, const T **out, char *err) {
  void *p = nullptr;
  CKB(cudaMalloc(&p, std::max<size_t>(1, v.size()) * sizeof(T)));
  h->allocs.push_back(p);
  if (!v.empty()) CKB(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  *out = (const T *)p;
  return 0;
}

static int balloc(song2_bispectra *h, size_t bytes, void **out, char *err) {
  CKB(cudaMalloc(out, std::max<size_t>(1, bytes)));
  h->allocs.push_back(*out);
  return 0;
}

extern "C" void song2_bispectra_destroy(song2_bispectra *h) {
  if (!h) return;
  for (void *p : h->allocs) cudaFree(p);
  if (h->e0) cudaEventDestroy(h->e0);
  if (h->e1) cudaEventDestroy(h->e1);
  delete h;
}

extern "C" int song2_bispectra_create(song2_los *los, const song2_bispectra_spec *bs, song2_bispectra **out,
                                      char *err) {
  *out = nullptr;
  if (!los || !bs || bs->bf_size < 1 || bs->bf_size > 3 || !bs->bf || bs->r_size < 2 || !bs->r || bs->q_size < 2 ||
      !bs->q || !bs->pk || !bs->transfer1) {
    snprintf(err, SONG2_ERRLEN, "bispectrum spec needs 1-3 fields, an r grid, a q grid, P(q) and the first-order "
                                "transfers");
    return 1;
  }
  song2_bispectra *h = new song2_bispectra();
  auto fail = [&](void) {
    song2_bispectra_destroy(h);
    return 1;
  };
  h->los = los;
  if (s2los_view(los, &h->v, err)) return fail();
  const S2LosView &v = h->v;
  const song2_spec &s = *v.spec;
  const int has[3] = {s.has_source_T, s.has_source_E, s.has_source_B};
  h->bf = bs->bf_size;
  for (int i = 0; i < h->bf; ++i) {
    int f = bs->bf[i];
    if (f < 0 || f > 2 || !has[f]) {
      snprintf(err, SONG2_ERRLEN, "bispectrum field %d has no second-order transfer functions", f);
      return fail();
    }
    for (int j = 0; j < i; ++j)
      if (bs->bf[j] == f) {
        snprintf(err, SONG2_ERRLEN, "bispectrum fields must be distinct");
        return fail();
      }
    h->bfs[i] = f;
  }
  // one parity for every combination: that of the last one (bispectra2.c:967)
  h->parity = (3 * field_parity(h->bfs[h->bf - 1])) % 2;
  h->l_size = v.l_size;
  h->r_size = bs->r_size;
  h->q_size = bs->q_size;
  h->k_size = s.k_size;
  h->k.assign(s.k, s.k + s.k_size);
  h->m.assign(s.m, s.m + s.m_size);
  h->m_size = s.m_size;
  for (int x : h->m) h->m_max = std::max(h->m_max, x);
  const int L = h->l_size, R = h->r_size, K = h->k_size, Q = h->q_size;
  const bool k1c = bs->k1_interpolation == SONG2_INTERP_CUBIC, k2c = bs->k2_interpolation == SONG2_INTERP_CUBIC;
  if (K < 2 || ((k1c || k2c) && K < 3) || K > BI_MAX_K) {
    snprintf(err, SONG2_ERRLEN, "bispectrum needs 2 (3 for cubic) to %d k values, got %d", BI_MAX_K, K);
    return fail();
  }
  for (int i = 0; i < R; ++i)
    if (!(bs->r[i] > 0) || (i && bs->r[i] <= bs->r[i - 1])) {
      snprintf(err, SONG2_ERRLEN, "r grid must be positive and ascending");
      return fail();
    }
  for (int i = 0; i < Q; ++i)
    if (!(bs->q[i] > 0) || (i && bs->q[i] <= bs->q[i - 1])) {
      snprintf(err, SONG2_ERRLEN, "q grid must be positive and ascending");
      return fail();
    }
  if (bs->q[Q - 1] > h->k[K - 1]) {
    snprintf(err, SONG2_ERRLEN, "q=%g beyond the largest k=%g of the sources (bispectra2.c:1534-1536)", bs->q[Q - 1],
             h->k[K - 1]);
    return fail();
  }
  // every x = k r inside the Bessel table
  {
    double kmax = bs->q[Q - 1];
    for (long long u = 0; u < v.n_units; ++u) kmax = std::max(kmax, v.unit_k[u]);
    double xm = kmax * bs->r[R - 1];
    if ((int)(xm / v.x_step) + 2 > v.x_size - 1) {
      snprintf(err, SONG2_ERRLEN, "x_max=%g does not cover k r = %g; increase x_max", v.x_max, xm);
      return fail();
    }
  }
  if ((double)h->l_size * v.n_pairs * R >= 2147483647.0) {
    snprintf(err, SONG2_ERRLEN, "l_size * pairs * r_size too large for one k3 launch");
    return fail();
  }
  // Bessel rows of every order needed: l (first-order convolution) and
  // |l - M3| .. l + M3 (the extended list holds them)
  std::vector<int> row_of(v.l1[v.n_l1 - 1] + 1, -1);
  for (int i = 0; i < v.n_l1; ++i) row_of[v.l1[i]] = i;
  for (int i = 0; i < L; ++i)
    for (int d = -h->m_max; d <= h->m_max; ++d) {
      int o = v.l[i] + d;
      if (o < 0) continue;
      if (o >= (int)row_of.size() || row_of[o] < 0) {
        snprintf(err, SONG2_ERRLEN, "Bessel order %d missing from the line-of-sight table", o);
        return fail();
      }
    }
  // transfer types
  {
    std::vector<int> ty(v.n_tt), tl(v.n_tt), tm(v.n_tt);
    song2_transfer_types(v.spec, v.los, ty.data(), tl.data(), tm.data());
    h->tt.assign((size_t)h->bf * L * h->m_size, -1);
    for (int o = 0; o < v.n_tt; ++o)
      for (int b = 0; b < h->bf; ++b)
        if (ty[o] == h->bfs[b]) {
          int il = (int)(std::lower_bound(v.l, v.l + L, tl[o]) - v.l);
          int im = 0;
          while (h->m[im] != tm[o]) ++im;
          h->tt[((size_t)b * L + il) * h->m_size + im] = o;
        }
  }
  // triangles and configurations
  h->tri_min.resize((size_t)L * L);
  h->tri_max.resize((size_t)L * L);
  h->tri_off.resize((size_t)L * L);
  for (int a = 0; a < L; ++a)
    for (int b = 0; b < L; ++b) {
      int t = a * L + b;
      tri_range(v.l, L, a, b, &h->tri_min[t], &h->tri_max[t]);
      h->tri_off[t] = h->n_tri;
      h->n_tri += std::max(0, h->tri_max[t] - h->tri_min[t] + 1);
    }
  std::vector<int> ta(h->n_tri), tb(h->n_tri), tc(h->n_tri);
  for (int a = 0; a < L; ++a)
    for (int b = 0; b < L; ++b) {
      int t = a * L + b;
      for (int c = h->tri_min[t]; c <= h->tri_max[t]; ++c) {
        long long e = h->tri_off[t] + (c - h->tri_min[t]);
        ta[e] = a;
        tb[e] = b;
        tc[e] = c;
      }
    }
  h->n_conf = song2_bispectra_configs(L, v.l, nullptr, nullptr, nullptr);
  std::vector<int> c1(h->n_conf), c2(h->n_conf), c3(h->n_conf);
  song2_bispectra_configs(L, v.l, c1.data(), c2.data(), c3.data());
  // ln n!
  int lf_n = 4 * (v.l1[v.n_l1 - 1] + h->m_max) + 16;
  std::vector<double> lf(lf_n);
  for (int i = 0; i < lf_n; ++i) lf[i] = (double)lgammal((long double)i + 1.0L);
  // grids and weights
  std::vector<double> r(bs->r, bs->r + R), dr(R), rfac(R), q(bs->q, bs->q + Q), dq(Q), window(K);
  trapezoid(r.data(), R, dr.data());
  trapezoid(q.data(), Q, dq.data());
  for (int i = 0; i < R; ++i) rfac[i] = 0.25 * r[i] * r[i] * dr[i];  // the k1 and r trapezoids' 1/2 each
  for (int i = 0; i < K; ++i) window[i] = 1.0 / (h->k[i] * h->k[i]);
  std::vector<double> qw(Q), qa(Q), qb(Q), hk(K - 1);
  std::vector<int> qbeg(K + 1, Q);
  for (int i = 0; i < K - 1; ++i) hk[i] = h->k[i + 1] - h->k[i];
  {
    // the interval search of bispectra2_interpolate_over_k2/k1 (bispectra2.c:1524-1545)
    int ik = 0;
    std::vector<int> qi(Q);
    for (int iq = 0; iq < Q; ++iq) {
      while (ik + 1 < K && h->k[ik + 1] < q[iq]) ++ik;
      if (ik + 1 >= K) {
        snprintf(err, SONG2_ERRLEN, "q=%g beyond the largest k", q[iq]);
        return fail();
      }
      qi[iq] = ik;
      double b = (q[iq] - h->k[ik]) / hk[ik];
      qb[iq] = b;
      qa[iq] = 1. - b;
      qw[iq] = dq[iq] * q[iq] * q[iq] * q[iq] * q[iq] * bs->pk[iq];
    }
    for (int iq = Q - 1; iq >= 0; --iq) qbeg[qi[iq]] = iq;
    for (int i = K - 1; i >= 0; --i) qbeg[i] = std::min(qbeg[i], qbeg[i + 1]);
  }
  // spline operator of the k grid: M = S y
  std::vector<double> S((size_t)K * K, 0.0);
  if (K >= 3) {
    std::vector<double> e(K), col(K);
    for (int j = 0; j < K; ++j) {
      std::fill(e.begin(), e.end(), 0.0);
      e[j] = 1.0;
      spline_est(h->k.data(), e.data(), K, col.data());
      for (int i = 0; i < K; ++i) S[(size_t)i * K + j] = col[i];
    }
  }
  // transfer k grid measures
  std::vector<long long> uoff(v.n_pairs);
  std::vector<int> un(v.n_pairs);
  std::vector<double> udk(v.n_units);
  {
    long long o = 0;
    for (int p = 0; p < v.n_pairs; ++p) {
      uoff[p] = o;
      un[p] = v.unit_size[p];
      if (un[p] < 2) {
        snprintf(err, SONG2_ERRLEN, "integration grid has less than two elements (bispectra2.c:1268-1270)");
        return fail();
      }
      trapezoid(v.unit_k + o, un[p], udk.data() + o);
      for (int i = 0; i < un[p]; ++i) udk[o + i] *= v.unit_k[o + i] * v.unit_k[o + i];  // k^2 dk
      o += un[p];
    }
  }
  std::vector<int> lv(v.l, v.l + L);
  const double *d_q, *d_qw, *d_qa, *d_qb, *d_hk, *d_S, *d_win, *d_rfac, *d_ones, *d_T1;
  const int *d_qbeg;
  std::vector<double> ones(R, 0.5);  // the k2 trapezoid's 1/2
  std::vector<double> T1(bs->transfer1, bs->transfer1 + (size_t)h->bf * L * Q);
  const int *d_jxmin;
  const double *d_jxmin_u;
  std::vector<int> jx(v.jxmin, v.jxmin + v.n_l1);
  std::vector<double> jxu(v.n_l1);
  for (int i = 0; i < v.n_l1; ++i) jxu[i] = s2los_x_of(jx[i], v.x_size, v.x_max) / v.x_step;
  if (bup(h, lv, &h->d_l, err) || bup(h, row_of, &h->d_row_of_L, err) || bup(h, h->tri_min, &h->d_tri_min, err) ||
      bup(h, h->tri_max, &h->d_tri_max, err) || bup(h, h->tri_off, &h->d_tri_off, err) ||
      bup(h, un, &h->d_unit_n, err) || bup(h, uoff, &h->d_unit_off, err) || bup(h, udk, &h->d_unit_w, err) ||
      bup(h, c1, &h->d_c1, err) || bup(h, c2, &h->d_c2, err) || bup(h, c3, &h->d_c3, err) ||
      bup(h, h->tt, &h->d_tt, err) || bup(h, r, &h->d_r, err) || bup(h, h->k, &h->d_k, err) ||
      bup(h, lf, &h->d_lf, err) || bup(h, q, &d_q, err) || bup(h, qw, &d_qw, err) || bup(h, qa, &d_qa, err) ||
      bup(h, qb, &d_qb, err) || bup(h, hk, &d_hk, err) || bup(h, S, &d_S, err) || bup(h, window, &d_win, err) ||
      bup(h, rfac, &d_rfac, err) || bup(h, ones, &d_ones, err) || bup(h, T1, &d_T1, err) ||
      bup(h, qbeg, &d_qbeg, err) || bup(h, jx, &d_jxmin, err) || bup(h, jxu, &d_jxmin_u, err) ||
      bup(h, ta, &h->d_ta, err) || bup(h, tb, &h->d_tb, err) || bup(h, tc, &h->d_tc, err))
    return fail();
  void *tmp;
  if (balloc(h, sizeof(int) * 4, &tmp, err)) return fail();
  h->d_status = (int *)tmp;
  CKB(cudaMemset(h->d_status, 0, sizeof(int) * 4));
  h->jt.tab = v.jtab_dev;
  h->jt.dd = v.ddj_dev;
  h->jt.xmin = d_jxmin;
  h->jt.xmin_u = d_jxmin_u;
  h->jt.x_size = v.x_size;
  h->jt.x_max = v.x_max;
  h->jt.x_step = v.x_step;
  h->jt.inv_step = 1.0 / v.x_step;
  h->jt.cubic = v.los->bessel_interpolation == SONG2_INTERP_CUBIC;
  h->jt.status = h->d_status;
  // coefficient tables
  const size_t slab = (size_t)R * L * K;
  if (balloc(h, sizeof(double) * slab * h->bf, &tmp, err)) return fail();
  h->d_C = (double *)tmp;
  h->n_dslots = 0;
  h->d_slot.assign((size_t)h->m_size * (h->m_max + 1), -1);
  for (int im = 0; im < h->m_size; ++im)
    for (int o = 0; o <= 2 * h->m[im]; o += 2) h->d_slot[(size_t)im * (h->m_max + 1) + o / 2] = h->n_dslots++;
  if (balloc(h, sizeof(double) * slab * h->bf * h->n_dslots, &tmp, err)) return fail();
  h->d_D = (double *)tmp;
  CoefArgs ca{};
  ca.jt = h->jt;
  ca.l_size = L;
  ca.r_size = R;
  ca.k_size = K;
  ca.q_size = Q;
  ca.q = d_q;
  ca.qw = d_qw;
  ca.qa = d_qa;
  ca.qb = d_qb;
  ca.qbeg = d_qbeg;
  ca.hk = d_hk;
  ca.S = d_S;
  ca.window = d_win;
  ca.r = h->d_r;
  size_t csm = sizeof(double) * 4 * K;
  std::vector<int> rows(L);
  const int *d_rows;
  std::vector<const int *> row_tables;
  for (int b = 0; b < h->bf; ++b) {
    for (int i = 0; i < L; ++i) rows[i] = row_of[v.l[i]];
    if (bup(h, rows, &d_rows, err)) return fail();
    ca.row_of_l = d_rows;
    ca.T1 = d_T1 + (size_t)b * L * Q;
    ca.cubic = k2c;
    ca.rfac = d_ones;
    ca.l_major = 0;
    ca.out = h->d_C + (size_t)b * slab;
    coef_kernel<<<L * R, 128, csm>>>(ca);
    CKB(cudaGetLastError());
    for (int im = 0; im < h->m_size; ++im) {
      int M3 = h->m[im];
      for (int o = 0; o <= 2 * M3; o += 2) {
        for (int i = 0; i < L; ++i) {
          int l1 = v.l[i];
          int L1 = std::abs(l1 - M3) + o;
          rows[i] = (M3 > l1 || L1 > l1 + M3) ? -1 : row_of[L1];
        }
        if (bup(h, rows, &d_rows, err)) return fail();
        ca.row_of_l = d_rows;
        ca.cubic = k1c;
        ca.rfac = d_rfac;
        ca.l_major = 1;
        ca.out = h->d_D + ((size_t)b * h->n_dslots + h->d_slot[(size_t)im * (h->m_max + 1) + o / 2]) * slab;
        coef_kernel<<<L * R, 128, csm>>>(ca);
        CKB(cudaGetLastError());
      }
    }
  }
  {
    const int rows = h->bf * (int)h->n_dslots * L;
    if (balloc(h, sizeof(float2) * (size_t)rows * R * K, &tmp, err)) return fail();
    h->d_D2 = (float2 *)tmp;
    if (balloc(h, sizeof(int) * (size_t)rows, &tmp, err)) return fail();
    h->d_De = (int *)tmp;
    split_rows_kernel<<<rows, 256>>>(h->d_D, rows, R * K, h->d_D2, h->d_De);
    CKB(cudaGetLastError());
    const int crows = h->bf * R * L;
    if (balloc(h, sizeof(float2) * (size_t)crows * K, &tmp, err)) return fail();
    h->d_C2 = (float2 *)tmp;
    if (balloc(h, sizeof(int) * (size_t)crows, &tmp, err)) return fail();
    h->d_Ce = (int *)tmp;
    split_rows_kernel<<<crows, 64>>>(h->d_C, crows, K, h->d_C2, h->d_Ce);
    CKB(cudaGetLastError());
  }
  CKB(cudaDeviceSynchronize());
  int st[4];
  CKB(cudaMemcpy(st, h->d_status, sizeof(st), cudaMemcpyDeviceToHost));
  if (st[0]) {
    snprintf(err, SONG2_ERRLEN, "a Bessel argument fell outside the table");
    return fail();
  }
  // scratch
  if (balloc(h, sizeof(double) * (size_t)L * R * v.n_pairs, &tmp, err)) return fail();
  h->d_I3 = (double *)tmp;
  if (balloc(h, sizeof(double) * (size_t)L * L * R * K, &tmp, err)) return fail();
  h->d_I2 = (double *)tmp;
  if (balloc(h, sizeof(double) * (size_t)h->bf * h->bf * h->bf * std::max<long long>(1, h->n_tri), &tmp, err))
    return fail();
  h->d_U = (double *)tmp;
  if (balloc(h, sizeof(double) * (size_t)(h->m_max + 1) * std::max<long long>(1, h->n_tri), &tmp, err))
    return fail();
  h->d_geo = (double *)tmp;
  {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    const size_t need2 = (sizeof(double) + sizeof(float2)) * (size_t)K * K;
    if (need2 > (size_t)optin) {
      snprintf(err, SONG2_ERRLEN, "k_size = %d too large for the k2 integral's shared memory", K);
      return fail();
    }
    CKB(cudaFuncSetAttribute(k2_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)need2));
    size_t need = sizeof(float2) * (size_t)R * K;
    if (need > (size_t)optin) {
      snprintf(err, SONG2_ERRLEN, "r_size * k_size = %d * %d too large for the k1 integral's shared memory", R, K);
      return fail();
    }
    h->g2 = (BI_MAX_G2 * need <= (size_t)optin) ? BI_MAX_G2 : 1;
    CKB(cudaFuncSetAttribute(k1r_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(need * h->g2)));
  }
  cudaEventCreate(&h->e0);
  cudaEventCreate(&h->e1);
  *out = h;
  return 0;
}

extern "C" int64_t song2_bispectra_size(const song2_bispectra *h) {
  return (int64_t)h->bf * h->bf * h->bf * h->n_conf;
}

extern "C" float song2_bispectra_last_ms(const song2_bispectra *h) { return h->last_ms; }

extern "C" int song2_bispectra_run(song2_bispectra *h, const double *transfer2_dev, double *out_dev, void *stream,
                                   char *err) {
  cudaStream_t st = (cudaStream_t)stream;
  const S2LosView &v = h->v;
  const int L = h->l_size, R = h->r_size, K = h->k_size, bf = h->bf;
  const size_t slab = (size_t)R * L * K;
  CKB(cudaEventRecord(h->e0, st));
  CKB(cudaMemsetAsync(h->d_status, 0, sizeof(int) * 4, st));
  CKB(cudaMemsetAsync(h->d_U, 0, sizeof(double) * (size_t)bf * bf * bf * std::max<long long>(1, h->n_tri), st));
  const int even = h->parity == 0;
  for (int X = 0; X < bf; ++X)
    for (int im = 0; im < h->m_size; ++im) {
      const int M3 = h->m[im];
      double fa = 1, f2a = 1;
      for (int c = M3; c > 0; --c) fa *= c;
      for (int c = 2 * M3; c > 0; --c) f2a *= c;
      const double coef = std::pow(2., M3) * fa / std::sqrt(f2a);  // bispectra2.c:1010-1022
      for (int oL3 = 0; oL3 < 2 * M3 + 1; ++oL3) {
        if (even ? (oL3 % 2 != 0) : (oL3 % 2 == 0)) continue;
        K3Args ka{};
        ka.jt = h->jt;
        ka.l_size = L;
        ka.r_size = R;
        ka.n_pairs = v.n_pairs;
        ka.M3 = M3;
        ka.offset_L3 = oL3;
        ka.coef = coef;
        ka.l = h->d_l;
        ka.row_of_L = h->d_row_of_L;
        ka.tt = h->d_tt + (size_t)X * L * h->m_size + im;
        ka.tt_stride = h->m_size;
        ka.r = h->d_r;
        ka.unit_k = v.unit_k_dev;
        ka.unit_w = h->d_unit_w;
        ka.unit_off = h->d_unit_off;
        ka.unit_n = h->d_unit_n;
        ka.T2 = transfer2_dev;
        ka.n_units = v.n_units;
        ka.I3 = h->d_I3;
        GeoArgs ga{};
        ga.l_size = L;
        ga.M3 = M3;
        ga.offset_L3 = oL3;
        ga.parity = h->parity;
        ga.m_max = h->m_max;
        ga.n_off = M3 + 1;
        ga.n_tri = h->n_tri;
        ga.l = h->d_l;
        ga.ta = h->d_ta;
        ga.tb = h->d_tb;
        ga.tc = h->d_tc;
        ga.lf = h->d_lf;
        ga.geo = h->d_geo;
        if (h->n_tri > 0) {
          long long ng = h->n_tri * (M3 + 1);
          geo_kernel<<<(unsigned)((ng + 255) / 256), 256, 0, st>>>(ga);
          CKB(cudaGetLastError());
        }
        long long threads = (long long)L * v.n_pairs * R;
        k3_kernel<<<(unsigned)((threads + BI_THREADS - 1) / BI_THREADS), BI_THREADS, 0, st>>>(ka);
        CKB(cudaGetLastError());
        for (int Y = 0; Y < bf; ++Y) {
          K2Args k2{};
          k2.l_size = L;
          k2.r_size = R;
          k2.k_size = K;
          k2.n_pairs = v.n_pairs;
          k2.M3 = M3;
          k2.l = h->d_l;
          k2.k = h->d_k;
          k2.I3 = h->d_I3;
          k2.C = h->d_C2 + (size_t)Y * slab;
          k2.Ce = h->d_Ce + (size_t)Y * R * L;
          k2.I2 = h->d_I2;
          k2_kernel<<<L * R, BI_THREADS, (sizeof(double) + sizeof(float2)) * K * K, st>>>(k2);
          CKB(cudaGetLastError());
          K1Args k1{};
          k1.l_size = L;
          k1.r_size = R;
          k1.k_size = K;
          k1.M3 = M3;
          k1.offset_L3 = oL3;
          k1.parity = h->parity;
          k1.m_max = h->m_max;
          k1.bf = bf;
          k1.l = h->d_l;
          k1.tri_min = h->d_tri_min;
          k1.tri_max = h->d_tri_max;
          k1.tri_off = h->d_tri_off;
          k1.I2 = h->d_I2;
          for (int Z = 0; Z < bf; ++Z) {
            const size_t sl0 = (size_t)Z * h->n_dslots + h->d_slot[(size_t)im * (h->m_max + 1)];
            k1.D[Z] = h->d_D2 + sl0 * slab;
            k1.De[Z] = h->d_De + sl0 * L;
            k1.U[Z] = h->d_U + ((size_t)(X * bf + Y) * bf + Z) * h->n_tri;
          }
          k1.lf = h->d_lf;
          k1.g2 = h->g2;
          k1.geo = h->d_geo;
          k1.n_tri = h->n_tri;
          k1r_kernel<<<L * ((L + h->g2 - 1) / h->g2), BI_THREADS, sizeof(float2) * R * K * h->g2, st>>>(k1);
          CKB(cudaGetLastError());
        }
      }
    }
  SymArgs sa{};
  sa.bf = bf;
  sa.l_size = L;
  sa.n_conf = h->n_conf;
  sa.n_tri = h->n_tri;
  sa.c1 = h->d_c1;
  sa.c2 = h->d_c2;
  sa.c3 = h->d_c3;
  sa.tri_min = h->d_tri_min;
  sa.tri_off = h->d_tri_off;
  sa.U = h->d_U;
  sa.out = out_dev;
  long long n = (long long)bf * bf * bf * h->n_conf;
  if (n > 0) {
    sym_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(sa);
    CKB(cudaGetLastError());
  }
  CKB(cudaEventRecord(h->e1, st));
  CKB(cudaEventSynchronize(h->e1));
  CKB(cudaEventElapsedTime(&h->last_ms, h->e0, h->e1));
  int stv[4];
  CKB(cudaMemcpy(stv, h->d_status, sizeof(stv), cudaMemcpyDeviceToHost));
  if (stv[0]) {
    snprintf(err, SONG2_ERRLEN, "a Bessel argument fell outside the table");
    return 1;
  }
  return 0;
}

extern "C" int song2_gpu_bispectra(const song2_spec *spec, const song2_los_spec *los, const song2_bispectra_spec *bs,
                                   const double *transfer2_flat, double *out, char *err) {
  song2_los *lh = nullptr;
  if (song2_los_create(spec, los, &lh, err)) return 1;
  song2_bispectra *h = nullptr;
  if (song2_bispectra_create(lh, bs, &h, err)) {
    song2_los_destroy(lh);
    return 1;
  }
  size_t n_in = (size_t)song2_los_transfer_size(lh), n_out = (size_t)song2_bispectra_size(h);
  double *d_in = nullptr, *d_out = nullptr;
  int rc = 0;
  if (cudaMalloc((void **)&d_in, sizeof(double) * std::max<size_t>(1, n_in)) != cudaSuccess ||
      cudaMalloc((void **)&d_out, sizeof(double) * std::max<size_t>(1, n_out)) != cudaSuccess) {
    snprintf(err, SONG2_ERRLEN, "device allocation failed for the transfers and bispectra");
    rc = 1;
  }
  if (!rc && cudaMemcpy(d_in, transfer2_flat, sizeof(double) * n_in, cudaMemcpyHostToDevice) != cudaSuccess) {
    snprintf(err, SONG2_ERRLEN, "upload of the transfers failed");
    rc = 1;
  }
  if (!rc) rc = song2_bispectra_run(h, d_in, d_out, nullptr, err);
  if (!rc && cudaMemcpy(out, d_out, sizeof(double) * n_out, cudaMemcpyDeviceToHost) != cudaSuccess) {
    snprintf(err, SONG2_ERRLEN, "download of the bispectra failed");
    rc = 1;
  }
  cudaFree(d_in);
  cudaFree(d_out);
  song2_bispectra_destroy(h);
  song2_los_destroy(lh);
  return rc;
}

extern "C" void song2_bispectra_add_quadratic(double *b, const double *b_quadratic, int64_t n, int use_delta_tilde) {
  for (int64_t i = 0; i < n; ++i) {
    double bolometric = -3 / 8. * b_quadratic[i];
    double delta_tilde = use_delta_tilde ? +4 / 8. * b_quadratic[i] : 0.0;
    b[i] += bolometric + delta_tilde;
  }
}
