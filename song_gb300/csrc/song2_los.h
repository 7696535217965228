/* song2_los.h - helpers shared by the host (C) and device (CUDA) halves of the
 * line-of-sight integration: the spherical Bessel recurrence and the x grid of
 * the projection functions.
 */
#ifndef SONG2_LOS_H
#define SONG2_LOS_H

#include <math.h>

#include "song2.h"

#ifdef __CUDACC__
#define S2LOS_HD static __host__ __device__ __forceinline__
#else
#define S2LOS_HD static inline
#endif

/* The downward recurrence rescales by a power of two whenever |f| exceeds
   2^800, so that the stored values can be brought to the final scale exactly
   (ldexp) however many rescalings followed them. */
#define S2LOS_SCALE_BITS 800
#define S2LOS_BIG 0x1p800
#define S2LOS_SMALL 0x1p-800
/* CLASS smallest_allowed_variation (the bisection's stop on an empty bracket) */
#define S2LOS_SMALLEST_VARIATION 1e-16

#ifdef __cplusplus
extern "C" {
#endif

/* Start of the downward recurrence: above both lmax and x by a margin that
   keeps the admixture of y_l below double precision. */
S2LOS_HD int s2los_miller_start(double x, int lmax) {
  double m = x > (double)lmax ? x : (double)lmax;
  return (int)(m + 30.0 + 2.0 * sqrt(m)) + 1;
}

/* Normalisation of the recurrence's f_0, f_1 (at the final scale): by j_0 or
   j_1, whichever is larger in magnitude at x (they never vanish together). */
S2LOS_HD double s2los_miller_norm(double x, double f0, double f1) {
  double s = sin(x), c = cos(x);
  double j0 = s / x, j1;
  if (fabs(x) < 0.1) {
    double x2 = x * x;
    j1 = x / 3.0 * (1.0 - x2 / 10.0 * (1.0 - x2 / 28.0 * (1.0 - x2 / 54.0)));
  } else {
    j1 = (s / x - c) / x;
  }
  return (fabs(j0) >= fabs(j1)) ? j0 / f0 : j1 / f1;
}

/* x grid of the projection functions: lin_space(0, x_max, x_size)
   (bessel2_get_xx_list, bessel2.c:960-1000) */
S2LOS_HD double s2los_x_of(int i, int x_size, double x_max) { return 0.0 + (double)i * (x_max - 0.0) / (x_size - 1); }

/* Grid size: x_max / x_step + 1, truncated (bessel2.c:979) */
S2LOS_HD int s2los_x_size(double x_max, double x_step) { return (int)(x_max / x_step + 1); }

/* host helpers of song2_transfer_host.c */
void s2los_bessel_all(double x, int lmax, double *out);
int s2los_bessel_xmin(int l1, const song2_los_spec *los, int x_size, double x_max);
int s2los_index_m_max(const song2_spec *s, int l);

#ifdef __cplusplus
}
#endif

#endif /* SONG2_LOS_H */
