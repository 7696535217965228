// song2_los_view.h - what the bispectrum integrals read from a line-of-sight
// handle: its spec, l list, Bessel table and transfer k grids (host and device
// copies).  Internal to the library.
#pragma once
#include <cstdint>

#include "song2.h"

struct S2LosView {
  const song2_spec *spec;
  const song2_los_spec *los;
  int l_size;
  const int *l;              // host
  // Bessel table j_l1 on the x grid, [n_l1][x_size], zero below each row's x_min
  int x_size;
  double x_max, x_step;
  int n_l1;
  const int *l1;             // host, ascending
  const int *jxmin;          // host, first stored x index of each row (x_size: negligible everywhere)
  const double *jtab_dev;
  const double *ddj_dev;     // natural-spline second derivatives of the rows (cubic Bessel interpolation), or null
  // transfer k grids: pairs (k1 ascending, k2 <= k1) back to back
  int n_pairs;
  int64_t n_units;
  const int *unit_size;      // host, per pair
  const double *unit_k;      // host, per unit
  const double *unit_k_dev;  // device, per unit
  int n_tt;                  // transfer types (flat output: [tt][unit])
};

// Fills the view; with cubic Bessel interpolation builds the j_l1 spline table
// on the first call.  Returns 0, or 1 with a message.
int s2los_view(song2_los *h, S2LosView *v, char *err);
