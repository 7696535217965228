/*
 * song2_oracle.h - CPU restatement of SONG's second-order evolution.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker of the GPU
 * evolver: only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg may load it.  It is never part of the product path.
 *
 * Parity status: the reference (coccoinomane/song) cannot be built here
 * because its CLASS submodule (class.git, branch song_support, commit not
 * recorded) is empty, and it ships no golden vectors, so parity against the
 * reference's own run is unpinned.  The restatement is pinned instead by the
 * reference's built-in self-checks (geometry identities, perturbations2.c:
 * 5864-6065), by its documented limits (quadratic_sources=no reduces SONG to
 * a first-order code, perturbations2.h:270-287) and by golden fixtures
 * generated from this restatement (tests/golden/).
 */
#ifndef SONG2_ORACLE_H
#define SONG2_ORACLE_H
#include "song2.h"
#ifdef __cplusplus
extern "C" {
#endif

/* Second-order run: sources_flat holds tp2_size * song2_sources_per_type()
   doubles in the flat layout of song2.h; stats one entry per triplet in work
   order (k1 descending, k2 <= k1 ascending, k3 ascending).  Returns 0/1. */
int song2_oracle_evolve(const song2_spec *spec, const song2_tables *tab, double *sources_flat,
                        song2_triplet_stats *stats, int nthreads, char *err);

/* Same, restricted to the triplets whose work-order index is in
   [first, first+count): used to time a bounded sample. */
int song2_oracle_evolve_range(const song2_spec *spec, const song2_tables *tab, double *sources_flat,
                              song2_triplet_stats *stats, int64_t first, int64_t count,
                              int nthreads, char *err);

/* Same, for an explicit list of work-order indices (one rank's shard). */
int song2_oracle_evolve_list(const song2_spec *spec, const song2_tables *tab, double *sources_flat,
                             song2_triplet_stats *stats, const int64_t *items, int64_t count, int nthreads,
                             char *err);

/* First-order mode (SONG with quadratic sources off and has_ad_first_order
   initial conditions, perturbations2.c:4096-4185) for every k of spec->k:
   fills fo_out[k][tau][q] on a uniform ln(tau) grid. */
int song2_oracle_first_order(const song2_spec *spec, const song2_tables *bg_only, int fo_l_max,
                             int fo_tau_size, double fo_lntau0, double fo_dlntau, double *fo_out,
                             int nthreads, char *err);

/* Coupling coefficients from Wigner 3j symbols (Racah formula), kind:
   0 c_minus, 1 c_plus, 2 d_minus, 3 d_plus, 4 d_zero. */
double song2_oracle_coupling(int kind, int l, int m1, int m);

/* delta-tilde coupling ppt2->coupling_coefficients of field 0/1/2 = T/E/B at
   (l, m, l1, m1, l2) (perturbations2.c:1380-1490), from the same 3j symbols. */
double song2_oracle_delta_tilde_coupling(int field, int l, int m, int l1, int m1, int l2);

/* Right-hand side of one triplet at (tau, y) for tests, in the vector layout of
   tca = 0 (no approximation), 1 (tight coupling) or 2 (radiation streaming).
   Returns n or -1. */
int song2_oracle_rhs(const song2_spec *spec, const song2_tables *tab, int index_k1, int index_k2,
                     int index_k3, int tca, double tau, const double *y, double *dy, char *err);

/* Geometry self-checks of perturbations2.c:5864-6065 for one triplet;
   returns the number of failed checks (0 = all passed). */
int song2_oracle_geometry_checks(const song2_spec *spec, int index_k1, int index_k2, int index_k3,
                                 double *max_dev);

#ifdef __cplusplus
}
#endif
#endif
