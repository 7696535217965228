/* song2_output.c - self-describing source files: the sources of one (k1,k2)
 * pair as a function of (k3, tau), or of every triplet at one source time, with
 * the grids, the background and the first-order quantities beside them, in the
 * layout of perturb2_output (perturbations2.c:14688-15340) that the reference's
 * python/songy.py reads (Fixedk1k2File, FixedTauFile).
 *
 * File layout: an ASCII header of HEADER_BYTES bytes (NUL padded) whose first
 * line names the file type, followed by the binary blocks back to back.  The
 * header ends with a block map: a line holding "BLOCK", then one line per block
 * beginning with '#', its fields separated by two spaces: the block number, the
 * type (char, int, double), the number of elements, the bytes, the byte offset
 * in the file, a description and a name.  Block 0 is the header itself.
 */
#include <math.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "song2.h"

#define HEADER_BYTES 65536
#define MAX_BLOCKS 512
#define LABEL 40 /* _MAX_LENGTH_LABEL_ */

typedef struct {
  char type[8];
  int64_t count, bytes;
  const void *data;
  char desc[160], name[120];
} block;

typedef struct {
  char text[HEADER_BYTES];
  size_t len;
  int n;
  block b[MAX_BLOCKS];
  int overflow;
} bfile;

static void line(bfile *f, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  int w = vsnprintf(f->text + f->len, HEADER_BYTES - f->len, fmt, ap);
  va_end(ap);
  if (w < 0 || f->len + (size_t)w + 1 >= HEADER_BYTES) {
    f->overflow = 1;
    return;
  }
  f->len += (size_t)w;
  f->text[f->len++] = '\n';
  f->text[f->len] = 0;
}

static void add(bfile *f, const char *type, size_t elsize, int64_t count, const void *data, const char *desc,
                const char *name) {
  if (f->n >= MAX_BLOCKS) {
    f->overflow = 1;
    return;
  }
  block *b = &f->b[f->n++];
  snprintf(b->type, sizeof b->type, "%s", type);
  b->count = count;
  b->bytes = count * (int64_t)elsize;
  b->data = data;
  snprintf(b->desc, sizeof b->desc, "%s", desc);
  snprintf(b->name, sizeof b->name, "%s", name);
}

static int write_file(bfile *f, const char *path, char *err) {
  /* the map: block 0 is the header, then the data blocks from HEADER_BYTES on */
  line(f, "");
  line(f, "BLOCK  TYPE  SIZE  BYTES  START  DESCRIPTION  NAME");
  int64_t off = HEADER_BYTES;
  line(f, "#  0  char  %d  %d  0  this header  header", HEADER_BYTES, HEADER_BYTES);
  for (int i = 0; i < f->n; ++i) {
    line(f, "#  %d  %s  %lld  %lld  %lld  %s  %s", i + 1, f->b[i].type, (long long)f->b[i].count,
         (long long)f->b[i].bytes, (long long)off, f->b[i].desc, f->b[i].name);
    off += f->b[i].bytes;
  }
  line(f, "END OF MAP");
  if (f->overflow) {
    snprintf(err, SONG2_ERRLEN, "header of %.800s exceeds %d bytes", path, HEADER_BYTES);
    return 1;
  }
  FILE *fp = fopen(path, "wb");
  if (!fp) {
    snprintf(err, SONG2_ERRLEN, "cannot open %.900s for writing", path);
    return 1;
  }
  int rc = fwrite(f->text, 1, HEADER_BYTES, fp) != HEADER_BYTES;
  for (int i = 0; i < f->n && !rc; ++i)
    if (f->b[i].bytes && fwrite(f->b[i].data, 1, (size_t)f->b[i].bytes, fp) != (size_t)f->b[i].bytes) rc = 1;
  if (fclose(fp)) rc = 1;
  if (rc) snprintf(err, SONG2_ERRLEN, "short write to %.900s", path);
  return rc;
}

/* ------------------------------------------------------ table look-ups */

static double spl(int n, int ncol, double x0, double dx, const double *y, const double *dd, int col, double x) {
  double u = (x - x0) / dx;
  int i = (int)floor(u);
  if (i < 0) i = 0;
  if (i > n - 2) i = n - 2;
  double b = u - i, a = 1.0 - b;
  const double *y0 = y + (size_t)i * ncol, *y1 = y0 + ncol, *d0 = dd + (size_t)i * ncol, *d1 = d0 + ncol;
  return a * y0[col] + b * y1[col] + ((a * a * a - a) * d0[col] + (b * b * b - b) * d1[col]) * dx * dx / 6.0;
}

static void background(const song2_tables *t, double tau, double *a, double *H) {
  double x = log(tau);
  double lna = spl(t->bg_size, SONG2_BG_SIZE, t->bg_lntau0, t->bg_dlntau, t->bg, t->bg_dd, SONG2_BG_LN_A, x);
  double lnhc = spl(t->bg_size, SONG2_BG_SIZE, t->bg_lntau0, t->bg_dlntau, t->bg, t->bg_dd, SONG2_BG_LN_HC, x);
  *a = exp(lna);
  *H = exp(lnhc - lna); /* cosmic-time Hubble rate (aH)/a, 1/Mpc */
}

/* the scalar first-order quantities of the table (labels for SONG2_FO_PHI..) */
static const char *FO_LABELS[] = {"phi", "psi", "phi_prime", "psi_prime", "phi_prime_prime", "delta_g", "v_g",
                                  "delta_b", "v_b", "delta_b_prime", "v_b_prime", "delta_cdm", "v_cdm",
                                  "v_cdm_prime", "delta_ur", "v_ur", "dipole_b", "dipole_cdm"};
#define N_FO ((int)(sizeof FO_LABELS / sizeof FO_LABELS[0]))

static void first_order(const song2_tables *t, int index_k, double tau, double *out) {
  const double *fo = t->fo + (size_t)index_k * t->fo_tau_size * t->fo_size;
  const double *dd = t->fo_dd + (size_t)index_k * t->fo_tau_size * t->fo_size;
  for (int q = 0; q < N_FO; ++q)
    out[q] = spl(t->fo_tau_size, t->fo_size, t->fo_lntau0, t->fo_dlntau, fo, dd, q, log(tau));
}

/* source-type labels in the reference's form (T_l_m, E_l_m, B_l_m, delta_cdm;
   perturbations2.c:12416-12780) */
static char *labels(const song2_spec *s, int *n_out) {
  int n = song2_tp2_size(s);
  char *lab = (char *)calloc((size_t)n * LABEL, 1);
  int i = 0;
  const char *kind[3] = {"T", "E", "B"};
  int has[3] = {s->has_source_T, s->has_source_E, s->has_source_B};
  int lmax[3] = {s->l_max_los_t, s->l_max_los_p, s->l_max_los_p};
  for (int t = 0; t < 3; ++t) {
    if (!has[t]) continue;
    for (int l = 0; l <= lmax[t]; ++l)
      for (int im = 0; im < s->m_size; ++im)
        if (s->m[im] <= l) snprintf(lab + (size_t)(i++) * LABEL, LABEL, "%s_%d_%d", kind[t], l, s->m[im]);
  }
  if (s->has_source_delta_cdm) snprintf(lab + (size_t)(i++) * LABEL, LABEL, "delta_cdm");
  *n_out = n;
  return lab;
}

static void common_header(bfile *f, const song2_spec *s, const song2_tables *t) {
  line(f, "This binary file was generated by the GB300 second-order evolver, in the layout of SONG's source "
          "files.");
  line(f, "");
  line(f, "Background: tau0 = %g Mpc, a_eq = %g", t->tau0, t->a_eq);
  line(f, "Perturbations: l_max_g = %d, l_max_pol_g = %d, l_max_ur = %d, rtol = %g, modes: %d", s->l_max_g,
       s->l_max_pol_g, s->l_max_ur, s->rtol, s->m_size);
  line(f, "gauge = newtonian");
}

int song2_write_sources_k(const song2_spec *s, const song2_tables *t, const double *flat, int i1, int i2,
                          const char *path, char *err) {
  if (i1 < 0 || i1 >= s->k_size || i2 < 0 || i2 > i1) {
    snprintf(err, SONG2_ERRLEN, "pair (%d, %d) outside the k grid (k2 <= k1 < %d)", i1, i2, s->k_size);
    return 1;
  }
  if (!t->fo || !t->fo_dd || t->fo_size < N_FO) {
    snprintf(err, SONG2_ERRLEN, "the first-order table is needed for the source files");
    return 1;
  }
  static bfile f;
  memset(&f, 0, sizeof f);
  int n3 = s->k3_size[i1 * s->k_size + i2], nt = s->tau_size;
  double k1 = s->k[i1], k2 = s->k[i2];
  /* the pair's k3 grid: the pairs before it hold pair_offset / tau_size k3 values */
  const double *k3 = s->k3 + song2_pair_offset(s, i1, i2) / s->tau_size;
  double *a = (double *)malloc(sizeof(double) * nt), *H = (double *)malloc(sizeof(double) * nt);
  double *mu = (double *)malloc(sizeof(double) * n3);
  double *f1 = (double *)malloc(sizeof(double) * nt * N_FO), *f2 = (double *)malloc(sizeof(double) * nt * N_FO);
  char *qs = (char *)calloc((size_t)N_FO * LABEL, 1);
  int ntp;
  char *tpl = labels(s, &ntp);
  for (int i = 0; i < nt; ++i) {
    background(t, s->tau[i], a + i, H + i);
    first_order(t, i1, s->tau[i], f1 + (size_t)i * N_FO);
    first_order(t, i2, s->tau[i], f2 + (size_t)i * N_FO);
  }
  for (int j = 0; j < n3; ++j) mu[j] = (k3[j] * k3[j] - k1 * k1 - k2 * k2) / (2 * k1 * k2);
  for (int q = 0; q < N_FO; ++q) snprintf(qs + (size_t)q * LABEL, LABEL, "%s", FO_LABELS[q]);
  int label = LABEL, nfo = N_FO, block = nt * n3;
  line(&f, "Table of the source function S_lm(k1,k2,k3,tau) tabulated as a function of (l,m,k3,tau) for fixed k1 "
           "and k2.");
  common_header(&f, s, t);
  line(&f, "k1 = %g, k2 = %g", k1, k2);
  line(&f, "index_k1 = %d/%d, index_k2 = %d/%d, k3_size = %d", i1, s->k_size - 1, i2, s->k_size - 1, n3);
  char d[160], nm[120];
  add(&f, "int", 4, 1, &label, "length of a label", "_MAX_LENGTH_LABEL_");
  add(&f, "double", 8, 1, &k1, "wavemode k1", "ppt2->k[index_k1]");
  add(&f, "double", 8, 1, &k2, "wavemode k2", "ppt2->k[index_k2]");
  add(&f, "int", 4, 1, &s->tau_size, "size of tau, scale factor and H arrays", "ppt2->tau_size");
  add(&f, "double", 8, nt, s->tau, "tau array of conformal times", "ppt2->tau_sampling");
  add(&f, "double", 8, nt, a, "scale factor array", "a");
  add(&f, "double", 8, nt, H, "Hubble factor array", "H");
  add(&f, "int", 4, 1, &s->k3_size[i1 * s->k_size + i2], "size of k3 and mu arrays", "ppt2->k3_size");
  add(&f, "double", 8, n3, k3, "k3 array", "ppt2->k3");
  add(&f, "double", 8, n3, mu, "array of the cosine of the angle between k1 and k2", "mu");
  add(&f, "int", 4, 1, &nfo, "number of first-order perturbations", "ppt->qs_size_short");
  add(&f, "char", 1, (int64_t)N_FO * LABEL, qs, "array of names of first-order perturbations", "ppt->qs_labels");
  add(&f, "double", 8, (int64_t)nt * N_FO, f1, "first-order perturbations in k1: [index_tau][index_qs]",
      "pvec_sources1");
  add(&f, "double", 8, (int64_t)nt * N_FO, f2, "first-order perturbations in k2: [index_tau][index_qs]",
      "pvec_sources2");
  add(&f, "int", 4, 1, &ntp, "number of source types, including l,m", "ppt2->tp2_size");
  add(&f, "char", 1, (int64_t)ntp * LABEL, tpl, "array of names of source types", "ppt2->tp2_labels");
  add(&f, "int", 4, 1, &block, "size of a (k3,tau) block", "ppt2->tau_size * ppt2->k3_size");
  int64_t per_type = song2_sources_per_type(s), off = song2_pair_offset(s, i1, i2);
  for (int tp = 0; tp < ntp; ++tp) {
    snprintf(d, sizeof d, "source function %s for all values of k3 and tau", tpl + (size_t)tp * LABEL);
    snprintf(nm, sizeof nm, "ppt2->sources[index_tp2=%d][index_k1=%d][index_k2=%d]", tp, i1, i2);
    add(&f, "double", 8, block, flat + (size_t)tp * per_type + off, d, nm);
  }
  int rc = write_file(&f, path, err);
  free(a);
  free(H);
  free(mu);
  free(f1);
  free(f2);
  free(qs);
  free(tpl);
  return rc;
}

int song2_write_sources_tau(const song2_spec *s, const song2_tables *t, const double *flat, int index_tau,
                            const char *path, char *err) {
  if (index_tau < 0 || index_tau >= s->tau_size) {
    snprintf(err, SONG2_ERRLEN, "index_tau %d outside 0..%d", index_tau, s->tau_size - 1);
    return 1;
  }
  if (!t->fo || !t->fo_dd || t->fo_size < N_FO) {
    snprintf(err, SONG2_ERRLEN, "the first-order table is needed for the source files");
    return 1;
  }
  static bfile f;
  memset(&f, 0, sizeof f);
  double tau = s->tau[index_tau], a, H;
  background(t, tau, &a, &H);
  double z = 1 / a - 1;
  int n_pairs = s->k_size * (s->k_size + 1) / 2;
  int *sizes = (int *)malloc(sizeof(int) * n_pairs);
  int64_t nk3 = 0;
  {
    int p = 0;
    for (int i1 = 0; i1 < s->k_size; ++i1)
      for (int i2 = 0; i2 <= i1; ++i2, ++p) {
        sizes[p] = s->k3_size[i1 * s->k_size + i2];
        nk3 += sizes[p];
      }
  }
  double *fo = (double *)malloc(sizeof(double) * s->k_size * N_FO);
  for (int k = 0; k < s->k_size; ++k) first_order(t, k, tau, fo + (size_t)k * N_FO);
  char *qs = (char *)calloc((size_t)N_FO * LABEL, 1);
  for (int q = 0; q < N_FO; ++q) snprintf(qs + (size_t)q * LABEL, LABEL, "%s", FO_LABELS[q]);
  int ntp;
  char *tpl = labels(s, &ntp);
  /* every source type at this time, packed over the pairs in pair order */
  double *src = (double *)malloc(sizeof(double) * (size_t)ntp * (nk3 ? nk3 : 1));
  int64_t per_type = song2_sources_per_type(s);
  for (int tp = 0; tp < ntp; ++tp) {
    int64_t o = 0;
    for (int i1 = 0; i1 < s->k_size; ++i1)
      for (int i2 = 0; i2 <= i1; ++i2) {
        int n3 = s->k3_size[i1 * s->k_size + i2];
        const double *blk = flat + (size_t)tp * per_type + song2_pair_offset(s, i1, i2) + (size_t)index_tau * n3;
        memcpy(src + (size_t)tp * nk3 + o, blk, sizeof(double) * n3);
        o += n3;
      }
  }
  int label = LABEL, nfo = N_FO;
  line(&f, "Table of the source function S_lm(k1,k2,k3,tau) tabulated as a function of (l,m,k1,k2,k3) for fixed "
           "tau=%g (z=%g).",
       tau, z);
  common_header(&f, s, t);
  line(&f, "tau = %g, z = %g, a = %g, y = %g", tau, z, a, log10(a / t->a_eq));
  char d[160];
  add(&f, "int", 4, 1, &label, "length of a label", "_MAX_LENGTH_LABEL_");
  add(&f, "double", 8, 1, &z, "redshift", "z");
  add(&f, "double", 8, 1, &tau, "conformal time", "tau");
  add(&f, "int", 4, 1, &index_tau, "index of tau inside ppt2->tau_sampling", "index_tau");
  add(&f, "double", 8, 1, &a, "scale factor", "a");
  add(&f, "double", 8, 1, &H, "Hubble factor", "H");
  add(&f, "int", 4, 1, &s->k_size, "size of k array", "ppt2->k_size");
  add(&f, "double", 8, s->k_size, s->k, "k array", "ppt2->k");
  add(&f, "int", 4, n_pairs, sizes, "size of k3 grid: k3_size[index_k1][index_k2], index_k2 <= index_k1",
      "ppt2->k3_size");
  add(&f, "double", 8, nk3, s->k3, "k3 array: k3[index_k1][index_k2], index_k2 <= index_k1", "ppt2->k3");
  add(&f, "int", 4, 1, &nfo, "number of first-order perturbations", "ppt->qs_size_short");
  add(&f, "char", 1, (int64_t)N_FO * LABEL, qs, "array of names of first-order perturbations", "ppt->qs_labels");
  add(&f, "double", 8, (int64_t)s->k_size * N_FO, fo, "first-order perturbations: [index_k][index_qs]",
      "pvec_sources");
  add(&f, "int", 4, 1, &ntp, "number of source types, including l,m", "ppt2->tp2_size");
  add(&f, "char", 1, (int64_t)ntp * LABEL, tpl, "array of names of source types", "ppt2->tp2_labels");
  for (int tp = 0; tp < ntp; ++tp) {
    snprintf(d, sizeof d, "source function %s for all values of (k1,k2,k3)", tpl + (size_t)tp * LABEL);
    add(&f, "double", 8, nk3, src + (size_t)tp * nk3, d, "ppt2->sources");
  }
  int rc = write_file(&f, path, err);
  free(sizes);
  free(fo);
  free(qs);
  free(tpl);
  free(src);
  return rc;
}
