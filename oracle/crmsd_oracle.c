/*
 * crmsd_oracle.c -- CPU FP64 oracle for all-vs-all crmsd.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links or calls
 * this file; it is used by tests/ (as the checker), by __graft_entry__.smoke()
 * and by the cpu_baseline / --impl reference legs of bench.py.
 *
 * The reference snapshot (BioShell 4.0.0-dev) has no crmsd function: the only
 * trace is the dependency comment at bioshell-pdb/Cargo.toml:27
 * ("nalgebra ... # for helical axis and crmsd"), and bioshell-pdb/src/calc/
 * mod.rs:1-10 exports no superposition routine.  This file therefore restates
 * the published QCP method (D. L. Theobald, Acta Cryst. A61:478, 2005;
 * P. Liu, D. K. Agrafiotis, D. L. Theobald, J. Comput. Chem. 31:1561, 2010)
 * from the mathematics, in the conventions the reference uses elsewhere:
 *   - coordinates are f64 AoS xyz triples (bioshell-core/src/vec3.rs:44-51);
 *   - every atom has the same weight, centring is by the arithmetic mean
 *     (bioshell-pdb/src/calc/substructures.rs:26-31);
 *   - only proper rotations are allowed.
 * Parity with the reference is therefore UNPINNED for the crmsd values
 * themselves; tests pin this oracle with analytic known answers (identity,
 * rigid motion, mirror images) and an independent numpy SVD-Kabsch.
 *
 * Method, per pair (A, B) of L index-matched points:
 *   a_k, b_k   centred coordinates,   G_a = sum |a_k|^2,  G_b = sum |b_k|^2
 *   S_xy       = sum_k a_kx b_ky                       (3x3)
 *   K(S)       4x4 symmetric, traceless key matrix (quaternion form)
 *   P(l)       = det(K - l I) = l^4 + c2 l^2 + c1 l + c0
 *              c2 = -2 ||S||_F^2, c1 = -8 det S, c0 = det K
 *   l_max      largest root, by Newton from (G_a + G_b)/2 (an upper bound)
 *   RMSD       = sqrt(max(0, (G_a + G_b - 2 l_max) / L))
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORACLE_API __attribute__((visibility("default")))

/* ------------------------------------------------------------------ */
/* 3x3 and 4x4 helpers                                                */
/* ------------------------------------------------------------------ */
static double det3(const double m[9]) {
  return m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
         m[2] * (m[3] * m[7] - m[4] * m[6]);
}

/* Determinant of a 4x4 matrix by Laplace expansion over the 2x2 minors of
 * rows (0,1) and their complements in rows (2,3). */
static double det4(const double k[16]) {
  const double *r0 = k, *r1 = k + 4, *r2 = k + 8, *r3 = k + 12;
  double s01 = r0[0] * r1[1] - r0[1] * r1[0];
  double s02 = r0[0] * r1[2] - r0[2] * r1[0];
  double s03 = r0[0] * r1[3] - r0[3] * r1[0];
  double s12 = r0[1] * r1[2] - r0[2] * r1[1];
  double s13 = r0[1] * r1[3] - r0[3] * r1[1];
  double s23 = r0[2] * r1[3] - r0[3] * r1[2];
  double c23 = r2[2] * r3[3] - r2[3] * r3[2];
  double c13 = r2[1] * r3[3] - r2[3] * r3[1];
  double c12 = r2[1] * r3[2] - r2[2] * r3[1];
  double c03 = r2[0] * r3[3] - r2[3] * r3[0];
  double c02 = r2[0] * r3[2] - r2[2] * r3[0];
  double c01 = r2[0] * r3[1] - r2[1] * r3[0];
  return s01 * c23 - s02 * c13 + s03 * c12 + s12 * c03 - s13 * c02 + s23 * c01;
}

/* Key matrix K(S), row-major, S row-major with S[3*x+y] = sum a_x b_y. */
static void key_matrix(const double s[9], double k[16]) {
  double sxx = s[0], sxy = s[1], sxz = s[2];
  double syx = s[3], syy = s[4], syz = s[5];
  double szx = s[6], szy = s[7], szz = s[8];
  double m[16] = {sxx + syy + szz, syz - szy,        szx - sxz,        sxy - syx,
                  syz - szy,       sxx - syy - szz,  sxy + syx,        szx + sxz,
                  szx - sxz,       sxy + syx,        -sxx + syy - szz, syz + szy,
                  sxy - syx,       szx + sxz,        syz + szy,        -sxx - syy + szz};
  memcpy(k, m, sizeof(m));
}

/* Largest eigenvalue of K(S) by Newton on the characteristic quartic,
 * started from the upper bound lambda0 = (G_a + G_b) / 2. */
static double qcp_lambda_max(const double s[9], double lambda0) {
  double k[16];
  key_matrix(s, k);
  double fro2 = 0.0;
  for (int i = 0; i < 9; ++i) fro2 += s[i] * s[i];
  const double c2 = -2.0 * fro2;
  const double c1 = -8.0 * det3(s);
  const double c0 = det4(k);
  double x = lambda0;
  for (int it = 0; it < 60; ++it) {
    double x2 = x * x;
    double p = (x2 + c2) * x2 + c1 * x + c0;
    double dp = (4.0 * x2 + 2.0 * c2) * x + c1;
    if (dp == 0.0) break;
    double dx = p / dp;
    x -= dx;
    if (fabs(dx) <= 1e-15 * fabs(x)) break;
  }
  return x;
}

/* ------------------------------------------------------------------ */
/* Per-structure preparation: centred copy (K-major [3][L]) and G     */
/* ------------------------------------------------------------------ */
typedef struct {
  int64_t n;
  int L;
  double *cen; /* [n][3][L] centred coordinates */
  double *g;   /* [n] sum of squared centred coordinates */
} prepared_t;

static int prepare(const double *xyz, int64_t n, int L, prepared_t *p) {
  p->n = n;
  p->L = L;
  p->cen = (double *)malloc(sizeof(double) * (size_t)n * 3 * (size_t)L);
  p->g = (double *)malloc(sizeof(double) * (size_t)n);
  if (!p->cen || !p->g) {
    free(p->cen);
    free(p->g);
    return -1;
  }
  for (int64_t s = 0; s < n; ++s) {
    const double *x = xyz + (size_t)s * 3 * L;
    double c[3] = {0, 0, 0};
    for (int k = 0; k < L; ++k)
      for (int d = 0; d < 3; ++d) c[d] += x[3 * k + d];
    for (int d = 0; d < 3; ++d) c[d] /= (double)L;
    double g = 0.0;
    double *y = p->cen + (size_t)s * 3 * L;
    for (int k = 0; k < L; ++k)
      for (int d = 0; d < 3; ++d) {
        double v = x[3 * k + d] - c[d];
        y[(size_t)d * L + k] = v;
        g += v * v;
      }
    p->g[s] = g;
  }
  return 0;
}

static void release(prepared_t *p) {
  free(p->cen);
  free(p->g);
}

static double pair_rmsd(const prepared_t *p, int64_t i, int64_t j) {
  const int L = p->L;
  const double *a = p->cen + (size_t)i * 3 * L;
  const double *b = p->cen + (size_t)j * 3 * L;
  double s[9];
  for (int x = 0; x < 3; ++x)
    for (int y = 0; y < 3; ++y) {
      const double *ax = a + (size_t)x * L, *by = b + (size_t)y * L;
      double acc = 0.0;
      for (int k = 0; k < L; ++k) acc += ax[k] * by[k];
      s[3 * x + y] = acc;
    }
  const double gsum = p->g[i] + p->g[j];
  const double lmax = qcp_lambda_max(s, 0.5 * gsum);
  double e = (gsum - 2.0 * lmax) / (double)L;
  return e > 0.0 ? sqrt(e) : 0.0;
}

/* ------------------------------------------------------------------ */
/* Public oracle entry points                                         */
/* ------------------------------------------------------------------ */

/* crmsd of one pair, raw (uncentred) AoS coordinates a[L][3], b[L][3]. */
ORACLE_API double bs_oracle_crmsd(const double *a, const double *b, int L) {
  double both[2 * 3 * 4096];
  double *buf = both;
  if (L > 4096) buf = (double *)malloc(sizeof(double) * 6 * (size_t)L);
  if (!buf) return NAN;
  memcpy(buf, a, sizeof(double) * 3 * (size_t)L);
  memcpy(buf + 3 * (size_t)L, b, sizeof(double) * 3 * (size_t)L);
  prepared_t p;
  double r = NAN;
  if (prepare(buf, 2, L, &p) == 0) {
    r = pair_rmsd(&p, 0, 1);
    release(&p);
  }
  if (buf != both) free(buf);
  return r;
}

/* Largest key-matrix eigenvalue and the three terms of the cancellation for
 * one pair; used by tests that pin the quartic against numpy eigvalsh. */
ORACLE_API void bs_oracle_pair_terms(const double *a, const double *b, int L, double *out4) {
  double both[2 * 3 * 4096];
  if (L > 4096) {
    out4[0] = out4[1] = out4[2] = out4[3] = NAN;
    return;
  }
  memcpy(both, a, sizeof(double) * 3 * (size_t)L);
  memcpy(both + 3 * (size_t)L, b, sizeof(double) * 3 * (size_t)L);
  prepared_t p;
  if (prepare(both, 2, L, &p) != 0) return;
  const double *ca = p.cen, *cb = p.cen + 3 * (size_t)L;
  double s[9];
  for (int x = 0; x < 3; ++x)
    for (int y = 0; y < 3; ++y) {
      double acc = 0.0;
      for (int k = 0; k < L; ++k) acc += ca[(size_t)x * L + k] * cb[(size_t)y * L + k];
      s[3 * x + y] = acc;
    }
  out4[0] = qcp_lambda_max(s, 0.5 * (p.g[0] + p.g[1]));
  out4[1] = p.g[0];
  out4[2] = p.g[1];
  out4[3] = pair_rmsd(&p, 0, 1);
  release(&p);
}

typedef struct {
  const prepared_t *p;
  const int64_t *ii, *jj; /* explicit pair list, or NULL for the triangle */
  int64_t npairs;
  double *out;
  int64_t row_begin, row_end; /* triangle rows [row_begin, row_end) */
} job_t;

static int64_t tri_index(int64_t n, int64_t i, int64_t j) {
  return i * n - i * (i + 1) / 2 + (j - i - 1);
}

static void *worker_tri(void *arg) {
  job_t *jb = (job_t *)arg;
  const int64_t n = jb->p->n;
  for (int64_t i = jb->row_begin; i < jb->row_end; ++i)
    for (int64_t j = i + 1; j < n; ++j) jb->out[tri_index(n, i, j)] = pair_rmsd(jb->p, i, j);
  return NULL;
}

static void *worker_pairs(void *arg) {
  job_t *jb = (job_t *)arg;
  for (int64_t t = jb->row_begin; t < jb->row_end; ++t) jb->out[t] = pair_rmsd(jb->p, jb->ii[t], jb->jj[t]);
  return NULL;
}

/* Row ranges with roughly equal pair counts for the upper triangle. */
static void split_triangle(int64_t n, int nt, int64_t *bounds) {
  const double total = 0.5 * (double)n * (double)(n - 1);
  int64_t row = 0;
  bounds[0] = 0;
  for (int t = 1; t < nt; ++t) {
    const double target = total * t / nt;
    double done = 0.0;
    row = 0;
    /* pairs in rows [0, r) = r*n - r(r+1)/2 */
    int64_t lo = 0, hi = n;
    while (lo < hi) {
      int64_t mid = (lo + hi) / 2;
      done = (double)mid * n - 0.5 * (double)mid * (mid + 1);
      if (done < target) lo = mid + 1; else hi = mid;
    }
    row = lo;
    bounds[t] = row < bounds[t - 1] ? bounds[t - 1] : row;
  }
  bounds[nt] = n;
}

/* Full upper triangle, row-major without the diagonal:
 * out[i*n - i(i+1)/2 + (j-i-1)] = crmsd(i, j) for i < j. */
ORACLE_API int bs_oracle_all_vs_all(const double *xyz, int64_t n, int L, double *out, int nthreads) {
  if (n < 0 || L < 1 || nthreads < 1) return -1;
  if (n < 2) return 0;
  prepared_t p;
  if (prepare(xyz, n, L, &p) != 0) return -2;
  if (nthreads > 256) nthreads = 256;
  pthread_t th[256];
  job_t jobs[256];
  int64_t bounds[257];
  split_triangle(n, nthreads, bounds);
  for (int t = 0; t < nthreads; ++t) {
    jobs[t] = (job_t){&p, NULL, NULL, 0, out, bounds[t], bounds[t + 1]};
    pthread_create(&th[t], NULL, worker_tri, &jobs[t]);
  }
  for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
  release(&p);
  return 0;
}

/* Explicit pair list: out[t] = crmsd(ii[t], jj[t]). */
ORACLE_API int bs_oracle_pairs(const double *xyz, int64_t n, int L, const int64_t *ii, const int64_t *jj,
                               int64_t npairs, double *out, int nthreads) {
  if (n < 1 || L < 1 || nthreads < 1 || npairs < 0) return -1;
  for (int64_t t = 0; t < npairs; ++t)
    if (ii[t] < 0 || ii[t] >= n || jj[t] < 0 || jj[t] >= n) return -3;
  prepared_t p;
  if (prepare(xyz, n, L, &p) != 0) return -2;
  if (nthreads > 256) nthreads = 256;
  pthread_t th[256];
  job_t jobs[256];
  for (int t = 0; t < nthreads; ++t) {
    int64_t b = npairs * t / nthreads, e = npairs * (t + 1) / nthreads;
    jobs[t] = (job_t){&p, ii, jj, npairs, out, b, e};
    pthread_create(&th[t], NULL, worker_pairs, &jobs[t]);
  }
  for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
  release(&p);
  return 0;
}
