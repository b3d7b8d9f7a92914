/* Test infrastructure: NOT part of the product.
 *
 * CPU restatement, in plain C + OpenMP, of the reference's scalar IMSRG(2)
 * commutator and BCH transform (IMSRG++ src/Commutator.cc, src/BCH.cc,
 * src/TwoBodyME.cc).  It is the checker for the GPU product at sizes the
 * golden fixtures do not cover and the timed CPU baseline ("port") of the
 * benchmark.  Only tests/, __graft_entry__.smoke() and bench.py's CPU legs use
 * it.  Every function cites the reference lines it follows; the loop structure,
 * the skipped zero blocks, the |6j| < 1e-8 cut and the OpenMP decomposition are
 * the reference's.  Matrix products go through a dgemm the caller supplies
 * (the Python wrapper hands in SciPy's BLAS, matching the reference's BLAS
 * path); without one a plain triple loop is used.
 *
 * Operators are "arenas": ZeroBody at [0], OneBody N x N column-major at [32],
 * one n x n column-major block per two-body channel at off2[ch].
 * Hermiticity flags: +1 hermitian, -1 anti-hermitian, 0 neither.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "ref_stubs/coupling_stub.c"

#define SQRT2 1.4142135623730950488
#define OCC_CUT 1e-6

typedef void (*dgemm_fn)(const char*, const char*, const int*, const int*, const int*, const double*,
                         const double*, const int*, const double*, const int*, const double*, double*,
                         const int*);

typedef struct {
  int n;
  int *p, *q;          /* kets, local order */
  int *hh, *ph, *pp;   /* local indices by class (ascending) */
  int nhh, nph, npp;
  double *occ_hh, *unocc_hh, *occ_ph, *unocc_ph;
} ochan;

typedef struct {
  int norb, nch, nkets, emax;
  int *l, *j2, *tz2;
  double* occ;
  int nholes;
  int* holes;
  ochan* ch;
  ochan* cc;
  int* ketmap;   /* [nch * nkets] local index or -1 */
  int* ccketmap; /* [nch * nkets] */
  int64_t* off2;
  int64_t arena;
  /* SixJCache_112112 (src/AngMomCache.cc:58-104): jj1 <= jjmax, J <= jjmax */
  int d1, d2;
  double* sixj;
  dgemm_fn gemm;
  /* term switches: 110 220 111 121 122 222pphh 221 222ph */
  int term_on[8];
} ospace;

enum { T110, T220, T111, T121, T122, T222PPHH, T221, T222PH };

/* ---------------------------------------------------------------- helpers */
static int iphase(int x) { return (x % 2 == 0) ? 1 : -1; }

static int index2(const ospace* s, int p, int q) { return p * (2 * s->norb - 1 - p) / 2 + q; }

static int chan_index(int J, int par, int Tz) { return 6 * J + 2 * (Tz + 1) + par; }

static double sixj_cached(const ospace* s, int jj1, int jj2, int j3, int jj4, int jj5, int j6)
{
  /* JJSToIndex, src/AngMomCache.hh:15-22 */
  size_t d1 = s->d1, d2 = s->d2;
  size_t idx = d1 * d2 * d1 * d1 * d2 * ((jj1 - 1) / 2) + d2 * d1 * d1 * d2 * ((jj2 - 1) / 2) +
               d1 * d1 * d2 * (size_t)j3 + d1 * d2 * ((jj4 - 1) / 2) + d2 * ((jj5 - 1) / 2) + (size_t)j6;
  return s->sixj[idx];
}

static void gemm_nn(const ospace* s, int m, int n, int k, double alpha, const double* A, int lda,
                    const double* B, int ldb, double beta, double* C, int ldc)
{
  if (m <= 0 || n <= 0) return;
  if (k <= 0) {
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < m; ++i) C[(size_t)j * ldc + i] *= beta;
    return;
  }
  if (s->gemm) {
    s->gemm("N", "N", &m, &n, &k, &alpha, A, &lda, B, &ldb, &beta, C, &ldc);
    return;
  }
  for (int j = 0; j < n; ++j) {
    double* c = C + (size_t)j * ldc;
    for (int i = 0; i < m; ++i) c[i] *= beta;
    for (int kk = 0; kk < k; ++kk) {
      double b = alpha * B[(size_t)j * ldb + kk];
      const double* a = A + (size_t)kk * lda;
      for (int i = 0; i < m; ++i) c[i] += a[i] * b;
    }
  }
}

/* TwoBodyME::GetTBME_J_norm for a scalar operator (src/TwoBodyME.cc:339-356,132-153) */
static double tbme_J_norm(const ospace* s, const double* op, int J, int a, int b, int c, int d)
{
  int pb = (s->l[a] + s->l[b]) % 2, pk = (s->l[c] + s->l[d]) % 2;
  int tb = (s->tz2[a] + s->tz2[b]) / 2, tk = (s->tz2[c] + s->tz2[d]) / 2;
  if ((pb + pk) % 2) return 0.0;
  if (tb != tk) return 0.0;
  int ch = chan_index(J, pb, tb);
  if (ch >= s->nch) return 0.0;
  int n = s->ch[ch].n;
  int bi = s->ketmap[(size_t)ch * s->nkets + index2(s, a < b ? a : b, a < b ? b : a)];
  int ki = s->ketmap[(size_t)ch * s->nkets + index2(s, c < d ? c : d, c < d ? d : c)];
  if (bi < 0 || ki < 0) return 0.0;
  double ph = 1.0;
  if (a > b) ph *= iphase((s->j2[a] + s->j2[b]) / 2 + 1 + J);
  if (c > d) ph *= iphase((s->j2[c] + s->j2[d]) / 2 + 1 + J);
  return ph * op[s->off2[ch] + (int64_t)ki * n + bi];
}

static double tbme_J(const ospace* s, const double* op, int J, int a, int b, int c, int d)
{
  double nrm = 1.0;
  if (a == b) nrm *= SQRT2;
  if (c == d) nrm *= SQRT2;
  return nrm * tbme_J_norm(s, op, J, a, b, c, d);
}

/* TwoBodyME::GetTBMEmonopole (src/TwoBodyME.cc:615-682) */
static double tbme_monopole(const ospace* s, const double* op, int a, int b, int c, int d)
{
  int pab = (s->l[a] + s->l[b]) % 2, pcd = (s->l[c] + s->l[d]) % 2;
  int tab = (s->tz2[a] + s->tz2[b]) / 2, tcd = (s->tz2[c] + s->tz2[d]) / 2;
  if ((pab + pcd) % 2) return 0.0;
  if (tab != tcd) return 0.0;
  int jmin = abs(s->j2[a] - s->j2[b]) / 2, jmax = (s->j2[a] + s->j2[b]) / 2;
  double mon = 0.0;
  for (int J = jmin; J <= jmax; ++J) mon += (2 * J + 1) * tbme_J_norm(s, op, J, a, b, c, d);
  mon /= (double)((s->j2[a] + 1) * (s->j2[b] + 1));
  double nrm = 1.0;
  if (a == b) nrm *= SQRT2;
  if (c == d) nrm *= SQRT2;
  return nrm * mon;
}

/* ------------------------------------------------------------ the space */
static int* ialloc(size_t n) { return (int*)calloc(n ? n : 1, sizeof(int)); }
static double* dalloc(size_t n) { return (double*)calloc(n ? n : 1, sizeof(double)); }

/* Build the oracle's tables from the channel ket lists (which the Python
 * restatement of ModelSpace::SetupKets provides).  kets_p/kets_q hold, channel
 * after channel, the kets of the 2b channels; cc_p/cc_q those of the
 * cross-coupled channels. */
ospace* oracle_space_create(int emax, int norb, const int* l, const int* j2, const int* tz2, const double* occ,
                            int nch, const int* ch_n, const int* kets_p, const int* kets_q, const int* cc_n,
                            const int* cc_p, const int* cc_q)
{
  ospace* s = (ospace*)calloc(1, sizeof(ospace));
  s->emax = emax;
  s->norb = norb;
  s->nch = nch;
  s->nkets = norb * (norb + 1) / 2;
  s->l = ialloc(norb);
  s->j2 = ialloc(norb);
  s->tz2 = ialloc(norb);
  s->occ = dalloc(norb);
  memcpy(s->l, l, norb * sizeof(int));
  memcpy(s->j2, j2, norb * sizeof(int));
  memcpy(s->tz2, tz2, norb * sizeof(int));
  memcpy(s->occ, occ, norb * sizeof(double));
  s->holes = ialloc(norb);
  for (int i = 0; i < norb; ++i)
    if (occ[i] >= OCC_CUT) s->holes[s->nholes++] = i;
  for (int t = 0; t < 8; ++t) s->term_on[t] = 1;
  s->ch = (ochan*)calloc(nch, sizeof(ochan));
  s->cc = (ochan*)calloc(nch, sizeof(ochan));
  s->ketmap = ialloc((size_t)nch * s->nkets);
  s->ccketmap = ialloc((size_t)nch * s->nkets);
  for (size_t i = 0; i < (size_t)nch * s->nkets; ++i) s->ketmap[i] = s->ccketmap[i] = -1;
  s->off2 = (int64_t*)calloc(nch, sizeof(int64_t));
  int64_t cur = ((int64_t)32 + (int64_t)norb * norb + 31) / 32 * 32;
  int kofs = 0, cofs = 0;
  for (int c = 0; c < nch; ++c) {
    for (int pass = 0; pass < 2; ++pass) {
      ochan* C = pass == 0 ? &s->ch[c] : &s->cc[c];
      int n = pass == 0 ? ch_n[c] : cc_n[c];
      const int* P = pass == 0 ? kets_p + kofs : cc_p + cofs;
      const int* Q = pass == 0 ? kets_q + kofs : cc_q + cofs;
      int* map = (pass == 0 ? s->ketmap : s->ccketmap) + (size_t)c * s->nkets;
      C->n = n;
      C->p = ialloc(n);
      C->q = ialloc(n);
      C->hh = ialloc(n);
      C->ph = ialloc(n);
      C->pp = ialloc(n);
      C->occ_hh = dalloc(n);
      C->unocc_hh = dalloc(n);
      C->occ_ph = dalloc(n);
      C->unocc_ph = dalloc(n);
      for (int i = 0; i < n; ++i) {
        int p = P[i], q = Q[i];
        C->p[i] = p;
        C->q[i] = q;
        map[index2(s, p, q)] = i;
        double op = occ[p], oq = occ[q];
        if (op < OCC_CUT && oq < OCC_CUT) C->pp[C->npp++] = i;
        if ((op > OCC_CUT) != (oq > OCC_CUT)) {
          C->occ_ph[C->nph] = op * oq;
          C->unocc_ph[C->nph] = (1 - op) * (1 - oq);
          C->ph[C->nph++] = i;
        }
        if (op > OCC_CUT && oq > OCC_CUT) {
          C->occ_hh[C->nhh] = op * oq;
          C->unocc_hh[C->nhh] = (1 - op) * (1 - oq);
          C->hh[C->nhh++] = i;
        }
      }
    }
    kofs += ch_n[c];
    cofs += cc_n[c];
    s->off2[c] = cur;
    cur = (cur + (int64_t)ch_n[c] * ch_n[c] + 31) / 32 * 32;
  }
  s->arena = cur;
  /* SixJCache_112112(2*emax+1) */
  int jjmax = 2 * emax + 1;
  s->d1 = (jjmax - 1) / 2 + 1;
  s->d2 = jjmax + 1;
  size_t d1 = s->d1, d2 = s->d2;
  size_t tot = d1 * d1 * d2 * d1 * d1 * d2;
  s->sixj = dalloc(tot);
#pragma omp parallel for schedule(dynamic, 1)
  for (int a = 0; a < s->d1; ++a)
    for (int b = 0; b < s->d1; ++b)
      for (int J3 = 0; J3 < s->d2; ++J3)
        for (int c = 0; c < s->d1; ++c)
          for (int d = 0; d < s->d1; ++d)
            for (int J6 = 0; J6 < s->d2; ++J6) {
              size_t idx = d1 * d2 * d1 * d1 * d2 * a + d2 * d1 * d1 * d2 * b + d1 * d1 * d2 * J3 +
                           d1 * d2 * c + d2 * d + J6;
              s->sixj[idx] = gsl_sf_coupling_6j(2 * a + 1, 2 * b + 1, 2 * J3, 2 * c + 1, 2 * d + 1, 2 * J6);
            }
  return s;
}

void oracle_space_destroy(ospace* s)
{
  if (!s) return;
  for (int c = 0; c < s->nch; ++c)
    for (int pass = 0; pass < 2; ++pass) {
      ochan* C = pass == 0 ? &s->ch[c] : &s->cc[c];
      free(C->p); free(C->q); free(C->hh); free(C->ph); free(C->pp);
      free(C->occ_hh); free(C->unocc_hh); free(C->occ_ph); free(C->unocc_ph);
    }
  free(s->ch); free(s->cc); free(s->ketmap); free(s->ccketmap); free(s->off2);
  free(s->l); free(s->j2); free(s->tz2); free(s->occ); free(s->holes); free(s->sixj);
  free(s);
}

int64_t oracle_arena_size(const ospace* s) { return s->arena; }
void oracle_set_dgemm(ospace* s, void* fn) { s->gemm = (dgemm_fn)fn; }
void oracle_set_term(ospace* s, int term, int on) { if (term >= 0 && term < 8) s->term_on[term] = on; }
double oracle_sixj(const ospace* s, int jj1, int jj2, int j3, int jj4, int jj5, int j6)
{
  return sixj_cached(s, jj1, jj2, j3, jj4, jj5, j6);
}

#define ONE(op, r, c) ((op)[32 + (size_t)(c) * N + (r)])

/* ------------------------------------------------------------- 0b / 1b terms */
/* comm110ss, src/Commutator.cc:564-581 */
void oracle_comm110ss(const ospace* s, const double* X, const double* Y, double* Z, int hX, int hY)
{
  if (hX == hY && hX != 0) return;
  int N = s->norb;
  for (int k = 0; k < s->nholes; ++k) {
    int a = s->holes[k];
    double xy = 0, yx = 0;
    for (int b = 0; b < N; ++b) {
      xy += ONE(X, a, b) * ONE(Y, b, a);
      yx += ONE(Y, a, b) * ONE(X, b, a);
    }
    Z[0] += (s->j2[a] + 1) * s->occ[a] * (xy - yx);
  }
}

/* comm220ss, src/Commutator.cc:601-631 */
void oracle_comm220ss(const ospace* s, const double* X, const double* Y, double* Z, int hX, int hY)
{
  if (hX == hY && hX != 0) return;
  for (int c = 0; c < s->nch; ++c) {
    const ochan* C = &s->ch[c];
    if (C->nhh == 0) continue;
    int J = c / 6, n = C->n;
    const double* Xc = X + s->off2[c];
    const double* Yc = Y + s->off2[c];
    double tr = 0;
    for (int ih = 0; ih < C->nhh; ++ih) {
      int h = C->hh[ih];
      double d = 0;
      /* nbar_indices = [hh, ph, pp]; hh and ph rows of Y weighted by nbar nbar */
      for (int k = 0; k < C->nhh; ++k) d += Xc[(size_t)C->hh[k] * n + h] * Yc[(size_t)h * n + C->hh[k]] * C->unocc_hh[k];
      for (int k = 0; k < C->nph; ++k) d += Xc[(size_t)C->ph[k] * n + h] * Yc[(size_t)h * n + C->ph[k]] * C->unocc_ph[k];
      for (int k = 0; k < C->npp; ++k) d += Xc[(size_t)C->pp[k] * n + h] * Yc[(size_t)h * n + C->pp[k]];
      tr += d * C->occ_hh[ih];
    }
    Z[0] += 2 * (2 * J + 1) * tr;
  }
}

/* comm111ss, src/Commutator.cc:644-649 */
void oracle_comm111ss(const ospace* s, const double* X, const double* Y, double* Z)
{
  int N = s->norb;
  double* t = dalloc((size_t)N * N);
  gemm_nn(s, N, N, N, 1.0, X + 32, N, Y + 32, N, 0.0, t, N);
  gemm_nn(s, N, N, N, -1.0, Y + 32, N, X + 32, N, 1.0, t, N);
  for (size_t i = 0; i < (size_t)N * N; ++i) Z[32 + i] += t[i];
  free(t);
}

static int same_1b_channel(const ospace* s, int a, int b)
{
  return s->l[a] == s->l[b] && s->j2[a] == s->j2[b] && s->tz2[a] == s->tz2[b];
}

/* comm121ss, src/Commutator.cc:670-728 */
void oracle_comm121ss(const ospace* s, const double* X, const double* Y, double* Z, int hZ)
{
  int N = s->norb;
#pragma omp parallel for schedule(dynamic, 1)
  for (int i = 0; i < N; ++i) {
    int jmin = (hZ == 0) ? 0 : i;
    for (int j = 0; j < N; ++j) {
      if (!same_1b_channel(s, i, j) || j < jmin) continue;
      double zij = 0;
      for (int ia = 0; ia < s->nholes; ++ia) {
        int a = s->holes[ia];
        for (int b = 0; b < N; ++b) {
          if (!same_1b_channel(s, a, b)) continue;
          double nanb = s->occ[a] * (1 - s->occ[b]);
          if (fabs(nanb) < OCC_CUT) continue;
          double ybiaj = tbme_monopole(s, Y, b, i, a, j);
          double yaibj = tbme_monopole(s, Y, a, i, b, j);
          zij += (s->j2[b] + 1) * nanb * ONE(X, a, b) * ybiaj;
          zij -= (s->j2[a] + 1) * nanb * ONE(X, b, a) * yaibj;
        }
        for (int b = 0; b < N; ++b) {
          if (!same_1b_channel(s, a, b)) continue;
          double nanb = s->occ[a] * (1 - s->occ[b]);
          if (fabs(nanb) < OCC_CUT) continue;
          zij -= (s->j2[b] + 1) * nanb * ONE(Y, a, b) * tbme_monopole(s, X, b, i, a, j);
          zij += (s->j2[a] + 1) * nanb * ONE(Y, b, a) * tbme_monopole(s, X, a, i, b, j);
        }
      }
      Z[32 + (size_t)j * N + i] += zij;
      if (jmin == i && j != i) Z[32 + (size_t)i * N + j] += hZ * zij;
    }
  }
}

/* ------------------------------------------------------------------ comm122ss */
/* comm122ss, src/Commutator.cc:837-932 */
void oracle_comm122ss(const ospace* s, const double* X, const double* Y, double* Z, int hZ)
{
  int N = s->norb;
#pragma omp parallel for schedule(dynamic, 1)
  for (int c = 0; c < s->nch; ++c) {
    const ochan* C = &s->ch[c];
    int n = C->n;
    if (n == 0) continue;
    int J = c / 6;
    const double* X2 = X + s->off2[c];
    const double* Y2 = Y + s->off2[c];
    double* Z2 = Z + s->off2[c];
    double* W2 = dalloc((size_t)n * n);
    const int* map = s->ketmap + (size_t)c * s->nkets;
    for (int ij = 0; ij < n; ++ij) {
      int i = C->p[ij], j = C->q[ij];
      int flip = -iphase((s->j2[i] + s->j2[j]) / 2 - J);
      double* w = W2 + (size_t)ij * n;
      /* a in the one-body channel of i, |aj> in this channel */
      for (int a = 0; a < N; ++a) {
        if (!same_1b_channel(s, a, i)) continue;
        int loc = map[index2(s, a < j ? a : j, a < j ? j : a)];
        if (loc < 0) continue;
        double f = a > j ? flip : (a == j ? SQRT2 : 1.0);
        if (i == j) f /= SQRT2;
        double xa = ONE(X, a, i) * f, ya = ONE(Y, a, i) * f;
        for (int r = 0; r < n; ++r) w[r] += Y2[(size_t)loc * n + r] * xa - X2[(size_t)loc * n + r] * ya;
      }
      if (i != j) {
        for (int a = 0; a < N; ++a) {
          if (!same_1b_channel(s, a, j)) continue;
          int loc = map[index2(s, a < i ? a : i, a < i ? i : a)];
          if (loc < 0) continue;
          double f = i > a ? flip : (i == a ? SQRT2 : 1.0);
          double xa = ONE(X, a, j) * f, ya = ONE(Y, a, j) * f;
          for (int r = 0; r < n; ++r) w[r] += Y2[(size_t)loc * n + r] * xa - X2[(size_t)loc * n + r] * ya;
        }
      } else {
        for (int r = 0; r < n; ++r) w[r] *= 2;
      }
    }
    for (int cc = 0; cc < n; ++cc)
      for (int r = 0; r < n; ++r) Z2[(size_t)cc * n + r] -= W2[(size_t)cc * n + r] + hZ * W2[(size_t)r * n + cc];
    free(W2);
  }
}

/* ----------------------------------------------------- pp/hh ladder + 221 */
static int is_zero_block(const double* a, size_t n)
{
  for (size_t i = 0; i < n; ++i)
    if (a[i] != 0.0) return 0;
  return 1;
}

/* M += A(:, idx) diag(w) B(idx, :) for an n x n channel block */
static void ladder_term(const ospace* s, int n, const double* A, const double* B, const int* idx, const double* w,
                        int k, double alpha, double* M)
{
  if (k == 0) return;
  double* Ac = dalloc((size_t)n * k);
  double* Br = dalloc((size_t)k * n);
  for (int t = 0; t < k; ++t) {
    memcpy(Ac + (size_t)t * n, A + (size_t)idx[t] * n, n * sizeof(double));
    double wt = w ? w[t] : 1.0;
    for (int c = 0; c < n; ++c) Br[(size_t)c * k + t] = wt * B[(size_t)c * n + idx[t]];
  }
  gemm_nn(s, n, n, k, alpha, Ac, n, Br, k, 1.0, M, n);
  free(Ac);
  free(Br);
}

/* ConstructScalarMpp_Mhh, src/Commutator.cc:1082-1210 (scalar X, Y) */
static void construct_mpp_mhh(const ospace* s, const double* X, const double* Y, int hZ, double* Mpp, double* Mhh)
{
#pragma omp parallel for schedule(dynamic, 1)
  for (int c = 0; c < s->nch; ++c) {
    const ochan* C = &s->ch[c];
    int n = C->n;
    if (n == 0) continue;
    const double* Xc = X + s->off2[c];
    const double* Yc = Y + s->off2[c];
    if (is_zero_block(Xc, (size_t)n * n) || is_zero_block(Yc, (size_t)n * n)) continue;
    double* P = Mpp + s->off2[c];
    double* H = Mhh + s->off2[c];
    ladder_term(s, n, Xc, Yc, C->pp, NULL, C->npp, 1.0, P);
    ladder_term(s, n, Xc, Yc, C->hh, C->occ_hh, C->nhh, 1.0, H);
    ladder_term(s, n, Xc, Yc, C->hh, C->unocc_hh, C->nhh, 1.0, P);
    ladder_term(s, n, Xc, Yc, C->ph, C->unocc_ph, C->nph, 1.0, P);
    if (hZ != 0) {
      for (int cc = 0; cc < n; ++cc)
        for (int r = cc; r < n; ++r) {
          double a = P[(size_t)cc * n + r], b = P[(size_t)r * n + cc];
          P[(size_t)cc * n + r] = a + hZ * b;
          P[(size_t)r * n + cc] = b + hZ * a;
          a = H[(size_t)cc * n + r];
          b = H[(size_t)r * n + cc];
          H[(size_t)cc * n + r] = a + hZ * b;
          H[(size_t)r * n + cc] = b + hZ * a;
        }
    } else {
      ladder_term(s, n, Yc, Xc, C->pp, NULL, C->npp, -1.0, P);
      ladder_term(s, n, Yc, Xc, C->hh, C->occ_hh, C->nhh, -1.0, H);
      ladder_term(s, n, Yc, Xc, C->hh, C->unocc_hh, C->nhh, -1.0, P);
      ladder_term(s, n, Yc, Xc, C->ph, C->unocc_ph, C->nph, -1.0, P);
    }
  }
}

/* the one-body part of comm222_pp_hh_221ss / comm221ss, src/Commutator.cc:1250-1294 */
static void onebody_from_m(const ospace* s, const double* Mpp, const double* Mhh, double* Z, int hZ)
{
  int N = s->norb;
#pragma omp parallel for schedule(dynamic, 1)
  for (int i = 0; i < N; ++i) {
    int jmin = hZ == 0 ? 0 : i;
    for (int j = 0; j < N; ++j) {
      if (!same_1b_channel(s, i, j) || j < jmin) continue;
      double zij = 0;
      for (int c = 0; c < N; ++c) {
        double nc = s->occ[c], nbarc = 1.0 - nc;
        int Jmin = abs(s->j2[c] - s->j2[i]);
        if (abs(s->j2[c] - s->j2[j]) > Jmin) Jmin = abs(s->j2[c] - s->j2[j]);
        Jmin /= 2;
        int Jmax = (s->j2[c] + (s->j2[i] < s->j2[j] ? s->j2[i] : s->j2[j])) / 2;
        if (fabs(nc) > 1e-9)
          for (int J = Jmin; J <= Jmax; ++J) zij += (2 * J + 1) * nc * tbme_J(s, Mpp, J, c, i, c, j);
        if (fabs(nbarc) > 1e-9)
          for (int J = Jmin; J <= Jmax; ++J) zij += (2 * J + 1) * nbarc * tbme_J(s, Mhh, J, c, i, c, j);
      }
      Z[32 + (size_t)j * N + i] += zij / (s->j2[i] + 1.0);
      if (jmin == i && i != j) Z[32 + (size_t)i * N + j] += hZ * zij / (s->j2[i] + 1.0);
    }
  }
}

/* comm222_pp_hh_221ss (src/Commutator.cc:1215-1301); do2b / do1b select
 * comm222_pp_hhss (src/Commutator.cc:1062-1076) and comm221ss
 * (src/Commutator.cc:760-819) */
void oracle_comm222_pp_hh_221ss(const ospace* s, const double* X, const double* Y, double* Z, int hZ, int do2b,
                                int do1b)
{
  double* Mpp = dalloc(s->arena);
  double* Mhh = dalloc(s->arena);
  construct_mpp_mhh(s, X, Y, hZ, Mpp, Mhh);
  if (do2b) {
    for (int c = 0; c < s->nch; ++c) {
      size_t nn = (size_t)s->ch[c].n * s->ch[c].n;
      double* z = Z + s->off2[c];
      const double* p = Mpp + s->off2[c];
      const double* h = Mhh + s->off2[c];
      for (size_t i = 0; i < nn; ++i) z[i] += p[i] - h[i];
    }
  }
  if (do1b) onebody_from_m(s, Mpp, Mhh, Z, hZ);
  free(Mpp);
  free(Mhh);
}

/* ------------------------------------------------------------- ph channel */
/* DoPandyaTransformation_SingleChannel_XandY, src/Commutator.cc:1392-1485.
 * Xb: nKets_cc x 2nph column-major, Yb: 2nph x nKets_cc column-major */
static void pandya_xy(const ospace* s, const double* X, const double* Y, int hY, int chcc, double* Xb, double* Yb,
                      int nph, const int* kets_ph)
{
  const ochan* C = &s->cc[chcc];
  int ncc = C->n;
  int Jcc = chcc / 6;
  for (int ibra = 0; ibra < nph; ++ibra) {
    int bp = C->p[kets_ph[ibra]], bq = C->q[kets_ph[ibra]];
    for (int ab_case = 0; ab_case <= 1; ++ab_case) {
      int a = ab_case ? bq : bp;
      int b = ab_case ? bp : bq;
      int shift = ab_case * nph;
      double na_nb = s->occ[a] - s->occ[b];
      for (int ik = 0; ik < ncc; ++ik) {
        int c = C->p[ik], d = C->q[ik];
        if (s->tz2[a] + s->tz2[d] - s->tz2[b] - s->tz2[c] != 0) continue;
        double nf = 1.0;
        if (a == d) nf *= SQRT2;
        if (c == b) nf *= SQRT2;
        int jmin = abs(s->j2[a] - s->j2[d]);
        if (abs(s->j2[c] - s->j2[b]) > jmin) jmin = abs(s->j2[c] - s->j2[b]);
        jmin /= 2;
        int jmax = s->j2[a] + s->j2[d];
        if (s->j2[c] + s->j2[b] < jmax) jmax = s->j2[c] + s->j2[b];
        jmax /= 2;
        int dJ = 1;
        if (a == d || c == b) {
          dJ = 2;
          jmin += jmin % 2;
        }
        double xbar = 0, ybar = 0;
        for (int J = jmin; J <= jmax; J += dJ) {
          double sj = sixj_cached(s, s->j2[a], s->j2[b], Jcc, s->j2[c], s->j2[d], J);
          if (fabs(sj) < 1e-8) continue;
          /* GetTBME_J_norm_twoOps(Y, J, J, c, b, a, d) */
          double xcbad = tbme_J_norm(s, X, J, c, b, a, d);
          double ycbad = tbme_J_norm(s, Y, J, c, b, a, d);
          xbar -= (2 * J + 1) * sj * xcbad;
          ybar -= (2 * J + 1) * sj * ycbad * hY;
        }
        Xb[(size_t)(ibra + shift) * ncc + ik] = xbar * nf * na_nb;
        Yb[(size_t)ik * (2 * nph) + ibra + shift] = ybar * nf;
      }
    }
  }
}

/* AddInversePandyaTransformation, src/Commutator.cc:1501-1616 */
static void inverse_pandya(const ospace* s, double** Zbar, double* Z, int hZ)
{
  int64_t total = 0;
  for (int c = 0; c < s->nch; ++c) total += s->ch[c].n;
  int* chv = ialloc(total);
  int* brv = ialloc(total);
  int64_t t = 0;
  for (int c = 0; c < s->nch; ++c)
    for (int b = 0; b < s->ch[c].n; ++b) {
      chv[t] = c;
      brv[t++] = b;
    }
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t it = 0; it < total; ++it) {
    int ch = chv[it], ibra = brv[it];
    const ochan* C = &s->ch[ch];
    int J = ch / 6, nk = C->n;
    double* ZM = Z + s->off2[ch];
    int i = C->p[ibra], j = C->q[ibra];
    int jji = s->j2[i], jjj = s->j2[j];
    int ketmin = hZ == 1 ? ibra : ibra + 1;
    for (int iket = ketmin; iket < nk; ++iket) {
      int k = C->p[iket], l = C->q[iket];
      int jjk = s->j2[k], jjl = s->j2[l];
      double commij = 0, commji = 0;
      int par = (s->l[i] + s->l[l]) % 2;
      int tz = abs(s->tz2[i] - s->tz2[l]) / 2;
      int Jpmin = abs(jji - jjl) / 2, t2 = abs(jjk - jjj) / 2;
      if (t2 > Jpmin) Jpmin = t2;
      int Jpmax = (jji + jjl) / 2;
      t2 = (jjk + jjj) / 2;
      if (t2 < Jpmax) Jpmax = t2;
      for (int Jp = Jpmin; Jp <= Jpmax; ++Jp) {
        double sj = sixj_cached(s, jji, jjj, J, jjk, jjl, Jp);
        if (fabs(sj) < 1e-8) continue;
        int cc = chan_index(Jp, par, tz);
        int ncc = s->cc[cc].n;
        const int* map = s->ccketmap + (size_t)cc * s->nkets;
        int il = map[index2(s, i < l ? i : l, i < l ? l : i)] + (i > l ? ncc : 0);
        int kj = map[index2(s, j < k ? j : k, j < k ? k : j)] + (k > j ? ncc : 0);
        commij -= (2 * Jp + 1) * sj * Zbar[cc][(size_t)kj * ncc + il];
      }
      if (k == l) {
        commji = commij;
      } else if (i == j) {
        commji = iphase((jji + jjj + jjk + jjl) / 2) * commij;
      } else {
        par = (s->l[i] + s->l[k]) % 2;
        tz = abs(s->tz2[i] - s->tz2[k]) / 2;
        Jpmin = abs(jjj - jjl) / 2;
        t2 = abs(jjk - jji) / 2;
        if (t2 > Jpmin) Jpmin = t2;
        Jpmax = (jjj + jjl) / 2;
        t2 = (jjk + jji) / 2;
        if (t2 < Jpmax) Jpmax = t2;
        for (int Jp = Jpmin; Jp <= Jpmax; ++Jp) {
          double sj = sixj_cached(s, jjj, jji, J, jjk, jjl, Jp);
          if (fabs(sj) < 1e-8) continue;
          int cc = chan_index(Jp, par, tz);
          int ncc = s->cc[cc].n;
          const int* map = s->ccketmap + (size_t)cc * s->nkets;
          int ik = map[index2(s, i < k ? i : k, i < k ? k : i)] + (i > k ? ncc : 0);
          int lj = map[index2(s, l < j ? l : j, l < j ? j : l)] + (l > j ? ncc : 0);
          commji -= (2 * Jp + 1) * sj * Zbar[cc][(size_t)lj * ncc + ik];
        }
      }
      int bra_d = (i == j), ket_d = (k == l);
      double norm = bra_d == ket_d ? 1 + bra_d : SQRT2;
      double z = -(commij - iphase((jjk + jjl) / 2 - J) * commji) / norm;
      ZM[(size_t)iket * nk + ibra] += z;
      if (ibra != iket) ZM[(size_t)ibra * nk + iket] += hZ * z;
    }
  }
  free(chv);
  free(brv);
}

/* comm222_phss, src/Commutator.cc:1681-1823 */
void oracle_comm222_phss(const ospace* s, const double* X, const double* Y, double* Z, int hY, int hZ)
{
  double** Zbar = (double**)calloc(s->nch, sizeof(double*));
  for (int c = 0; c < s->nch; ++c) Zbar[c] = dalloc((size_t)s->cc[c].n * 2 * s->cc[c].n);
#pragma omp parallel for schedule(dynamic, 1)
  for (int c = 0; c < s->nch; ++c) {
    const ochan* C = &s->cc[c];
    int ncc = C->n;
    int nph = C->nhh + C->nph;
    if (ncc == 0 || nph == 0) continue;
    int* kph = ialloc(nph);
    for (int t = 0; t < C->nhh; ++t) kph[t] = C->hh[t];
    for (int t = 0; t < C->nph; ++t) kph[C->nhh + t] = C->ph[t];
    double* Xb = dalloc((size_t)ncc * 2 * nph);
    double* Yb = dalloc((size_t)2 * nph * 2 * ncc); /* [Ybar | Ybar_flip] */
    double* Ytmp = dalloc((size_t)2 * nph * ncc);
    pandya_xy(s, X, Y, hY, c, Xb, Ytmp, nph, kph);
    int* phz = ialloc(ncc);
    for (int k = 0; k < ncc; ++k) phz[k] = iphase((s->j2[C->p[k]] + s->j2[C->q[k]]) / 2);
    int K = 2 * nph;
    for (int col = 0; col < ncc; ++col) {
      for (int r = 0; r < K; ++r) Yb[(size_t)col * K + r] = Ytmp[(size_t)col * K + r];
      for (int r = 0; r < nph; ++r) {
        double ph = phz[kph[r]] * phz[col] * hY;
        Yb[(size_t)(ncc + col) * K + r] = Ytmp[(size_t)col * K + nph + r] * ph;
        Yb[(size_t)(ncc + col) * K + nph + r] = Ytmp[(size_t)col * K + r] * ph;
      }
    }
    double* Zb = Zbar[c];
    gemm_nn(s, ncc, 2 * ncc, K, 1.0, Xb, ncc, Yb, K, 0.0, Zb, ncc);
    /* head: += hZ * transpose;  tail: += transpose % PhaseMatZ */
    for (int col = 0; col < ncc; ++col)
      for (int r = col; r < ncc; ++r) {
        double a = Zb[(size_t)col * ncc + r], b = Zb[(size_t)r * ncc + col];
        if (r == col) {
          Zb[(size_t)col * ncc + r] = a + hZ * a;
        } else {
          Zb[(size_t)col * ncc + r] = a + hZ * b;
          Zb[(size_t)r * ncc + col] = b + hZ * a;
        }
        double* tail = Zb + (size_t)ncc * ncc;
        double pm = phz[r] * phz[col];
        a = tail[(size_t)col * ncc + r];
        b = tail[(size_t)r * ncc + col];
        if (r == col) {
          tail[(size_t)col * ncc + r] = a + a * pm;
        } else {
          tail[(size_t)col * ncc + r] = a + b * pm;
          tail[(size_t)r * ncc + col] = b + a * pm;
        }
      }
    free(kph); free(Xb); free(Yb); free(Ytmp); free(phz);
  }
  inverse_pandya(s, Zbar, Z, hZ);
  for (int c = 0; c < s->nch; ++c) free(Zbar[c]);
  free(Zbar);
}

/* --------------------------------------------------------- full commutator */
static int z_herm(int hX, int hY)
{
  if ((hX == 1 && hY == 1) || (hX == -1 && hY == -1)) return -1;
  if ((hX == 1 && hY == -1) || (hX == -1 && hY == 1)) return 1;
  return 0;
}

/* CommutatorScalarScalar, src/Commutator.cc:280-428 (IMSRG(2) part); Z must be zeroed */
void oracle_commutator(const ospace* s, const double* X, const double* Y, double* Z, int hX, int hY)
{
  int hZ = z_herm(hX, hY);
  if (s->term_on[T110]) oracle_comm110ss(s, X, Y, Z, hX, hY);
  if (s->term_on[T220]) oracle_comm220ss(s, X, Y, Z, hX, hY);
  if (s->term_on[T111]) oracle_comm111ss(s, X, Y, Z);
  if (s->term_on[T121]) oracle_comm121ss(s, X, Y, Z, hZ);
  if (s->term_on[T122]) oracle_comm122ss(s, X, Y, Z, hZ);
  if (s->term_on[T222PPHH] || s->term_on[T221])
    oracle_comm222_pp_hh_221ss(s, X, Y, Z, hZ, s->term_on[T222PPHH], s->term_on[T221]);
  if (s->term_on[T222PH]) oracle_comm222_phss(s, X, Y, Z, hY, hZ);
}

/* Operator::Norm for a scalar operator, src/Operator.cc:1610-1651, src/TwoBodyME.cc:703-723 */
double oracle_norm(const ospace* s, const double* A)
{
  int N = s->norb;
  double n1 = 0;
  for (int p = 0; p < N; ++p)
    for (int q = 0; q < N; ++q)
      if (same_1b_channel(s, p, q)) n1 += ONE(A, p, q) * ONE(A, p, q) * (s->j2[p] + 1);
  double n2 = 0;
  for (int c = 0; c < s->nch; ++c) {
    size_t nn = (size_t)s->ch[c].n * s->ch[c].n;
    const double* b = A + s->off2[c];
    double f = 0;
    for (size_t i = 0; i < nn; ++i) f += b[i] * b[i];
    f = sqrt(f) * (2 * (c / 6) + 1);
    n2 += f * f;
  }
  return sqrt(n1 + n2);
}

/* Standard_BCH_Transform, src/BCH.cc:87-201 (no goose-tank / factorized
 * corrections).  Returns the number of nested commutators evaluated. */
int oracle_bch_transform(const ospace* s, const double* OpIn, int hIn, const double* Omega, int hOm, double* OpOut,
                         double threshold)
{
  int64_t A = s->arena;
  double nx = oracle_norm(s, OpIn), ny = oracle_norm(s, Omega);
  memcpy(OpOut, OpIn, A * sizeof(double));
  int iters = 0;
  if (nx > threshold) {
    double* nested = dalloc(A);
    double* next = dalloc(A);
    memcpy(nested, OpOut, A * sizeof(double));
    int hN = hIn;
    double epsilon = nx * exp(-2 * ny) * threshold / (2 * ny);
    double fden = 1.0;
    for (int i = 1; i <= 40; ++i) {
      memset(next, 0, A * sizeof(double));
      oracle_commutator(s, Omega, nested, next, hOm, hN);
      hN = z_herm(hOm, hN);
      double* tmp = nested;
      nested = next;
      next = tmp;
      fden /= i;
      for (int64_t t = 0; t < A; ++t) OpOut[t] += fden * nested[t];
      iters = i;
      epsilon *= i + 1;
      if (oracle_norm(s, nested) < epsilon) break;
    }
    free(nested);
    free(next);
  }
  return iters;
}

/* Commutator::DoPandyaTransformation_SingleChannel, src/Commutator.cc:1319-1390:
 * the Pandya transform of one operator in cross-coupled channel chcc.
 * Bras are the channel's hh then ph kets (a,b) in both orders (rows ibra and
 * ibra + nph), kets (c,d) all of the channel's kets;
 *   Xbar = - sum_J (2J+1) {ja jb Jcc; jc jd J} Z^J_{ad,cb}     (|6j| < 1e-8 skipped)
 * normal orientation: out is 2nph x ncc column-major, out(bra, ket) = Xbar;
 * transpose: out is ncc x 2nph, out(ket, bra) = herm (na - nb) Xbar.
 * Returns nph. */
int oracle_pandya_channel(const ospace* s, const double* Z, int herm, int chcc, int transpose, double* out)
{
  const ochan* K = &s->cc[chcc];
  int ncc = K->n, nph = K->nhh + K->nph;
  int Jcc = chcc / 6;
  for (int ib = 0; ib < nph; ++ib) {
    int kb = ib < K->nhh ? K->hh[ib] : K->ph[ib - K->nhh];
    int pq[2] = {K->p[kb], K->q[kb]};
    for (int ab_case = 0; ab_case <= 1; ++ab_case) {
      int a = pq[ab_case], b = pq[1 - ab_case];
      int row = ib + ab_case * nph;
      double nanb = s->occ[a] - s->occ[b];
      for (int ik = 0; ik < ncc; ++ik) {
        int c = K->p[ik], d = K->q[ik];
        int ja2 = s->j2[a], jb2 = s->j2[b], jc2 = s->j2[c], jd2 = s->j2[d];
        int jmin = abs(ja2 - jd2) > abs(jc2 - jb2) ? abs(ja2 - jd2) / 2 : abs(jc2 - jb2) / 2;
        int jmax = (ja2 + jd2) < (jc2 + jb2) ? (ja2 + jd2) / 2 : (jc2 + jb2) / 2;
        double xbar = 0;
        for (int J = jmin; J <= jmax; ++J) {
          double sixj = sixj_cached(s, ja2, jb2, Jcc, jc2, jd2, J);
          if (fabs(sixj) < 1e-8) continue;
          xbar -= (2 * J + 1) * sixj * tbme_J(s, Z, J, a, d, c, b);
        }
        if (transpose)
          out[(size_t)row * ncc + ik] = herm * xbar * nanb;
        else
          out[(size_t)ik * 2 * nph + row] = xbar;
      }
    }
  }
  return nph;
}

/* BCH::BCH_Product, src/BCH.cc:267-350: Z with e^Z = e^X e^Y,
 *   Z = X + Y + 1/2 [X,Y] + 1/12 ([X,[X,Y]] + [Y,[Y,X]]) - 1/720 [Y,[Y,[Y,[Y,X]]]] + ...
 * with the Bernoulli coefficients of src/BCH.cc:273-274, the [X,[X,Y]] term
 * only when |[Y,X]| |X| exceeds the threshold (:289-292), and the loop stops of
 * :304-335 (the factorized correction, off by default, is not restated).
 * Z must not alias X or Y and is overwritten.  Returns the number of
 * commutators evaluated. */
int oracle_bch_product(const ospace* s, const double* X, int hX, const double* Y, int hY, double* Z,
                       double threshold)
{
  static const double bern[9] = {1.0, -0.5, 1. / 6, 0.0, -1. / 30, 0.0, 1. / 42, 0, -1. / 30};
  static const double fact[9] = {1.0, 1.0, 2.0, 6.0, 24., 120., 720., 5040., 40320.};
  int64_t A = s->arena;
  double nx = oracle_norm(s, X), ny = oracle_norm(s, Y);
  for (int64_t t = 0; t < A; ++t) Z[t] = X[t] + Y[t];
  double* nested = dalloc(A);
  double* next = dalloc(A);
  oracle_commutator(s, Y, X, nested, hY, hX);
  int hN = z_herm(hY, hX);
  int ncomm = 1;
  double nxy = oracle_norm(s, nested);
  if (nxy * nx > threshold) {
    oracle_commutator(s, nested, X, next, hN, hX);
    ++ncomm;
    for (int64_t t = 0; t < A; ++t) Z[t] += (1. / 12) * next[t];
  }
  size_t k = 1;
  while (nxy > threshold) {
    if (k < 2 || k % 2 == 0) {
      double c = bern[k] / fact[k];
      for (int64_t t = 0; t < A; ++t) Z[t] += c * nested[t];
    }
    ++k;
    if (k >= 9) break;
    if (2 * ny * nxy < threshold) break;
    memset(next, 0, A * sizeof(double));
    oracle_commutator(s, Y, nested, next, hY, hN);
    hN = z_herm(hY, hN);
    double* tmp = nested;
    nested = next;
    next = tmp;
    ++ncomm;
    nxy = oracle_norm(s, nested);
  }
  free(nested);
  free(next);
  return ncomm;
}

/* ------------------------------------------------------------- generator */
/* Generator types (src/Generator.cc:12-15) and denominator partitionings
 * (src/Generator.cc:23-28) restated here. */
enum { GEN_WHITE = 0, GEN_ATAN = 1, GEN_WEGNER = 2, GEN_IMAGTIME = 3 };
enum { PART_EPSTEIN_NESBET = 0, PART_MOLLER_PLESSET = 1 };
#define DELTA_ALL (-12345)

static double eta_func(int type, double hod, double den)
{
  switch (type) {
    case GEN_ATAN: return 0.5 * atan(2 * hod / den);
    case GEN_WEGNER: return hod * den;
    case GEN_IMAGTIME: return hod * ((den > 0) - (den < 0));
    default: return hod / den;
  }
}

/* Generator::Get1bDenominator, src/Generator.cc:110-139 */
static double denom_1b(const ospace* s, const double* H, int part, double cutoff, double delta, int delta_index,
                       int i, int j)
{
  int N = s->norb;
  double d = ONE(H, i, i) - ONE(H, j, j);
  if (part == PART_EPSTEIN_NESBET) d += (s->occ[i] - s->occ[j]) * tbme_monopole(s, H, i, j, i, j);
  if (delta_index == DELTA_ALL || i == delta_index || j == delta_index) d += delta;
  if (fabs(d) < cutoff) d = cutoff;
  return d;
}

/* Generator::Get2bDenominator, src/Generator.cc:142-188, bra (i,j), ket (k,l) */
static double denom_2b(const ospace* s, const double* H, int part, double cutoff, double delta, int delta_index,
                       int i, int j, int k, int l)
{
  int N = s->norb;
  double d = ONE(H, i, i) + ONE(H, j, j) - ONE(H, k, k) - ONE(H, l, l);
  if (delta_index == DELTA_ALL) d += delta;
  double ni = s->occ[i], nj = s->occ[j], nk = s->occ[k], nl = s->occ[l];
  if (part == PART_EPSTEIN_NESBET) {
    d += (1 - ni - nj) * tbme_monopole(s, H, i, j, i, j);
    d -= (1 - nk - nl) * tbme_monopole(s, H, k, l, k, l);
    d += (ni - nk) * tbme_monopole(s, H, i, k, i, k);
    d += (ni - nl) * tbme_monopole(s, H, i, l, i, l);
    d += (nj - nk) * tbme_monopole(s, H, j, k, j, k);
    d += (nj - nl) * tbme_monopole(s, H, j, l, j, l);
  }
  if (fabs(d) < cutoff) d = cutoff;
  return d;
}

/* Generator::Update -> ConstructGenerator_SingleRef, src/Generator.cc:32-76,
 * 236-297, for a single-reference space: the core is the set of occupied
 * orbits (src/ModelSpace.cc:278-280: the reference's own filling), every other
 * orbit is in the q space.  Eta is overwritten: zero except the 1b ph block
 * (core a, non-core i) and the 2b blocks <pp'|Eta|hh'> with both bra orbits
 * outside and both ket orbits inside the core, antisymmetrised. */
void oracle_generator(const ospace* s, const double* H, double* Eta, int type, int part, double cutoff, double delta,
                      int delta_index)
{
  int N = s->norb;
  memset(Eta, 0, s->arena * sizeof(double));
  for (int ia = 0; ia < s->nholes; ++ia) {
    int a = s->holes[ia];
    for (int i = 0; i < N; ++i) {
      if (s->occ[i] >= OCC_CUT) continue;
      double d = denom_1b(s, H, part, cutoff, delta, delta_index, i, a);
      double e = eta_func(type, ONE(H, i, a), d);
      ONE(Eta, i, a) = e;
      ONE(Eta, a, i) = -e;
    }
  }
#pragma omp parallel for schedule(dynamic, 1)
  for (int c = 0; c < s->nch; ++c) {
    const ochan* C = &s->ch[c];
    int n = C->n;
    const double* H2 = H + s->off2[c];
    double* E2 = Eta + s->off2[c];
    for (int ik = 0; ik < n; ++ik) {
      int k = C->p[ik], l = C->q[ik];
      if (s->occ[k] < OCC_CUT || s->occ[l] < OCC_CUT) continue;
      for (int ib = 0; ib < n; ++ib) {
        int i = C->p[ib], j = C->q[ib];
        if (s->occ[i] >= OCC_CUT || s->occ[j] >= OCC_CUT) continue;
        double d = denom_2b(s, H, part, cutoff, delta, delta_index, i, j, k, l);
        double e = eta_func(type, H2[(size_t)ik * n + ib], d);
        E2[(size_t)ik * n + ib] = e;
        E2[(size_t)ib * n + ik] = -e;
      }
    }
  }
}

/* ---------------------------------------------------------------- solver */
/* IMSRGSolver settings (src/IMSRGSolver.cc:31-37, src/IMSRGSolver.hh:117-148,
 * src/BCH.cc:16-17, src/Generator.cc:18-20). */
typedef struct {
  double ds, ds_max, smax, norm_domega, omega_norm_max, eta_criterion;
  int magnus_adaptive;
  int generator, partitioning;
  double denominator_cutoff, denominator_delta;
  int denominator_delta_index;
  double bch_transform_threshold, bch_product_threshold;
} oflow_params;

/* IMSRGSolver::Solve_magnus_euler, src/IMSRGSolver.cc:236-321, with
 * IMSRGSolver::NewOmega (src/IMSRGSolver.cc:44-83) for Omega splitting
 * (no scratch files: the earlier Omegas are not kept).  Starts from s = *s_io
 * and the flowing state Hs (H(s)), Omega (the last Omega), Hsaved (the
 * starting point of that Omega; equal to H0 while only one Omega exists) and
 * *n_omega (Omegas so far, >= 1).  Per step, the flow parameter and
 * H(s).ZeroBody are appended to s_hist / e0_hist (up to maxhist entries).
 * Returns the number of steps taken, or -1 if the flow blew up (the
 * reference's "things are clearly broken" exit, :263-270). */
int oracle_magnus_euler(const ospace* s, const double* H0, double* Hs, double* Hsaved, double* Omega, double* Eta,
                        const oflow_params* p, double* s_io, int* n_omega, double* s_hist, double* e0_hist,
                        int maxhist)
{
  int64_t A = s->arena;
  double sflow = *s_io;
  double ds = p->ds;
  double norm_domega = p->norm_domega;
  oracle_generator(s, Hs, Eta, p->generator, p->partitioning, p->denominator_cutoff, p->denominator_delta,
                   p->denominator_delta_index);
  if (fabs(p->omega_norm_max - norm_domega) < 1e-6) norm_domega += 1e-4;
  double Elast = H0[0];
  double* om = dalloc(A);
  int steps = 0;
  for (int istep = 1; sflow < p->smax; ++istep) {
    double norm_eta = oracle_norm(s, Eta);
    if (norm_eta < p->eta_criterion) break;
    if (norm_eta > 1e12 || fabs(Elast) > 1e9) {
      free(om);
      *s_io = sflow;
      return -1;
    }
    double norm_omega = oracle_norm(s, Omega);
    if (norm_omega > p->omega_norm_max) {
      memcpy(Hsaved, Hs, A * sizeof(double));
      memset(Omega, 0, A * sizeof(double));
      ++*n_omega;
      norm_omega = 0;
    }
    if (p->magnus_adaptive) {
      double a = norm_domega / norm_eta;
      double b = norm_domega / norm_eta / (norm_omega + 1.0e-9);
      double c = (p->omega_norm_max + 1e-5) / norm_eta;
      ds = a;
      if (b < ds) ds = b;
      if (c < ds) ds = c;
      if (p->ds_max < ds) ds = p->ds_max;
    }
    if (p->smax - sflow < ds) ds = p->smax - sflow;
    sflow += ds;
    for (int64_t t = 0; t < A; ++t) Eta[t] *= ds;
    oracle_bch_product(s, Eta, -1, Omega, -1, om, p->bch_product_threshold);
    memcpy(Omega, om, A * sizeof(double));
    oracle_bch_transform(s, *n_omega < 2 ? H0 : Hsaved, 1, Omega, -1, Hs, p->bch_transform_threshold);
    oracle_generator(s, Hs, Eta, p->generator, p->partitioning, p->denominator_cutoff, p->denominator_delta,
                     p->denominator_delta_index);
    Elast = Hs[0];
    if (steps < maxhist) {
      s_hist[steps] = sflow;
      e0_hist[steps] = Hs[0];
    }
    ++steps;
  }
  free(om);
  *s_io = sflow;
  return steps;
}

int oracle_num_threads(void)
{
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
