// Device view of a model space: flat tables the kernels read, passed by value.
#pragma once

#include <cstdint>

#include <vector_types.h>

#ifdef __CUDACC__
#define IMSRG_HD __host__ __device__ __forceinline__
#else
#define IMSRG_HD inline
#endif

namespace imsrg {

struct DevSpace {
  int norb, nch, nkets, NJ, d1;
  const int* l;
  const int* j2;
  const int* tz2;
  const double* occ;
  const int* ob_start;  // one-body channel of each orbit: ob_list[ob_start[i] .. +ob_count[i])
  const int* ob_count;
  const int* ob_list;
  const int* ketJ_loc;  // [J * nkets + ket] -> local index in the 2b channel (J, parity, Tz of the ket)
  const int* ccJ_loc;   // [J * nkets + ket] -> local index in the CC channel (J, parity, |dTz|)
  const int* ch_n;      // kets per 2b channel
  const long long* ch_off;  // arena offset per 2b channel
  const int* ch_kofs;   // start of the channel's kets in ket_p / ket_q
  const int* ket_p;
  const int* ket_q;
  const int* cc_n;
  const int* cc_kofs;
  const int* cc_p;
  const int* cc_q;
  const int* sixj_base;  // [((a*d1+b)*d1+c)*d1+d] -> offset into sixj_val
  const double* sixj_val;
  // (2 J6 + 1) {...}, exactly 0 where |{...}| < 1e-8: the weight of every
  // Pandya recoupling sum (both cut and factor are the reference's,
  // src/Commutator.cc:1456-1462, 1579-1583)
  const double* sixj_wval;
  // the same weights as (hi, lo) float pairs, hi + lo = weight to 2^-48
  const float2* sixj_wf;
};

// Device copies of the per-kernel work lists (built once per space).
// One output of the Pandya transform of X and Y (an (ik, t) element of the
// Xbar / Ybar panels of a cross-coupled channel), from per-space descriptors:
// its terms pf_e[beg .. beg+nterm) (arena indices) and pf_w (the signed
// (2J+1) 6j weights), its panel position and factors.
struct PfOut {
  int dest;        // Xbar / YbarT element (into the panel arrays)
  int dyf;         // YflipT element - dest
  int beg;
  unsigned code;   // nterm | (factors of sqrt 2 in normfactor) << 16 | (phi_bra phi_ik < 0) << 18
  double xs;       // normfactor * (n_a - n_b)
};

struct DevWork {
  const double* ket_wpp;  // flat over 2b channel kets (ch_kofs order)
  const double* ket_nn;
  const int* hh_off;      // per channel, into hh_list
  const int* hh_list;
  const int* items220; int n220;
  const int* pairs1b; int npairs1b;
  const int* items221; int n221;
  const int* cols122; int ncols122;
  const int* it122_loc;
  const int* it122_a;
  const int* it122_src;
  const double* it122_f;
  const int* kidx;        // ladder gather lists
  const double* kweight;
  const int* phase_tab;
  const int* cc_nph;      // Pandya
  const int* cc_ph_off;
  const int* cc_ph;
  const long long* xb_off;
  const long long* zb_off;
  const int* cc_phase_off;
  const PfOut* pf_out; int n_pfout;  // Pandya transform of X and Y, from descriptors
  const int* pf_e;
  const double* pf_w;
  const float2* pf_wf;  // pf_w as (hi, lo) float pairs (the split form's double-float sums)
};

// global index of ket (p, q), p <= q: ModelSpace::Index2 (src/ModelSpace.cc:1108-1118)
IMSRG_HD int ket_index(int norb, int p, int q) { return p * (2 * norb - 1 - p) / 2 + q; }

IMSRG_HD int chan_index(int J, int parity, int Tz) { return 6 * J + 2 * (Tz + 1) + parity; }

IMSRG_HD int iphase(int x) { return (x & 1) ? -1 : 1; }

// compact 6j lookup {jj1/2 jj2/2 J3; jj4/2 jj5/2 J6}; 0 outside the triads
IMSRG_HD int sixj_slot(int d1, const int* base, int jj1, int jj2, int J3, int jj4, int jj5, int J6)
{
  int J3min = (jj1 > jj2 ? jj1 - jj2 : jj2 - jj1) >> 1, J3max = (jj1 + jj2) >> 1;
  int t1 = jj1 > jj5 ? jj1 - jj5 : jj5 - jj1, t2 = jj4 > jj2 ? jj4 - jj2 : jj2 - jj4;
  int J6min = (t1 > t2 ? t1 : t2) >> 1;
  int s1 = jj1 + jj5, s2 = jj4 + jj2;
  int J6max = (s1 < s2 ? s1 : s2) >> 1;
  if (J3 < J3min || J3 > J3max || J6 < J6min || J6 > J6max) return -1;
  int a = (jj1 - 1) >> 1, b = (jj2 - 1) >> 1, c = (jj4 - 1) >> 1, d = (jj5 - 1) >> 1;
  return base[((a * d1 + b) * d1 + c) * d1 + d] + (J3 - J3min) * (J6max - J6min + 1) + (J6 - J6min);
}

// Inverse Pandya transform by orbit quadruple (i, j, k, l), bra (i, j), ket
// (k, l), i <= j, k <= l, (i, j) <= (k, l): the quadruple's element lives in every
// channel J of [Jlo, Jhi] (even J only when i == j or k == l), its first J'
// sum has n1 terms (J' from lo1), its second n2 (from lo2; none when i == j or
// k == l).  Returns false when the quadruple contributes nothing: an empty J
// window, the lower triangle (i == k, j > l), or the diagonal of an
// anti-hermitian Z (src/Commutator.cc:1541, 1559-1560, 1588-1589).
constexpr int kInvqMaxOrb = 64;  // orbits of one (parity, Tz) class in a block
constexpr int kInvqMaxJ = 32;    // J (or J') values one block spans: 2 j_max + 1 < 32

IMSRG_HD bool invq_counts(int i, int j, int k, int l, int ji, int jj, int jk, int jl, int hZ, int& n1, int& n2,
                          int& nJ, int& Jlo, int& lo1, int& lo2)
{
  n1 = n2 = nJ = 0;
  Jlo = lo1 = lo2 = 0;
  if (i == k && (j > l || (hZ < 0 && j == l))) return false;
  int a = ji > jj ? ji - jj : jj - ji, b = jk > jl ? jk - jl : jl - jk;
  int lo = (a > b ? a : b) >> 1;
  int hi = ((ji + jj) < (jk + jl) ? ji + jj : jk + jl) >> 1;
  const bool ev = (i == j) || (k == l);
  if (ev) lo += lo & 1;
  if (lo > hi) return false;
  nJ = ev ? ((hi - lo) >> 1) + 1 : hi - lo + 1;
  Jlo = lo;
  a = ji > jl ? ji - jl : jl - ji;
  b = jk > jj ? jk - jj : jj - jk;
  lo1 = (a > b ? a : b) >> 1;
  int h1 = ((ji + jl) < (jk + jj) ? ji + jl : jk + jj) >> 1;
  n1 = h1 >= lo1 ? h1 - lo1 + 1 : 0;
  if (!ev) {
    a = jj > jl ? jj - jl : jl - jj;
    b = jk > ji ? jk - ji : ji - jk;
    lo2 = (a > b ? a : b) >> 1;
    int h2 = ((jj + jl) < (jk + ji) ? jj + jl : jk + ji) >> 1;
    n2 = h2 >= lo2 ? h2 - lo2 + 1 : 0;
  }
  return true;
}

#ifdef __CUDACC__
__device__ __forceinline__ double dev_sixj(const DevSpace& S, int jj1, int jj2, int J3, int jj4, int jj5, int J6)
{
  int s = sixj_slot(S.d1, S.sixj_base, jj1, jj2, J3, jj4, jj5, J6);
  return s < 0 ? 0.0 : __ldg(S.sixj_val + s);
}

// (2 J6 + 1) {jj1/2 jj2/2 J3; jj4/2 jj5/2 J6}, 0 when the reference skips it
__device__ __forceinline__ double dev_sixj_w(const DevSpace& S, int jj1, int jj2, int J3, int jj4, int jj5, int J6)
{
  int s = sixj_slot(S.d1, S.sixj_base, jj1, jj2, J3, jj4, jj5, J6);
  return s < 0 ? 0.0 : __ldg(S.sixj_wval + s);
}

__device__ __forceinline__ bool dzero(double v) { return (__double_as_longlong(v) << 1) == 0; }
__device__ __forceinline__ double dneg_if(double v, bool neg)
{
  return __longlong_as_double(__double_as_longlong(v) ^ (neg ? (long long)0x8000000000000000ull : 0ll));
}

// Normalised J-coupled matrix element of a scalar operator arena, with the
// swap phases of TwoBodyME::GetTBME_J_norm (src/TwoBodyME.cc:132-153,339-356).
__device__ __forceinline__ double dev_tbme_J_norm(const DevSpace& S, const double* op, int J, int a, int b, int c,
                                                  int d)
{
  int la = __ldg(S.l + a), lb = __ldg(S.l + b), lc = __ldg(S.l + c), ld = __ldg(S.l + d);
  int ta = __ldg(S.tz2 + a), tb = __ldg(S.tz2 + b), tc = __ldg(S.tz2 + c), td = __ldg(S.tz2 + d);
  if (((la + lb + lc + ld) & 1) || (ta + tb != tc + td)) return 0.0;
  int kb = ket_index(S.norb, a < b ? a : b, a < b ? b : a);
  int kk = ket_index(S.norb, c < d ? c : d, c < d ? d : c);
  if (J >= S.NJ) return 0.0;
  int bi = __ldg(S.ketJ_loc + J * S.nkets + kb);
  int ki = __ldg(S.ketJ_loc + J * S.nkets + kk);
  if (bi < 0 || ki < 0) return 0.0;
  int ch = chan_index(J, (la + lb) & 1, (ta + tb) / 2);
  int n = __ldg(S.ch_n + ch);
  double ph = 1.0;
  if (a > b) ph *= iphase(((__ldg(S.j2 + a) + __ldg(S.j2 + b)) >> 1) + 1 + J);
  if (c > d) ph *= iphase(((__ldg(S.j2 + c) + __ldg(S.j2 + d)) >> 1) + 1 + J);
  return ph * op[__ldg(S.ch_off + ch) + (long long)ki * n + bi];
}
#endif

}  // namespace imsrg
