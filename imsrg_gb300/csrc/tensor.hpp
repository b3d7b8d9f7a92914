// Reduced tensor operators of rank (lambda, |delta Tz|, parity): the arena
// layout of their two-body blocks, the angular-momentum tables the
// scalar-tensor commutator needs (6j symbols with three integer and three
// half-integer arguments, 6j symbols with the half-integer range widened by
// lambda, and 9j symbols built from them), and the device view of all of it.
#pragma once

#include <cstdint>
#include <map>
#include <vector>

#include "devspace.cuh"

namespace imsrg {

struct Space;

// Device view of one tensor layout.  Arena of a tensor operator: ZeroBody at
// [0], OneBody N x N column-major at [32], then block b = (ch_bra[b] <=
// ch_ket[b]) as n_bra x n_ket column-major at off[b] (a multiple of 32), in
// TwoBodyME::Allocate order (src/TwoBodyME.cc:77-95).
struct DevTensor {
  int lam = 0, trank = 0, parity = 0, nblk = 0;
  long long total = 0;
  const int* bra = nullptr;
  const int* ket = nullptr;
  const long long* off = nullptr;
  const int* lookup = nullptr;  // [ch_bra * nch + ch_ket] -> block, -1 (ch_bra <= ch_ket)
  const unsigned char* ob_ok = nullptr;  // [i * N + j]: <i||T||j> allowed
  // 6j {I1 I2 lam; h1 h2 h3} for I1, I2 < NJ and doubled half-integers
  // 2h + 1 <= 2 d1x - 1: [(((I1 * NJ + I2) * d1x + a) * d1x + b) * d1x + c]
  const double* sixjA = nullptr;
  // 6j {h1 h2 I3; h4 h5 I6} with the compact layout of the space's table,
  // half-integers up to 2 d1x - 1 (the 9j sums reach j + lambda)
  const int* sixjx_base = nullptr;
  const double* sixjx_val = nullptr;
  int NJ = 0, d1x = 0;
  // comm222_phst: cross-coupled channel pairs (lo <= hi) of Zbar, n_lo x
  // 2 n_hi column-major at zb_off; and the ordered pairs (bra, ket) of the
  // tensor Pandya transform of Y, 2 nph_bra x n_ket column-major at yb_off
  int nzb = 0, nyb = 0;
  const int* zb_bra = nullptr;
  const int* zb_ket = nullptr;
  const long long* zb_off = nullptr;
  const long long* zb_lookup = nullptr;  // [lo * nch + hi] -> offset, -1
  const int* yb_bra = nullptr;
  const int* yb_ket = nullptr;
  const long long* yb_off = nullptr;
  const long long* yb_lookup = nullptr;  // [bra * nch + ket] -> offset, -1
  long long zb_total = 0, yb_total = 0;
  // tabulated 9j {ja jd J1; jb jc J2; Jbra Jket lam} for orbit j's (extent
  // d1): nj_base[((a d1 + b) d1 + c) d1 + d] starts an (nJ1, 2 lam + 1, nJbra,
  // 2 lam + 1) block over J1 in [|ja-jd|, ja+jd], J2 = J1 - lam + o2, Jbra in
  // [|ja-jb|, ja+jb], Jket = Jbra - lam + o4 (see ninej_slot).  nj_val holds
  // the 9j (host view only); nj_hat the 9j times sqrt((2J1+1)(2J2+1)(2Jbra+1)
  // (2Jket+1)), exactly 0 where |9j| < 1e-8 (the kernels' skip rule)
  const long long* nj_base = nullptr;
  const double* nj_val = nullptr;
  const double* nj_hat = nullptr;
  int d1 = 0;
  const double* hat2 = nullptr;  // [J1 * NJ + J2] = sqrt((2J1+1)(2J2+1))
  // per orbit i: the orbits j with <i||T||j> allowed (tob_list[tob_off[i] ..
  // tob_off[i + 1]))
  const int* tob_off = nullptr;
  const int* tob_list = nullptr;
  // per two-body channel: the ladder gather list (its start in the space's
  // kidx / kweight tables and its length, 0 when empty)
  const int* lad_koff = nullptr;
  const int* lad_woff = nullptr;
  const int* lad_n = nullptr;
};

struct SplitPlan;

struct TensorLayout {
  int lam = 0, trank = 0, parity = 0;
  std::vector<int> bra, ket, lookup;
  std::vector<int64_t> off;
  int64_t total = 0;
  std::vector<unsigned char> ob_ok;
  std::vector<double> sixjA;
  std::vector<int> sixjx_base;
  std::vector<double> sixjx_val;
  int NJ = 0, d1x = 0;
  std::vector<int> zb_bra, zb_ket, yb_bra, yb_ket;
  std::vector<int64_t> zb_off, yb_off, zb_lookup, yb_lookup;
  std::vector<long long> nj_base;
  std::vector<double> nj_val, nj_hat;
  int nj_d1 = 0;  // orbit j extent of the 9j table
  std::vector<double> hat2;
  std::vector<int> lad_koff, lad_woff, lad_n;
  std::vector<int> tob_off, tob_list;
  int max_ob = 0, max_tob = 0;  // longest one-body partner list (scalar, tensor) of an orbit
  // Operator::Norm of a tensor (src/Operator.cc:1610-1646, src/TwoBodyME.cc:
  // 703-725): the one-body elements with their degeneracy weights, and every
  // stored block in chunks with its weight (degeneracy^2, doubled when the
  // bra and ket channels differ)
  std::vector<int> nrm1_idx;
  std::vector<double> nrm1_w;
  std::vector<long long> nrm2_off;
  std::vector<int> nrm2_len;
  std::vector<double> nrm2_w;
  int* d_nrm1_idx = nullptr;
  double* d_nrm1_w = nullptr;
  long long* d_nrm2_off = nullptr;
  int* d_nrm2_len = nullptr;
  double *d_nrm2_w = nullptr, *d_nrm_partial = nullptr;
  std::vector<double> h_nrm_partial;
  // BCH_Transform's work operators of this rank (layout total each)
  double *d_bch_nested = nullptr, *d_bch_next = nullptr;
  long long lad_maxelems = 0;  // largest n_channel x gather length (grid sizing)
  int64_t zb_total = 0, yb_total = 0;
  int zb_maxelems = 0, yb_maxelems = 0;  // largest block of each list (grid sizing)
  int max_blk_elems = 0;                 // largest two-body block of the layout
  long long max_pair_elems = 0;          // largest n_bra x ceil(n_ket / 2) (column pairs)
  // scratch of the scalar-tensor commutator (device, lazily allocated):
  // Mpp - Mhh, Mhh (layout total), X bar (the space's xb_total), Y bar, Z bar,
  // and the two weighted copies of X the ladder reads (the space's arena each)
  double *d_mpp = nullptr, *d_mhh = nullptr, *d_xbar = nullptr, *d_ybar = nullptr, *d_zbar = nullptr;
  double *d_xw = nullptr, *d_wx = nullptr;
  // split form (lazily built): Y with every block transposed (layout total),
  // the tensor Pandya panels transposed and their half-swapped copies (yb_total
  // each), X bar's half-swapped copy (the space's xb_total), and the product
  // plans: ladder D = Xb w Yc (overwrite) and D -= Yc w Xk (accumulate), Z bar
  // first K half (overwrite) and second K half (accumulate)
  double *d_yt = nullptr, *d_ybt = nullptr, *d_ybtf = nullptr, *d_xbf = nullptr;
  SplitPlan *sp_lad1 = nullptr, *sp_lad2 = nullptr, *sp_zb1 = nullptr, *sp_zb2 = nullptr;
  int max_tiles32 = 0;        // largest block in 32 x 32 tiles (transpose grid)
  // orbit quadruples of the inverse tensor Pandya transform: (i | j << 16,
  // k | l << 16) for every bra ket i <= j and ket ket k <= l that own at
  // least one stored element, ordered by the class (ji, jj, jk, jl)
  std::vector<int2> tq;
  int tq_max_j3 = 0;          // largest J3 (or J1) range of a quadruple
  int2* d_tq = nullptr;
  long long max_xbf = 0;      // largest X bar panel (2 nph x n_cc)
  DevTensor dev;
  bool dev_ready = false;
  std::vector<void*> dev_allocs;
  ~TensorLayout();
};

// the space's layout of rank (lam, trank, parity), built on first use
// (host tables only; tensor_upload copies them to the device)
TensorLayout* tensor_layout(Space& s, int lam, int trank, int parity);
void tensor_upload(TensorLayout& t);
// the same view with host pointers (host-side 9j and 6j evaluation)
DevTensor tensor_host_view(const TensorLayout& t);

IMSRG_HD int sixjA_index(int NJ, int d1x, int I1, int I2, int jj1, int jj2, int jj3)
{
  if (I1 < 0 || I2 < 0 || I1 >= NJ || I2 >= NJ) return -1;
  if (jj1 < 1 || jj2 < 1 || jj3 < 1) return -1;
  int a = (jj1 - 1) >> 1, b = (jj2 - 1) >> 1, c = (jj3 - 1) >> 1;
  if (a >= d1x || b >= d1x || c >= d1x) return -1;
  return (((I1 * NJ + I2) * d1x + a) * d1x + b) * d1x + c;
}

// {I1 I2 lam; jj1/2 jj2/2 jj3/2}
IMSRG_HD double sixjA_get(const double* tab, int NJ, int d1x, int I1, int I2, int jj1, int jj2, int jj3)
{
  int k = sixjA_index(NJ, d1x, I1, I2, jj1, jj2, jj3);
  return k < 0 ? 0.0 : tab[k];
}

// {jj1/2 jj2/2 J3; jj4/2 jj5/2 J6} from a compact table of extent d1
IMSRG_HD double sixj_compact_get(const int* base, const double* val, int d1, int jj1, int jj2, int J3, int jj4,
                                 int jj5, int J6)
{
  if (jj1 < 1 || jj2 < 1 || jj4 < 1 || jj5 < 1) return 0.0;
  if (((jj1 - 1) >> 1) >= d1 || ((jj2 - 1) >> 1) >= d1 || ((jj4 - 1) >> 1) >= d1 || ((jj5 - 1) >> 1) >= d1)
    return 0.0;
  int s = sixj_slot(d1, base, jj1, jj2, J3, jj4, jj5, J6);
  return s < 0 ? 0.0 : val[s];
}

// 9j {ja/2 jd/2 J1; jb/2 jc/2 J2; Jbra Jket lam} for half-integer ja..jd and
// integer J1, J2, Jbra, Jket, as the sum over x of three 6j symbols
// (Edmonds, "Angular Momentum in Quantum Mechanics", eq. 6.4.3):
//   {j1 j2 j3; j4 j5 j6; j7 j8 j9} = sum_x (-1)^(2x) (2x+1)
//       {j1 j4 j7; j8 j9 x} {j2 j5 j8; j4 x j6} {j3 j6 j9; x j1 j2}
// with {ja jb Jbra; Jket lam x} = {Jket Jbra lam; ja x jb} and
// {J1 J2 lam; x ja jd} read from the integer-row table, and
// {jd jc Jket; jb x J2} from the widened compact table.
IMSRG_HD double ninej_tensor(const DevTensor& T, int lam, int ja, int jb, int jc, int jd, int J1, int J2, int Jbra,
                             int Jket)
{
  int xlo = ja > 2 * lam ? ja - 2 * lam : 2 * lam - ja;  // doubled x: |ja - lam| .. ja + lam
  int xhi = ja + 2 * lam;
  double s = 0.0;
  for (int x = xlo; x <= xhi; x += 2) {
    double a = sixjA_get(T.sixjA, T.NJ, T.d1x, Jket, Jbra, ja, x, jb);
    if (a == 0.0) continue;
    double b = sixj_compact_get(T.sixjx_base, T.sixjx_val, T.d1x, jd, jc, Jket, jb, x, J2);
    if (b == 0.0) continue;
    double c = sixjA_get(T.sixjA, T.NJ, T.d1x, J1, J2, x, ja, jd);
    s -= (x + 1) * a * b * c;  // (-1)^(2x) = -1 for half-integer x
  }
  return s;
}

// slot of {ja jd J1; jb jc J2; Jbra Jket lam} in the 9j tables, -1 outside
// their windows
IMSRG_HD long long ninej_slot(const DevTensor& T, int ja, int jb, int jc, int jd, int J1, int J2, int Jbra, int Jket)
{
  const int d1 = T.d1, L = T.lam, w = 2 * L + 1;
  const int a = (ja - 1) >> 1, b = (jb - 1) >> 1, c = (jc - 1) >> 1, d = (jd - 1) >> 1;
  if (a < 0 || b < 0 || c < 0 || d < 0 || a >= d1 || b >= d1 || c >= d1 || d >= d1) return -1;
  const int J1min = (ja > jd ? ja - jd : jd - ja) >> 1, J1max = (ja + jd) >> 1;
  const int Jbmin = (ja > jb ? ja - jb : jb - ja) >> 1, Jbmax = (ja + jb) >> 1;
  const int o2 = J2 - J1 + L, o4 = Jket - Jbra + L;
  if (J1 < J1min || J1 > J1max || Jbra < Jbmin || Jbra > Jbmax || o2 < 0 || o2 >= w || o4 < 0 || o4 >= w) return -1;
  const int nJb = Jbmax - Jbmin + 1;
  return T.nj_base[((a * d1 + b) * d1 + c) * d1 + d] +
         (((long long)(J1 - J1min) * w + o2) * nJb + (Jbra - Jbmin)) * w + o4;
}

// the tabulated 9j (the same value as ninej_tensor), 0 outside its windows
IMSRG_HD double ninej_get(const DevTensor& T, int ja, int jb, int jc, int jd, int J1, int J2, int Jbra, int Jket)
{
  const long long k = ninej_slot(T, ja, jb, jc, jd, J1, J2, Jbra, Jket);
  return k < 0 ? 0.0 : T.nj_val[k];
}

// the hat-weighted 9j of fixed (ja, jb, jc, jd, Jbra, Jket) as a function of
// (J1, J2): one row of the table, read with one load per (J1, J2)
struct NineJRow {
  const double* p = nullptr;  // slot of (J1min, o2 = 0)
  long long stride = 0;       // between consecutive (J1, o2) slots
  int J1min = 0, J1max = -1, w = 0, L = 0;
  IMSRG_HD long long slot(int J1, int J2) const
  {
    const int o2 = J2 - J1 + L;
    if (!p || J1 < J1min || J1 > J1max || o2 < 0 || o2 >= w) return -1;
    return ((long long)(J1 - J1min) * w + o2) * stride;
  }
  IMSRG_HD double get(int J1, int J2) const
  {
    const long long k = slot(J1, J2);
    return k < 0 ? 0.0 : p[k];
  }
};

IMSRG_HD NineJRow ninej_row(const DevTensor& T, int ja, int jb, int jc, int jd, int Jbra, int Jket)
{
  NineJRow r;
  const int d1 = T.d1, L = T.lam, w = 2 * L + 1;
  const int a = (ja - 1) >> 1, b = (jb - 1) >> 1, c = (jc - 1) >> 1, d = (jd - 1) >> 1;
  if (a < 0 || b < 0 || c < 0 || d < 0 || a >= d1 || b >= d1 || c >= d1 || d >= d1) return r;
  const int Jbmin = (ja > jb ? ja - jb : jb - ja) >> 1, Jbmax = (ja + jb) >> 1;
  const int o4 = Jket - Jbra + L;
  if (Jbra < Jbmin || Jbra > Jbmax || o4 < 0 || o4 >= w) return r;
  const int nJb = Jbmax - Jbmin + 1;
  const long long o = T.nj_base[((a * d1 + b) * d1 + c) * d1 + d] + (long long)(Jbra - Jbmin) * w + o4;
  r.p = T.nj_hat + o;
  r.stride = (long long)nJb * w;
  r.J1min = (ja > jd ? ja - jd : jd - ja) >> 1;
  r.J1max = (ja + jd) >> 1;
  r.w = w;
  r.L = L;
  return r;
}

// hat-weighted 9j: sqrt((2J1+1)(2J2+1)(2Jbra+1)(2Jket+1)) {ja jd J1; jb jc J2;
// Jbra Jket lam}, 0 where |9j| < 1e-8 or outside the windows
IMSRG_HD double ninej_hat(const DevTensor& T, int ja, int jb, int jc, int jd, int J1, int J2, int Jbra, int Jket)
{
  const long long k = ninej_slot(T, ja, jb, jc, jd, J1, J2, Jbra, Jket);
  return k < 0 ? 0.0 : T.nj_hat[k];
}

}  // namespace imsrg
