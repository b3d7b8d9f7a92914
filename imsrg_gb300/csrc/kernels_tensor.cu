// FP64 kernels of the IMSRG(2) scalar-tensor commutator Z = [X, Y], X a
// scalar and Y a reduced tensor of rank (lambda, |delta Tz|, parity)
// (Commutator::CommutatorScalarTensor, src/Commutator.cc:432-500, and its
// terms in src/TensorCommutators.cc).  One thread per output element; the
// angular factors come from the layout's tables (6j with an integer row, 6j
// with widened half-integers, 9j as sums of those).  Each kernel states the
// reference lines whose arithmetic it reproduces.
#include <cuda_runtime.h>

#include <algorithm>

#include "kernels.cuh"
#include "prof.hpp"
#include "tensor.hpp"

namespace imsrg {
namespace {

constexpr double kSqrt2t = 1.4142135623730950488;
constexpr double kOccCut = 1e-6;  // ModelSpace::OCC_CUT (src/ModelSpace.cc:14)

__device__ __forceinline__ double wsum(double v)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// v with its sign flipped when odd is odd: an integer XOR on the sign bit in
// place of a multiplication by (-1)^odd (FP64 instructions are the scarce
// resource of these kernels on this part)
__device__ __forceinline__ double flip(double v, int odd)
{
  return __longlong_as_double(__double_as_longlong(v) ^ ((long long)(odd & 1) << 63));
}

// v == 0 (either sign), tested on the bits
__device__ __forceinline__ bool is_zero(double v) { return (__double_as_longlong(v) << 1) == 0; }

constexpr double kInvSqrt2 = 0.70710678118654752440;

// z / norm for the normalisation of a (bra, ket) element:
// norm = 1 + delta (both or neither a == b pair), sqrt(2) otherwise
__device__ __forceinline__ double unnorm(double z, int bd, int kd)
{
  if (bd == kd) return bd ? z * 0.5 : z;
  return z * kInvSqrt2;
}

__device__ __forceinline__ int ch_J(int ch) { return ch / 6; }
__device__ __forceinline__ int ch_Tz(int ch) { return (ch % 6) / 2 - 1; }
__device__ __forceinline__ int ch_par(int ch) { return ch & 1; }

// local index of ket (a, b) in two-body channel ch, -1 if the ket is not there
__device__ __forceinline__ int ket_in(const DevSpace& S, int ch, int a, int b)
{
  if (((S.l[a] + S.l[b]) & 1) != ch_par(ch)) return -1;
  if ((S.tz2[a] + S.tz2[b]) / 2 != ch_Tz(ch)) return -1;
  int J = ch_J(ch);
  if (J >= S.NJ) return -1;
  return S.ketJ_loc[J * S.nkets + ket_index(S.norb, min(a, b), max(a, b))];
}

// <ab|X|cd> of a scalar operator in channel ch: TwoBodyME::GetTBME(ch, ch, a, b, c, d)
// (src/TwoBodyME.cc:123-150), with the swap phases and sqrt(2) factors
__device__ double x_tbme(const DevSpace& S, const double* X, int ch, int a, int b, int c, int d)
{
  int bi = ket_in(S, ch, a, b), ki = ket_in(S, ch, c, d);
  if (bi < 0 || ki < 0) return 0.0;
  int J = ch_J(ch), n = S.ch_n[ch];
  int odd = 0;
  if (a > b) odd += ((S.j2[a] + S.j2[b]) >> 1) + 1 + J;
  if (c > d) odd += ((S.j2[c] + S.j2[d]) >> 1) + 1 + J;
  double v = flip(X[S.ch_off[ch] + (long long)ki * n + bi], odd);
  if (a == b) v *= kSqrt2t;
  if (c == d) v *= kSqrt2t;
  return v;
}

// scalar <ab|X|cd>_J: TwoBodyME::GetTBME_J(J, J, a, b, c, d)
__device__ double x_tbme_J(const DevSpace& S, const double* X, int J, int a, int b, int c, int d)
{
  int pb = (S.l[a] + S.l[b]) & 1, pk = (S.l[c] + S.l[d]) & 1;
  int tb = (S.tz2[a] + S.tz2[b]) / 2, tk = (S.tz2[c] + S.tz2[d]) / 2;
  if (pb != pk || tb != tk || J >= S.NJ) return 0.0;
  return x_tbme(S, X, chan_index(J, pb, tb), a, b, c, d);
}

// where <ab|Y|cd> of a reduced tensor between channels chb and chk sits:
// TwoBodyME::GetTBME(chb, chk, a, b, c, d) with the conjugation of the block
// stored as (chk, chb) when chb > chk (src/TwoBodyME.cc:131-150).  The value is
// flip(Y[idx], odd), times sqrt(2) for each of a == b, c == d; idx < 0: zero.
struct YLoc {
  long long idx;
  int odd, sab, scd;
};

__device__ YLoc y_loc(const DevSpace& S, const DevTensor& T, int herm, int chb, int chk, int a, int b, int c, int d)
{
  YLoc L{-1, 0, a == b, c == d};
  int bi = ket_in(S, chb, a, b), ki = ket_in(S, chk, c, d);
  if (bi < 0 || ki < 0) return L;
  int Jb = ch_J(chb), Jk = ch_J(chk);
  if (chb <= chk) {
    int blk = T.lookup[chb * S.nch + chk];
    if (blk < 0) return L;
    L.idx = T.off[blk] + (long long)ki * S.ch_n[chb] + bi;
  } else {
    int blk = T.lookup[chk * S.nch + chb];
    if (blk < 0) return L;
    L.idx = T.off[blk] + (long long)bi * S.ch_n[chk] + ki;
    L.odd = (herm < 0) != ((Jb - Jk) & 1);
  }
  if (a > b) L.odd += ((S.j2[a] + S.j2[b]) >> 1) + 1 + Jb;
  if (c > d) L.odd += ((S.j2[c] + S.j2[d]) >> 1) + 1 + Jk;
  return L;
}

__device__ __forceinline__ double y_at(const YLoc& L, const double* Y)
{
  if (L.idx < 0) return 0.0;
  double v = flip(Y[L.idx], L.odd);
  if (L.sab) v *= kSqrt2t;
  if (L.scd) v *= kSqrt2t;
  return v;
}

// <ab|Y|cd> of a reduced tensor between channels chb and chk
__device__ double y_tbme(const DevSpace& S, const DevTensor& T, const double* Y, int herm, int chb, int chk, int a,
                         int b, int c, int d)
{
  return y_at(y_loc(S, T, herm, chb, chk, a, b, c, d), Y);
}

// where tensor <ab|Y|cd>_(Jb, Jk) sits: TwoBodyME::GetTBME_J(Jb, Jk, a, b, c, d)
// (src/TwoBodyME.cc:300-318)
__device__ YLoc y_loc_J(const DevSpace& S, const DevTensor& T, int herm, int Jb, int Jk, int a, int b, int c, int d)
{
  int pb = (S.l[a] + S.l[b]) & 1, pk = (S.l[c] + S.l[d]) & 1;
  int tb = (S.tz2[a] + S.tz2[b]) / 2, tk = (S.tz2[c] + S.tz2[d]) / 2;
  if (((T.parity + pb + pk) & 1) || abs(tb - tk) != T.trank || abs(Jb - Jk) > T.lam || Jb + Jk < T.lam ||
      Jb >= S.NJ || Jk >= S.NJ)
    return YLoc{-1, 0, 0, 0};
  return y_loc(S, T, herm, chan_index(Jb, pb, tb), chan_index(Jk, pk, tk), a, b, c, d);
}

__device__ double y_tbme_J(const DevSpace& S, const DevTensor& T, const double* Y, int herm, int Jb, int Jk, int a,
                           int b, int c, int d)
{
  return y_at(y_loc_J(S, T, herm, Jb, Jk, a, b, c, d), Y);
}

__device__ __forceinline__ double sixjA(const DevTensor& T, int I1, int I2, int jj1, int jj2, int jj3)
{
  return sixjA_get(T.sixjA, T.NJ, T.d1x, I1, I2, jj1, jj2, jj3);
}

// ---------------------------------------------------------------- comm111st
// Z1 += X1 Y1 - Y1 X1 (src/TensorCommutators.cc:25-30); a thread per element
__global__ void k_t111(DevSpace S, const double* __restrict__ X, const double* __restrict__ Y, double* __restrict__ Z)
{
  const int N = S.norb;
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= N * N) return;
  int j = e / N, i = e - j * N;
  const double *X1 = X + 32, *Y1 = Y + 32;
  double z = 0.0;
  for (int a = 0; a < N; ++a) z += X1[(long long)a * N + i] * Y1[(long long)j * N + a] - Y1[(long long)a * N + i] * X1[(long long)j * N + a];
  Z[32 + (long long)j * N + i] += z;
}

// -------------------------------------------------------------- comm121st
// src/TensorCommutators.cc:46-150: a warp per (i, j >= i) with <i||Z||j>
// allowed, lanes over (hole a, orbit b); the mirror element takes
// hZ (-1)^(ji - jj)
__global__ void k_t121(DevSpace S, DevTensor T, const int* __restrict__ holes, int nholes, const double* __restrict__ X,
                       const double* __restrict__ Y, int hY, double* __restrict__ Z, int hZ)
{
  const int N = S.norb;
  const int e = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (e >= N * N) return;
  const int i = e / N, j = e - i * N;
  if (j < i || !T.ob_ok[i * N + j]) return;
  const int Lam = T.lam;
  const int ji = S.j2[i], jj = S.j2[j];
  const double *X1 = X + 32, *Y1 = Y + 32;
  double zij = 0.0;
  for (int w = lane; w < nholes * N; w += 32) {
    const int a = holes[w / N], b = w - (w / N) * N;
    const int ja = S.j2[a], jb = S.j2[b];
    const double na = S.occ[a], nb = S.occ[b];
    // X one-body (b in a's one-body channel), Y two-body
    if (S.l[b] == S.l[a] && jb == ja && S.tz2[b] == S.tz2[a]) {
      const double nanb = na * (1 - nb);
      const int J1min = abs(ji - ja) >> 1, J1max = (ji + ja) >> 1;
      for (int J1 = J1min; J1 <= J1max; ++J1) {
        const int phasefactor = iphase(((jj + ja) >> 1) + J1 + Lam);
        const int J2min = max(abs(Lam - J1), abs(ja - jj) >> 1), J2max = min(Lam + J1, (ja + jj) >> 1);
        for (int J2 = J2min; J2 <= J2max; ++J2) {
          double pre = flip(nanb, phasefactor < 0) * T.hat2[J1 * T.NJ + J2] * sixjA(T, J1, J2, jj, ji, ja);
          zij += pre * (X1[(long long)b * N + a] * y_tbme_J(S, T, Y, hY, J1, J2, b, i, a, j) -
                        X1[(long long)a * N + b] * y_tbme_J(S, T, Y, hY, J1, J2, a, i, b, j));
        }
      }
    }
    // X two-body, Y one-body
    if (T.ob_ok[a * N + b] && !(fabs(nb - 1) < kOccCut)) {
      const double nanb = na * (1 - nb);
      double xab = 0.0;
      int J1min = max(abs(ji - jb), abs(jj - ja)) >> 1, J1max = min(ji + jb, jj + ja) >> 1;
      for (int J1 = J1min; J1 <= J1max; ++J1)
        xab -= (2 * J1 + 1) * dev_sixj(S, ji, jj, Lam, ja, jb, J1) * x_tbme_J(S, X, J1, i, b, a, j);
      zij -= nanb * Y1[(long long)b * N + a] * xab;
      double xba = 0.0;
      J1min = max(abs(ji - ja), abs(jj - jb)) >> 1;
      J1max = min(ji + ja, jj + jb) >> 1;
      for (int J1 = J1min; J1 <= J1max; ++J1)
        xba -= (2 * J1 + 1) * dev_sixj(S, ji, jj, Lam, jb, ja, J1) * x_tbme_J(S, X, J1, i, a, b, j);
      zij += nanb * Y1[(long long)a * N + b] * xba;
    }
  }
  zij = wsum(zij);
  if (lane) return;
  Z[32 + (long long)j * N + i] += zij;
  if (i != j) Z[32 + (long long)i * N + j] += flip(zij, (hZ < 0) + ((ji - jj) >> 1));
}

// -------------------------------------------------------------- comm122st
// src/TensorCommutators.cc:158-312: a thread per element of every stored block
// (blockIdx.y = block)
__global__ void k_t122(DevSpace S, DevTensor T, const double* __restrict__ X, const double* __restrict__ Y, int hY,
                       double* __restrict__ Z)
{
  const int blk = blockIdx.y;
  const int chb = T.bra[blk], chk = T.ket[blk];  // chb <= chk: the element's own block is stored
  const int nb = S.ch_n[chb], nk = S.ch_n[chk];
  long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)nb * nk) return;
  (void)hY;
  const int ik = (int)(e / nb), ib = (int)(e - (long long)ik * nb);
  const int N = S.norb, Lam = T.lam;
  const int i = S.ket_p[S.ch_kofs[chb] + ib], j = S.ket_q[S.ch_kofs[chb] + ib];
  const int k = S.ket_p[S.ch_kofs[chk] + ik], l = S.ket_q[S.ch_kofs[chk] + ik];
  const int J1 = ch_J(chb), J2 = ch_J(chk);
  const int ji = S.j2[i], jj = S.j2[j], jk = S.j2[k], jl = S.j2[l];
  const double* X1 = X + 32;
  const double* Y1 = Y + 32;
  // <ab|Y|kl> for a bra (a, b) of chb: column ik of the element's block;
  // <ij|Y|cd> for a ket (c, d) of chk: row ib of it (TwoBodyME::GetTBME with
  // the swap phase and sqrt(2) of the bra or ket that varies; the fixed side's
  // sqrt(2) is applied to the sums)
  const double* Yblk = Y + T.off[blk];
  const double* Ycol = Yblk + (long long)ik * nb;
  auto y_bra = [&](int a, int b) -> double {
    const int bi = ket_in(S, chb, a, b);
    if (bi < 0) return 0.0;
    double v = flip(Ycol[bi], a > b ? ((S.j2[a] + S.j2[b]) >> 1) + 1 + J1 : 0);
    return a == b ? v * kSqrt2t : v;
  };
  auto y_ket = [&](int c, int d) -> double {
    const int ki = ket_in(S, chk, c, d);
    if (ki < 0) return 0.0;
    double v = flip(Yblk[(long long)ki * nb + ib], c > d ? ((S.j2[c] + S.j2[d]) >> 1) + 1 + J2 : 0);
    return c == d ? v * kSqrt2t : v;
  };
  // scalar <ab|X|kl>_(J2) (column ik of X's chk block) and <ij|X|cd>_(J1)
  // (row ib of X's chb block)
  const double* Xk = X + S.ch_off[chk] + (long long)ik * nk;
  const double* Xb = X + S.ch_off[chb] + ib;
  auto x_bra = [&](int a, int b) -> double {
    const int bi = ket_in(S, chk, a, b);
    if (bi < 0) return 0.0;
    double v = flip(Xk[bi], a > b ? ((S.j2[a] + S.j2[b]) >> 1) + 1 + J2 : 0);
    return a == b ? v * kSqrt2t : v;
  };
  auto x_ket = [&](int c, int d) -> double {
    const int ki = ket_in(S, chb, c, d);
    if (ki < 0) return 0.0;
    double v = flip(Xb[(long long)ki * nb], c > d ? ((S.j2[c] + S.j2[d]) >> 1) + 1 + J1 : 0);
    return c == d ? v * kSqrt2t : v;
  };
  const double sk = k == l ? kSqrt2t : 1.0, sb = i == j ? kSqrt2t : 1.0;
  // X one-body, Y two-body
  double c1 = 0, c2 = 0, c3 = 0, c4 = 0;
  for (int q = 0; q < S.ob_count[i]; ++q) {
    const int a = S.ob_list[S.ob_start[i] + q];
    c1 = fma(X1[(long long)a * N + i], y_bra(a, j), c1);
  }
  if (i == j) {
    c2 = c1;
  } else {
    for (int q = 0; q < S.ob_count[j]; ++q) {
      const int a = S.ob_list[S.ob_start[j] + q];
      c2 = fma(X1[(long long)a * N + j], y_bra(i, a), c2);
    }
  }
  for (int q = 0; q < S.ob_count[k]; ++q) {
    const int a = S.ob_list[S.ob_start[k] + q];
    c3 = fma(X1[(long long)k * N + a], y_ket(a, l), c3);
  }
  if (k == l) {
    c4 = c3;
  } else {
    for (int q = 0; q < S.ob_count[l]; ++q) {
      const int a = S.ob_list[S.ob_start[l] + q];
      c4 = fma(X1[(long long)l * N + a], y_ket(k, a), c4);
    }
  }
  double cijkl = (c1 + c2) * sk - (c3 + c4) * sb;
  // Y one-body, X two-body
  c1 = c2 = c3 = c4 = 0;
  for (int q = T.tob_off[i]; q < T.tob_off[i + 1]; ++q) {
    const int a = T.tob_list[q];
    c1 -= sixjA(T, J2, J1, ji, S.j2[a], jj) * Y1[(long long)a * N + i] * x_bra(a, j);
  }
  if (i == j) {
    c2 = -c1;
  } else {
    for (int q = T.tob_off[j]; q < T.tob_off[j + 1]; ++q) {
      const int a = T.tob_list[q];
      c2 += sixjA(T, J2, J1, jj, S.j2[a], ji) * Y1[(long long)a * N + j] * x_bra(a, i);
    }
  }
  for (int q = T.tob_off[k]; q < T.tob_off[k + 1]; ++q) {
    const int a = T.tob_list[q];
    c3 -= sixjA(T, J1, J2, jk, S.j2[a], jl) * Y1[(long long)k * N + a] * x_ket(l, a);
  }
  if (k == l) {
    c4 = -c3;
  } else {
    for (int q = T.tob_off[l]; q < T.tob_off[l + 1]; ++q) {
      const int a = T.tob_list[q];
      c4 += sixjA(T, J1, J2, jl, S.j2[a], jk) * Y1[(long long)l * N + a] * x_ket(k, a);
    }
  }
  const int odd1 = ((ji + jj) >> 1) + J2 + Lam;
  const int odd2 = J1 - J2 + Lam, odd3 = odd2;
  const int odd4 = ((jk + jl) >> 1) - J1 + Lam;
  const double hat = T.hat2[J1 * T.NJ + J2];
  cijkl += hat * ((flip(c1, odd1) + flip(c2, odd2)) * sk + (flip(c3, odd3) + flip(c4, odd4)) * sb);
  Z[T.off[blk] + (long long)ik * nb + ib] += unnorm(cijkl, i == j, k == l);
}

// --------------------------------------------------- comm222_pp_hh_221st
// src/TensorCommutators.cc:314-495.  With per-ket weights wpp (pp 1; hh and
// ph (1-na)(1-nb)) and nn (hh na nb), for every stored block (chb, chk),
// Xb = X(chb, chb), Xk = X(chk, chk), Yc = Y(chb, chk):
//   Mpp = Xb wpp Yc - Yc wpp Xk,  Mhh = Xb nn Yc - Yc nn Xk,  Z2 += Mpp - Mhh,
// and the one-body part reads Mpp and Mhh.  Here D = Mpp - Mhh is one product
// with the combined weight w = wpp - nn over the kets where w != 0 (the scalar
// ladder's gather lists), Mhh runs over the hh kets only, and the one-body
// part reads Mpp as D + Mhh.

// weighted copies of X over the gather list K_t, w_t of each channel, at the
// channel's arena offset: XW[t n + r] = X(r, K_t) w_t, WX[t n + c] = w_t X(K_t, c)
__global__ void k_t222_weights(DevSpace S, DevWork W, DevTensor T, const double* __restrict__ X,
                               double* __restrict__ XW, double* __restrict__ WX)
{
  const int ch = blockIdx.y;
  const int n = S.ch_n[ch], K = T.lad_n[ch];
  long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)n * K) return;
  const int t = (int)(e / n), r = (int)(e - (long long)t * n);
  const int kt = W.kidx[T.lad_koff[ch] + t];
  const double w = W.kweight[T.lad_woff[ch] + t];
  const double* Xc = X + S.ch_off[ch];
  XW[S.ch_off[ch] + e] = Xc[(long long)kt * n + r] * w;
  WX[S.ch_off[ch] + e] = Xc[(long long)r * n + kt] * w;
}

// D and Mhh for the element pair (r, c0), (r, c1 = c0 + 1) of every stored
// block (blockIdx.y); Z2 += D
// (SPLIT: D is already there, from the split-form products; only Mhh and
// Z2 += D remain)
template <bool SPLIT>
__global__ void k_t222(DevSpace S, DevWork W, DevTensor T, const double* __restrict__ X,
                       const double* __restrict__ Y, const double* __restrict__ XW, const double* __restrict__ WX,
                       double* __restrict__ D, double* __restrict__ Mhh, double* __restrict__ Z)
{
  const int blk = blockIdx.y;
  const int chb = T.bra[blk], chk = T.ket[blk];
  const int nb = S.ch_n[chb], nk = S.ch_n[chk];
  long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)nb * ((nk + 1) >> 1)) return;
  const int q = (int)(e / nb), r = (int)(e - (long long)q * nb);
  const int c0 = 2 * q, c1 = min(c0 + 1, nk - 1);
  const double* Yc = Y + T.off[blk];
  const double* Y0 = Yc + (long long)c0 * nb;
  const double* Y1 = Yc + (long long)c1 * nb;
  double d0 = 0.0, d1 = 0.0, h0 = 0.0, h1 = 0.0;
  if (!SPLIT) {
    const int Kb = T.lad_n[chb];
    const int* kx = W.kidx + T.lad_koff[chb];
    const double* xw = XW + S.ch_off[chb] + r;
    for (int t = 0; t < Kb; ++t) {
      const double a = xw[(long long)t * nb];
      const int K = kx[t];
      d0 = fma(a, Y0[K], d0);
      d1 = fma(a, Y1[K], d1);
    }
  }
  if (!SPLIT) {
    const int Kk = T.lad_n[chk];
    const int* kx = W.kidx + T.lad_koff[chk];
    const double* wx = WX + S.ch_off[chk];
    for (int t = 0; t < Kk; ++t) {
      const double y = Yc[(long long)kx[t] * nb + r];
      const double* wt = wx + (long long)t * nk;
      d0 = fma(-y, wt[c0], d0);
      d1 = fma(-y, wt[c1], d1);
    }
  }
  {
    const int* hh = W.hh_list + W.hh_off[chb];
    const int nh = W.hh_off[chb + 1] - W.hh_off[chb];
    const double* nn = W.ket_nn + S.ch_kofs[chb];
    const double* Xb = X + S.ch_off[chb] + r;
    for (int t = 0; t < nh; ++t) {
      const int K = hh[t];
      const double a = Xb[(long long)K * nb] * nn[K];
      h0 = fma(a, Y0[K], h0);
      h1 = fma(a, Y1[K], h1);
    }
  }
  {
    const int* hh = W.hh_list + W.hh_off[chk];
    const int nh = W.hh_off[chk + 1] - W.hh_off[chk];
    const double* nn = W.ket_nn + S.ch_kofs[chk];
    const double* Xk = X + S.ch_off[chk];
    for (int t = 0; t < nh; ++t) {
      const int K = hh[t];
      const double y = Yc[(long long)K * nb + r] * nn[K];
      h0 = fma(-y, Xk[(long long)c0 * nk + K], h0);
      h1 = fma(-y, Xk[(long long)c1 * nk + K], h1);
    }
  }
  const long long o0 = T.off[blk] + (long long)c0 * nb + r;
  if (SPLIT) {
    d0 = D[o0];
    if (c1 != c0) d1 = D[o0 + nb];
  } else {
    D[o0] = d0;
    if (c1 != c0) D[o0 + nb] = d1;
  }
  Mhh[o0] = h0;
  Z[o0] += d0;
  if (c1 != c0) {
    Mhh[o0 + nb] = h1;
    Z[o0 + nb] += d1;
  }
}

// ------------------------------------------------------- split-form operands
// Y with every stored block transposed: YT[off + r n_ket + c] = Y[off + c n_bra + r]
// (32 x 32 tiles through shared memory; blockIdx.y = block)
__global__ void k_ttranspose(DevSpace S, DevTensor T, const double* __restrict__ Y, double* __restrict__ YT)
{
  __shared__ double tile[32][33];
  const int blk = blockIdx.y;
  const int nb = S.ch_n[T.bra[blk]], nk = S.ch_n[T.ket[blk]];
  const int tr = (nb + 31) >> 5, tcn = (nk + 31) >> 5;
  if ((int)blockIdx.x >= tr * tcn) return;
  const int r0 = (blockIdx.x % tr) * 32, c0 = (blockIdx.x / tr) * 32;
  const double* src = Y + T.off[blk];
  double* dst = YT + T.off[blk];
  for (int y = threadIdx.y; y < 32; y += 8) {
    const int r = r0 + threadIdx.x, c = c0 + y;
    if (r < nb && c < nk) tile[y][threadIdx.x] = src[(long long)c * nb + r];
  }
  __syncthreads();
  for (int y = threadIdx.y; y < 32; y += 8) {
    const int c = c0 + threadIdx.x, r = r0 + y;
    if (r < nb && c < nk) dst[(long long)r * nk + c] = tile[threadIdx.x][y];
  }
}

// X bar's half-swapped copy for the Z bar tails: per CC channel (blockIdx.y),
// XbF[K n + c] = (-1)^(ket c) (-1)^(ph ket Kh) Xb[swap(K) n + c], with swap
// exchanging the two halves of the 2 nph rows (src/TensorCommutators.cc:
// 1160-1185)
__global__ void k_xbar_flip(DevSpace S, DevWork W, const double* __restrict__ Xb, double* __restrict__ XbF)
{
  const int cc = blockIdx.y;
  const int n = S.cc_n[cc], nph = W.cc_nph[cc];
  long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= 2LL * nph * n) return;
  const int K = (int)(e / n), c = (int)(e - (long long)K * n);
  const int Kh = K < nph ? K : K - nph, src = K < nph ? K + nph : K - nph;
  const int* ph = W.phase_tab + W.cc_phase_off[cc];
  const int* phl = W.cc_ph + W.cc_ph_off[cc];
  const long long o = W.xb_off[cc];
  XbF[o + e] = flip(Xb[o + (long long)src * n + c], (ph[c] < 0) + (ph[phl[Kh]] < 0));
}

// one-body part, src/TensorCommutators.cc:421-495: a warp per (i, j >= i)
// with <i||Z||j> allowed, lanes over c; D and Mhh carry Z's hermiticity
__global__ void k_t221(DevSpace S, DevTensor T, const double* __restrict__ D, const double* __restrict__ Mhh,
                       int hZ, double* __restrict__ Z)
{
  const int N = S.norb;
  const int e = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (e >= N * N) return;
  const int i = e / N, j = e - i * N;
  if (j < i || !T.ob_ok[i * N + j]) return;
  const int Lam = T.lam, ji = S.j2[i], jj = S.j2[j];
  double cij = 0.0;
  for (int c = lane; c < N; c += 32) {
    const int jc = S.j2[c];
    const double nc = S.occ[c];
    const bool hole = nc >= kOccCut;
    const int J1min = abs(jc - ji) >> 1, J1max = (jc + ji) >> 1;
    for (int J1 = J1min; J1 <= J1max; ++J1) {
      const int J2min = max(abs(jc - jj) >> 1, abs(Lam - J1)), J2max = min((jc + jj) >> 1, J1 + Lam);
      for (int J2 = J2min; J2 <= J2max; ++J2) {
        const double w = flip(T.hat2[J1 * T.NJ + J2] * sixjA(T, J1, J2, jj, ji, jc), ((jj + jc) >> 1) + J1 + Lam);
        const YLoc L = y_loc_J(S, T, hZ, J1, J2, c, i, c, j);
        const double mhh = y_at(L, Mhh);
        if (hole)
          cij += w * (nc * (y_at(L, D) + mhh) + (1 - nc) * mhh);
        else
          cij += w * mhh;
      }
    }
  }
  cij = wsum(cij);
  if (lane) return;
  Z[32 + (long long)j * N + i] += cij;
  if (i != j) Z[32 + (long long)i * N + j] += flip(cij, (hZ < 0) + ((ji - jj) >> 1));
}

// ------------------------------------------------------------ comm222_phst
// tensor Pandya transform of Y for the ordered cross-coupled pair
// (bra, ket) = blockIdx.y (DoTensorPandyaTransformation_SingleChannel,
// src/TensorCommutators.cc:637-752): 2 nph_bra x n_ket, rows the bra's hh
// then ph kets (a, b) in both orders
// Split form (YbF != nullptr): the panel is written transposed, Yb[off +
// row n_ket + ik], and its half-swapped copy for the Z bar tails, YbF[off +
// swap(row) n_ket + ik] = hY (-1)^(bra ph ket) (-1)^(ket ik) value.
__global__ void k_tpandya(DevSpace S, DevWork W, DevTensor T, const double* __restrict__ Y, int hY,
                          double* __restrict__ Yb, double* __restrict__ YbF)
{
  const int p = blockIdx.y;
  const int cb = T.yb_bra[p], ck = T.yb_ket[p];
  const int nph = W.cc_nph[cb], nk = S.cc_n[ck];
  long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= 2LL * nph * nk) return;
  const int ik = (int)(e / (2 * nph)), row = (int)(e - (long long)ik * 2 * nph);
  double* out = Yb + T.yb_off[p];
  const int Jbra = ch_J(cb), Jket = ch_J(ck);
  const int Lam = T.lam;
  const int second = row >= nph;
  const int kb = W.cc_ph[W.cc_ph_off[cb] + row - second * nph];
  const long long et = (long long)row * nk + ik, ets = (long long)(second ? row - nph : row + nph) * nk + ik;
  if (Jbra + Jket < Lam || abs(Jbra - Jket) > Lam || ((ch_par(cb) + ch_par(ck) + T.parity) & 1)) {
    if (YbF) {
      out[et] = 0.0;
      YbF[T.yb_off[p] + ets] = 0.0;
    } else {
      out[e] = 0.0;
    }
    return;
  }
  const int p0 = S.cc_p[S.cc_kofs[cb] + kb], q0 = S.cc_q[S.cc_kofs[cb] + kb];
  const int a = second ? q0 : p0, b = second ? p0 : q0;
  const int c = S.cc_p[S.cc_kofs[ck] + ik], d = S.cc_q[S.cc_kofs[ck] + ik];
  const int ja = S.j2[a], jb = S.j2[b], jc = S.j2[c], jd = S.j2[d];
  double sm = 0.0;
  const int J1min = abs(ja - jd) >> 1, J1max = (ja + jd) >> 1;
  const NineJRow nj = ninej_row(T, ja, jb, jc, jd, Jbra, Jket);
  for (int J1 = J1min; J1 <= J1max; ++J1) {
    const int J2min = max(abs(jc - jb) >> 1, abs(J1 - Lam)), J2max = min((jc + jb) >> 1, J1 + Lam);
    for (int J2 = J2min; J2 <= J2max; ++J2) {
      // sm -= hat (-1)^(jb+jd+Jket+J2) 9j tbme; the table holds hat 9j, 0 where |9j| < 1e-8
      const double nh = nj.get(J1, J2);
      if (is_zero(nh)) continue;
      const double tbme = y_tbme_J(S, T, Y, hY, J1, J2, a, d, c, b);
      sm = fma(flip(nh, 1 + ((jb + jd) >> 1) + Jket + J2), tbme, sm);
    }
  }
  if (YbF) {
    out[et] = sm;
    const int* ph_b = W.phase_tab + W.cc_phase_off[cb];
    const int* ph_k = W.phase_tab + W.cc_phase_off[ck];
    YbF[T.yb_off[p] + ets] = flip(sm, (hY < 0) + (ph_b[kb] < 0) + (ph_k[ik] < 0));
  } else {
    out[e] = sm;
  }
}

// Zbar(lo, hi) = Mleft Mright for the pair blockIdx.y (src/TensorCommutators.cc:
// 1130-1190): n_lo x 2 n_hi, a thread per element.  With XJ = the "transpose"
// Pandya transform of X (n_cc x 2nph per channel, at the layout's xb offsets),
// Y12 = Ybar(lo, hi) and Y21 = Ybar(hi, lo):
//   Mleft  = [ XJ1 | -f Y21^T ],  f = hY (-1)^(Jlo - Jhi)
//   Mright = [ Y12 , swap(Y12) o PY ; hX [XJ2 ; swap(XJ2) o PX]^T ]
// where swap exchanges the two halves of the ph index and PY, PX carry the
// phases (-1)^(ja+jb) of the kets involved (PY also f).
__global__ void k_tzbar(DevSpace S, DevWork W, DevTensor T, const double* __restrict__ Xb, const double* __restrict__ Yb,
                        int hX, int hY, double* __restrict__ Zb, const int* __restrict__ phase_tab)
{
  const int p = blockIdx.y;
  const int lo = T.zb_bra[p], hi = T.zb_ket[p];
  const int nlo = S.cc_n[lo], nhi = S.cc_n[hi];
  long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= 2LL * nlo * nhi) return;
  const int col = (int)(e / nlo), r = (int)(e - (long long)col * nlo);
  const int nph1 = W.cc_nph[lo], nph2 = W.cc_nph[hi];
  const double* X1 = Xb + W.xb_off[lo];  // nlo x 2 nph1
  const double* X2 = Xb + W.xb_off[hi];  // nhi x 2 nph2
  const double* Y12 = Yb + T.yb_lookup[lo * S.nch + hi];  // 2 nph1 x nhi
  const double* Y21 = Yb + T.yb_lookup[hi * S.nch + lo];  // 2 nph2 x nlo
  const int fneg = (hY < 0) != ((ch_J(lo) - ch_J(hi)) & 1);  // f = -1
  const int* ph_lo = phase_tab + W.cc_phase_off[lo];     // (-1)^(ja+jb) per CC ket
  const int* ph_hi = phase_tab + W.cc_phase_off[hi];
  const int* phl_lo = W.cc_ph + W.cc_ph_off[lo];         // local index of each ph ket
  const int* phl_hi = W.cc_ph + W.cc_ph_off[hi];
  const bool tail = col >= nhi;
  const int c = tail ? col - nhi : col;
  const double* y12 = Y12 + (long long)c * 2 * nph1;
  const double* y21 = Y21 + (long long)r * 2 * nph2;
  const double* x1 = X1 + r;
  // the second product enters as -f hX Y21^T [...]
  const int sneg = 1 + fneg + (hX < 0);
  double s = 0.0;
  if (!tail) {
    for (int K = 0; K < 2 * nph1; ++K) s = fma(x1[(long long)K * nlo], y12[K], s);
    for (int K = 0; K < 2 * nph2; ++K) s = fma(flip(y21[K], sneg), X2[(long long)K * nhi + c], s);
  } else {
    // the halves of the ph index swap, with the phases of the kets involved
    const int cneg = ph_hi[c] < 0;
    for (int Kh = 0; Kh < nph1; ++Kh) {
      const int odd = fneg + cneg + (ph_lo[phl_lo[Kh]] < 0);
      s = fma(x1[(long long)Kh * nlo], flip(y12[Kh + nph1], odd), s);
      s = fma(x1[(long long)(Kh + nph1) * nlo], flip(y12[Kh], odd), s);
    }
    for (int Kh = 0; Kh < nph2; ++Kh) {
      const int odd = sneg + cneg + (ph_hi[phl_hi[Kh]] < 0);
      s = fma(flip(y21[Kh], odd), X2[(long long)(Kh + nph2) * nhi + c], s);
      s = fma(flip(y21[Kh + nph2], odd), X2[(long long)Kh * nhi + c], s);
    }
  }
  Zb[T.zb_off[p] + (long long)col * nlo + r] = s;
}

// Zbar(al | kb) at (J3, J4) as the inverse transform reads it: the element's
// place and phase follow the reference's four cases (src/TensorCommutators.cc:
// 830-852); 0 when the Zbar block is not stored
__device__ __forceinline__ double zbar_val(const DevSpace& S, const DevTensor& T, const double* Zb, int hZ, int a,
                                           int b, int k, int l, int J3, int J4)
{
  const int pbc = (S.l[a] + S.l[l]) & 1, pkc = (S.l[k] + S.l[b]) & 1;
  const int tbc = abs(S.tz2[a] - S.tz2[l]) / 2, tkc = abs(S.tz2[k] - S.tz2[b]) / 2;
  const int cbra = chan_index(J3, pbc, tbc), cket = chan_index(J4, pkc, tkc);
  const int lo = min(cbra, cket), hi = max(cbra, cket);
  const long long off = T.zb_lookup[lo * S.nch + hi];
  if (off < 0) return 0.0;
  const int ixil = S.ccJ_loc[J3 * S.nkets + ket_index(S.norb, min(a, l), max(a, l))];
  const int ixkj = S.ccJ_loc[J4 * S.nkets + ket_index(S.norb, min(b, k), max(b, k))];
  const double* M = Zb + off;
  const int nrow = S.cc_n[lo];
  const int sum4 = (S.j2[a] + S.j2[b] + S.j2[k] + S.j2[l]) >> 1, hneg = hZ < 0;
  if (cbra <= cket) {
    if (a <= l) return M[(long long)(ixkj + (k > b ? S.cc_n[cket] : 0)) * nrow + ixil];
    return flip(M[(long long)(ixkj + (k > b ? 0 : S.cc_n[cket])) * nrow + ixil], hneg + J3 - J4 + sum4);
  }
  if (k <= b) return flip(M[(long long)(ixil + (a > l ? S.cc_n[cbra] : 0)) * nrow + ixkj], hneg + J3 - J4);
  return flip(M[(long long)(ixil + (a > l ? 0 : S.cc_n[cbra])) * nrow + ixkj], sum4);
}

// the Zbar values one sum of the inverse transform reads for the quadruple
// (a, b, k, l): slot (J3 - J3min) w + (J4 - J3 + lam), lanes over slots
__device__ __forceinline__ void tinv_gather(const DevSpace& S, const DevTensor& T, const double* Zb, int hZ, int a,
                                            int b, int k, int l, double* in, int lane)
{
  const int ja = S.j2[a], jb = S.j2[b], jk = S.j2[k], jl = S.j2[l], Lam = T.lam, w = 2 * Lam + 1;
  const int J3min = abs(ja - jl) >> 1, nJ3 = ((ja + jl) >> 1) - J3min + 1;
  const int J4lo = abs(jk - jb) >> 1, J4hi = (jk + jb) >> 1;
  for (int s = lane; s < nJ3 * w; s += 32) {
    const int J3 = J3min + s / w, J4 = J3 - Lam + s % w;
    in[s] = (J4 < J4lo || J4 > J4hi) ? 0.0 : zbar_val(S, T, Zb, hZ, a, b, k, l, J3, J4);
  }
}

// one sum over the gathered values: sum_{J3, J4} hat 9j (-1)^(jb + jl + J2 + J4)
// Zbar (the 9j {ja jb J1; ...} row of (J1, J2))
__device__ __forceinline__ double tinv_dot(const DevSpace& S, const DevTensor& T, int a, int b, int k, int l, int J1,
                                           int J2, const double* in)
{
  const int ja = S.j2[a], jb = S.j2[b], jk = S.j2[k], jl = S.j2[l], Lam = T.lam, w = 2 * Lam + 1;
  const NineJRow nj = ninej_row(T, ja, jb, jk, jl, J1, J2);
  const int J3min = abs(ja - jl) >> 1, J3max = (ja + jl) >> 1;
  double acc = 0.0;
  for (int J3 = J3min; J3 <= J3max; ++J3) {
    const int J4min = max(abs(jk - jb) >> 1, abs(J3 - Lam)), J4max = min((jk + jb) >> 1, J3 + Lam);
    const double* row = in + (J3 - J3min) * w - J3 + Lam;
    for (int J4 = J4min; J4 <= J4max; ++J4) {
      const double nh = nj.get(J3, J4);
      if (is_zero(nh)) continue;
      acc = fma(flip(nh, ((jb + jl) >> 1) + J2 + J4), row[J4], acc);
    }
  }
  return acc;
}

// Inverse tensor Pandya transform by orbit quadruple (AddInverseTensor-
// PandyaTransformation, src/TensorCommutators.cc:754-920): a warp per (i <= j,
// k <= l) of the layout's quadruple list.  The Zbar values of both sums (over
// J3, J4) are gathered once into shared memory; then the lanes take the
// (J1, J2) slots whose element the quadruple owns (a stored block, the upper
// triangle of a diagonal one) and sum over them.  Each stored element is owned
// by exactly one quadruple and slot, so there are no write conflicts.
constexpr int kTqWarps = 8;

__global__ void __launch_bounds__(32 * kTqWarps) k_tinv_q(DevSpace S, DevTensor T, const double* __restrict__ Zb,
                                                         int hZ, double* __restrict__ Z,
                                                         const int2* __restrict__ tq, long long nq, int slots)
{
  extern __shared__ double s_in[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long qi = blockIdx.x * (long long)kTqWarps + warp;
  if (qi >= nq) return;
  double* in1 = s_in + (size_t)warp * 2 * slots;
  double* in2 = in1 + slots;
  const int2 v = tq[qi];
  const int i = v.x & 0xFFFF, j = v.x >> 16, k = v.y & 0xFFFF, l = v.y >> 16;
  tinv_gather(S, T, Zb, hZ, i, j, k, l, in1, lane);
  if (i != j) tinv_gather(S, T, Zb, hZ, j, i, k, l, in2, lane);
  __syncwarp();
  const int ji = S.j2[i], jj = S.j2[j], jk = S.j2[k], jl = S.j2[l], Lam = T.lam, w = 2 * Lam + 1;
  const int pb = (S.l[i] + S.l[j]) & 1, tb = (S.tz2[i] + S.tz2[j]) / 2;
  const int pk = (S.l[k] + S.l[l]) & 1, tk = (S.tz2[k] + S.tz2[l]) / 2;
  const int kb = ket_index(S.norb, i, j), kk = ket_index(S.norb, k, l);
  const int J1min = abs(ji - jj) >> 1, nJ1 = ((ji + jj) >> 1) - J1min + 1;
  const int J2lo = abs(jk - jl) >> 1, J2hi = (jk + jl) >> 1;
  for (int t = lane; t < nJ1 * w; t += 32) {
    const int J1 = J1min + t / w, J2 = J1 - Lam + t % w;
    if (J2 < J2lo || J2 > J2hi || J1 >= S.NJ || J2 >= S.NJ) continue;
    const int ib = S.ketJ_loc[J1 * S.nkets + kb], ik = S.ketJ_loc[J2 * S.nkets + kk];
    if (ib < 0 || ik < 0) continue;
    const int chb = chan_index(J1, pb, tb), chk = chan_index(J2, pk, tk);
    if (chb > chk || (chb == chk && ik < ib)) continue;
    const int blk = T.lookup[chb * S.nch + chk];
    if (blk < 0) continue;
    const double commij = tinv_dot(S, T, i, j, k, l, J1, J2, in1);
    const double commji = i == j ? commij : tinv_dot(S, T, j, i, k, l, J1, J2, in2);
    const double z = unnorm(commij + flip(commji, 1 + ((ji + jj) >> 1) - J1), i == j, k == l);
    const int nb = S.ch_n[chb];
    Z[T.off[blk] + (long long)ik * nb + ib] += z;
    if (chb == chk && ik != ib) Z[T.off[blk] + (long long)ib * nb + ik] += flip(z, hZ < 0);
  }
}

unsigned grid_for(long long n) { return (unsigned)std::max(1LL, (n + 255) / 256); }

cudaError_t launch_tinv_q(const Space& s, const TensorLayout& t, const double* Zbar, double* Z, int hZ,
                          cudaStream_t st)
{
  const long long nq = (long long)t.tq.size();
  if (nq == 0) return cudaSuccess;
  const int slots = t.tq_max_j3 * (2 * t.lam + 1);
  const size_t smem = (size_t)kTqWarps * 2 * slots * sizeof(double);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k_tinv_q, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  k_tinv_q<<<(unsigned)((nq + kTqWarps - 1) / kTqWarps), 32 * kTqWarps, smem, st>>>(s.dev, t.dev, Zbar, hZ, Z, t.d_tq,
                                                                                     nq, slots);
  count_launch();
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_tensor_111(const Space& s, const double* X, const double* Y, double* Z, cudaStream_t st)
{
  int nn = s.norb * s.norb;
  k_t111<<<grid_for(nn), 256, 0, st>>>(s.dev, X, Y, Z);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_tensor_121(const Space& s, const TensorLayout& t, const int* dev_holes, const double* X,
                              const double* Y, int hY, double* Z, int hZ, cudaStream_t st)
{
  int nn = s.norb * s.norb;
  k_t121<<<(nn + 7) / 8, 256, 0, st>>>(s.dev, t.dev, dev_holes, (int)s.holes.size(), X, Y, hY, Z, hZ);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_tensor_122(const Space& s, const TensorLayout& t, const double* X, const double* Y, int hY,
                              double* Z, cudaStream_t st)
{
  if (t.bra.empty() || t.max_blk_elems == 0) return cudaSuccess;
  dim3 grid(grid_for(t.max_blk_elems), (unsigned)t.bra.size());
  k_t122<<<grid, 256, 0, st>>>(s.dev, t.dev, X, Y, hY, Z);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_tensor_222_221(const Space& s, const TensorLayout& t, const double* X, const double* Y,
                                  double* XW, double* WX, double* D, double* Mhh, double* Z, int hZ, cudaStream_t st)
{
  cudaError_t e = cudaMemsetAsync(D, 0, t.total * sizeof(double), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(Mhh, 0, t.total * sizeof(double), st);
  if (e != cudaSuccess) return e;
  if (!t.bra.empty() && t.max_blk_elems > 0) {
    if (t.lad_maxelems > 0) {
      dim3 gw(grid_for(t.lad_maxelems), (unsigned)s.nch);
      k_t222_weights<<<gw, 256, 0, st>>>(s.dev, s.work, t.dev, X, XW, WX);
      count_launch();
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    // element pairs: a block's columns come two at a time
    dim3 grid(grid_for(t.max_pair_elems), (unsigned)t.bra.size());
    k_t222<false><<<grid, 256, 0, st>>>(s.dev, s.work, t.dev, X, Y, XW, WX, D, Mhh, Z);
    count_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  int nn = s.norb * s.norb;
  k_t221<<<(nn + 7) / 8, 256, 0, st>>>(s.dev, t.dev, D, Mhh, hZ, Z);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_tensor_ph(const Space& s, const TensorLayout& t, const double* Xbar, const double* Y, int hX,
                             int hY, double* Ybar, double* Zbar, double* Z, int hZ, cudaStream_t st)
{
  if (t.yb_bra.empty()) return cudaSuccess;
  dim3 gy(grid_for(std::max(1, t.yb_maxelems)), (unsigned)t.yb_bra.size());
  k_tpandya<<<gy, 256, 0, st>>>(s.dev, s.work, t.dev, Y, hY, Ybar, nullptr);
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  dim3 gz(grid_for(std::max(1, t.zb_maxelems)), (unsigned)t.zb_bra.size());
  k_tzbar<<<gz, 256, 0, st>>>(s.dev, s.work, t.dev, Xbar, Ybar, hX, hY, Zbar, s.work.phase_tab);
  count_launch();
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  return launch_tinv_q(s, t, Zbar, Z, hZ, st);
}

// ---------------------------------------------------------- split form
cudaError_t launch_tensor_split_operands(const Space& s, const TensorLayout& t, const double* Y, int hY,
                                         const double* Xbar, double* YT, double* YbT, double* YbTF, double* XbF,
                                         cudaStream_t st)
{
  cudaError_t e;
  if (!t.bra.empty() && t.max_tiles32 > 0) {
    k_ttranspose<<<dim3((unsigned)t.max_tiles32, (unsigned)t.bra.size()), dim3(32, 8), 0, st>>>(s.dev, t.dev, Y,
                                                                                              YT);
    count_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  if (!t.yb_bra.empty()) {
    dim3 gy(grid_for(std::max(1, t.yb_maxelems)), (unsigned)t.yb_bra.size());
    k_tpandya<<<gy, 256, 0, st>>>(s.dev, s.work, t.dev, Y, hY, YbT, YbTF);
    count_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  if (t.max_xbf > 0) {
    k_xbar_flip<<<dim3(grid_for(t.max_xbf), (unsigned)s.nch), 256, 0, st>>>(s.dev, s.work, Xbar, XbF);
    count_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_tensor_222_221_split(const Space& s, const TensorLayout& t, const double* X, const double* Y,
                                        double* D, double* Mhh, double* Z, int hZ, cudaStream_t st)
{
  cudaError_t e = cudaMemsetAsync(Mhh, 0, t.total * sizeof(double), st);
  if (e != cudaSuccess) return e;
  if (!t.bra.empty() && t.max_blk_elems > 0) {
    dim3 grid(grid_for(t.max_pair_elems), (unsigned)t.bra.size());
    k_t222<true><<<grid, 256, 0, st>>>(s.dev, s.work, t.dev, X, Y, nullptr, nullptr, D, Mhh, Z);
    count_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  int nn = s.norb * s.norb;
  k_t221<<<(nn + 7) / 8, 256, 0, st>>>(s.dev, t.dev, D, Mhh, hZ, Z);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_tensor_inverse_pandya(const Space& s, const TensorLayout& t, const double* Zbar, double* Z, int hZ,
                                         cudaStream_t st)
{
  return launch_tinv_q(s, t, Zbar, Z, hZ, st);
}

}  // namespace imsrg
