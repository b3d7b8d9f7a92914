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
  double v = X[S.ch_off[ch] + (long long)ki * n + bi];
  if (a > b) v *= iphase(((S.j2[a] + S.j2[b]) >> 1) + 1 + J);
  if (c > d) v *= iphase(((S.j2[c] + S.j2[d]) >> 1) + 1 + J);
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

// <ab|Y|cd> of a reduced tensor between channels chb and chk: TwoBodyME::
// GetTBME(chb, chk, a, b, c, d) with the conjugation of the block stored as
// (chk, chb) when chb > chk (src/TwoBodyME.cc:131-150)
__device__ double y_tbme(const DevSpace& S, const DevTensor& T, const double* Y, int herm, int chb, int chk, int a,
                         int b, int c, int d)
{
  int bi = ket_in(S, chb, a, b), ki = ket_in(S, chk, c, d);
  if (bi < 0 || ki < 0) return 0.0;
  int Jb = ch_J(chb), Jk = ch_J(chk);
  double v;
  if (chb <= chk) {
    int blk = T.lookup[chb * S.nch + chk];
    if (blk < 0) return 0.0;
    v = Y[T.off[blk] + (long long)ki * S.ch_n[chb] + bi];
  } else {
    int blk = T.lookup[chk * S.nch + chb];
    if (blk < 0) return 0.0;
    v = Y[T.off[blk] + (long long)bi * S.ch_n[chk] + ki];
    if ((herm < 0) != ((Jb - Jk) & 1)) v = -v;
  }
  if (a > b) v *= iphase(((S.j2[a] + S.j2[b]) >> 1) + 1 + Jb);
  if (c > d) v *= iphase(((S.j2[c] + S.j2[d]) >> 1) + 1 + Jk);
  if (a == b) v *= kSqrt2t;
  if (c == d) v *= kSqrt2t;
  return v;
}

// tensor <ab|Y|cd>_(Jb, Jk): TwoBodyME::GetTBME_J(Jb, Jk, a, b, c, d) (src/TwoBodyME.cc:300-318)
__device__ double y_tbme_J(const DevSpace& S, const DevTensor& T, const double* Y, int herm, int Jb, int Jk, int a,
                           int b, int c, int d)
{
  int pb = (S.l[a] + S.l[b]) & 1, pk = (S.l[c] + S.l[d]) & 1;
  int tb = (S.tz2[a] + S.tz2[b]) / 2, tk = (S.tz2[c] + S.tz2[d]) / 2;
  if ((T.parity + pb + pk) & 1) return 0.0;
  if (abs(tb - tk) != T.trank) return 0.0;
  if (abs(Jb - Jk) > T.lam || Jb + Jk < T.lam) return 0.0;
  if (Jb >= S.NJ || Jk >= S.NJ) return 0.0;
  return y_tbme(S, T, Y, herm, chan_index(Jb, pb, tb), chan_index(Jk, pk, tk), a, b, c, d);
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
          double pre = nanb * phasefactor * sqrt((double)((2 * J1 + 1) * (2 * J2 + 1))) * sixjA(T, J1, J2, jj, ji, ja);
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
  if (i != j) Z[32 + (long long)i * N + j] += hZ * iphase((ji - jj) >> 1) * zij;
}

// -------------------------------------------------------------- comm122st
// src/TensorCommutators.cc:158-312: a thread per element of every stored block
// (blockIdx.y = block)
__global__ void k_t122(DevSpace S, DevTensor T, const double* __restrict__ X, const double* __restrict__ Y, int hY,
                       double* __restrict__ Z)
{
  const int blk = blockIdx.y;
  const int chb = T.bra[blk], chk = T.ket[blk];
  const int nb = S.ch_n[chb], nk = S.ch_n[chk];
  long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)nb * nk) return;
  const int ik = (int)(e / nb), ib = (int)(e - (long long)ik * nb);
  const int N = S.norb, Lam = T.lam;
  const int i = S.ket_p[S.ch_kofs[chb] + ib], j = S.ket_q[S.ch_kofs[chb] + ib];
  const int k = S.ket_p[S.ch_kofs[chk] + ik], l = S.ket_q[S.ch_kofs[chk] + ik];
  const int J1 = ch_J(chb), J2 = ch_J(chk);
  const int ji = S.j2[i], jj = S.j2[j], jk = S.j2[k], jl = S.j2[l];
  const double* X1 = X + 32;
  const double* Y1 = Y + 32;
  double c1 = 0, c2 = 0, c3 = 0, c4 = 0;
  for (int q = 0; q < S.ob_count[i]; ++q) {
    int a = S.ob_list[S.ob_start[i] + q];
    c1 += X1[(long long)a * N + i] * y_tbme(S, T, Y, hY, chb, chk, a, j, k, l);
  }
  if (i == j) {
    c2 = c1;
  } else {
    for (int q = 0; q < S.ob_count[j]; ++q) {
      int a = S.ob_list[S.ob_start[j] + q];
      c2 += X1[(long long)a * N + j] * y_tbme(S, T, Y, hY, chb, chk, i, a, k, l);
    }
  }
  for (int q = 0; q < S.ob_count[k]; ++q) {
    int a = S.ob_list[S.ob_start[k] + q];
    c3 += X1[(long long)k * N + a] * y_tbme(S, T, Y, hY, chb, chk, i, j, a, l);
  }
  if (k == l) {
    c4 = c3;
  } else {
    for (int q = 0; q < S.ob_count[l]; ++q) {
      int a = S.ob_list[S.ob_start[l] + q];
      c4 += X1[(long long)l * N + a] * y_tbme(S, T, Y, hY, chb, chk, i, j, k, a);
    }
  }
  double cijkl = c1 + c2 - c3 - c4;
  c1 = c2 = c3 = c4 = 0;
  const int phase1 = iphase(((ji + jj) >> 1) + J2 + Lam);
  const int phase2 = iphase(J1 - J2 + Lam), phase3 = phase2;
  const int phase4 = iphase(((jk + jl) >> 1) - J1 + Lam);
  for (int a = 0; a < N; ++a) {
    if (!T.ob_ok[i * N + a]) continue;
    c1 -= sixjA(T, J2, J1, ji, S.j2[a], jj) * Y1[(long long)a * N + i] * x_tbme(S, X, chk, a, j, k, l);
  }
  if (i == j) {
    c2 = -c1;
  } else {
    for (int a = 0; a < N; ++a) {
      if (!T.ob_ok[j * N + a]) continue;
      c2 += sixjA(T, J2, J1, jj, S.j2[a], ji) * Y1[(long long)a * N + j] * x_tbme(S, X, chk, a, i, k, l);
    }
  }
  for (int a = 0; a < N; ++a) {
    if (!T.ob_ok[a * N + k]) continue;
    c3 -= sixjA(T, J1, J2, jk, S.j2[a], jl) * Y1[(long long)k * N + a] * x_tbme(S, X, chb, i, j, l, a);
  }
  if (k == l) {
    c4 = -c3;
  } else {
    for (int a = 0; a < N; ++a) {
      if (!T.ob_ok[a * N + l]) continue;
      c4 += sixjA(T, J1, J2, jl, S.j2[a], jk) * Y1[(long long)l * N + a] * x_tbme(S, X, chb, i, j, k, a);
    }
  }
  const double hat = sqrt((double)((2 * J1 + 1) * (2 * J2 + 1)));
  cijkl += hat * (phase1 * c1 + phase2 * c2 + phase3 * c3 + phase4 * c4);
  const int bd = i == j, kd = k == l;
  const double norm = bd == kd ? 1.0 + bd : kSqrt2t;
  Z[T.off[blk] + (long long)ik * nb + ib] += cijkl / norm;
}

// --------------------------------------------------- comm222_pp_hh_221st
// two-body part, src/TensorCommutators.cc:314-420: for every stored block
// (chb, chk), with Xb = X(chb, chb), Xk = X(chk, chk), Yc = Y(chb, chk) and
// per-ket weights wpp (pp 1, hh and ph (1-na)(1-nb)) and nn (hh na nb):
//   Mpp = Xb wpp_b Yc - Yc wpp_k Xk,  Mhh = Xb nn_b Yc - Yc nn_k Xk,
//   Z2 += Mpp - Mhh.  A thread per element; Mpp and Mhh are kept for the
// one-body part.
__global__ void k_t222(DevSpace S, DevWork W, DevTensor T, const double* __restrict__ X,
                       const double* __restrict__ Y, double* __restrict__ Mpp, double* __restrict__ Mhh,
                       double* __restrict__ Z)
{
  const int blk = blockIdx.y;
  const int chb = T.bra[blk], chk = T.ket[blk];
  const int nb = S.ch_n[chb], nk = S.ch_n[chk];
  long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)nb * nk) return;
  const int c = (int)(e / nb), r = (int)(e - (long long)c * nb);
  const double* Xb = X + S.ch_off[chb];
  const double* Xk = X + S.ch_off[chk];
  const double* Yc = Y + T.off[blk];
  const double* wb = W.ket_wpp + S.ch_kofs[chb];
  const double* nnb = W.ket_nn + S.ch_kofs[chb];
  const double* wk = W.ket_wpp + S.ch_kofs[chk];
  const double* nnk = W.ket_nn + S.ch_kofs[chk];
  double pp = 0.0, hh = 0.0;
  for (int K = 0; K < nb; ++K) {
    double xy = Xb[(long long)K * nb + r] * Yc[(long long)c * nb + K];
    pp += wb[K] * xy;
    hh += nnb[K] * xy;
  }
  for (int K = 0; K < nk; ++K) {
    double yx = Yc[(long long)K * nb + r] * Xk[(long long)c * nk + K];
    pp -= wk[K] * yx;
    hh -= nnk[K] * yx;
  }
  const long long o = T.off[blk] + (long long)c * nb + r;
  Mpp[o] = pp;
  Mhh[o] = hh;
  Z[o] += pp - hh;
}

// one-body part, src/TensorCommutators.cc:421-495: a warp per (i, j >= i)
// with <i||Z||j> allowed, lanes over c; Mpp and Mhh carry Z's hermiticity
__global__ void k_t221(DevSpace S, DevTensor T, const double* __restrict__ Mpp, const double* __restrict__ Mhh,
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
        double w = sqrt((double)((2 * J1 + 1) * (2 * J2 + 1))) * sixjA(T, J1, J2, jj, ji, jc) *
                   iphase(((jj + jc) >> 1) + J1 + Lam);
        double mhh = y_tbme_J(S, T, Mhh, hZ, J1, J2, c, i, c, j);
        if (hole)
          cij += w * (nc * y_tbme_J(S, T, Mpp, hZ, J1, J2, c, i, c, j) + (1 - nc) * mhh);
        else
          cij += w * mhh;
      }
    }
  }
  cij = wsum(cij);
  if (lane) return;
  Z[32 + (long long)j * N + i] += cij;
  if (i != j) Z[32 + (long long)i * N + j] += hZ * iphase((ji - jj) >> 1) * cij;
}

// ------------------------------------------------------------ comm222_phst
// tensor Pandya transform of Y for the ordered cross-coupled pair
// (bra, ket) = blockIdx.y (DoTensorPandyaTransformation_SingleChannel,
// src/TensorCommutators.cc:637-752): 2 nph_bra x n_ket, rows the bra's hh
// then ph kets (a, b) in both orders
__global__ void k_tpandya(DevSpace S, DevWork W, DevTensor T, const double* __restrict__ Y, int hY,
                          double* __restrict__ Yb)
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
  if (Jbra + Jket < Lam || abs(Jbra - Jket) > Lam || ((ch_par(cb) + ch_par(ck) + T.parity) & 1)) {
    out[e] = 0.0;
    return;
  }
  const int second = row >= nph;
  const int kb = W.cc_ph[W.cc_ph_off[cb] + row - second * nph];
  const int p0 = S.cc_p[S.cc_kofs[cb] + kb], q0 = S.cc_q[S.cc_kofs[cb] + kb];
  const int a = second ? q0 : p0, b = second ? p0 : q0;
  const int c = S.cc_p[S.cc_kofs[ck] + ik], d = S.cc_q[S.cc_kofs[ck] + ik];
  const int ja = S.j2[a], jb = S.j2[b], jc = S.j2[c], jd = S.j2[d];
  double sm = 0.0;
  const int J1min = abs(ja - jd) >> 1, J1max = (ja + jd) >> 1;
  for (int J1 = J1min; J1 <= J1max; ++J1) {
    const int J2min = max(abs(jc - jb) >> 1, abs(J1 - Lam)), J2max = min((jc + jb) >> 1, J1 + Lam);
    for (int J2 = J2min; J2 <= J2max; ++J2) {
      double nj = ninej_get(T, ja, jb, jc, jd, J1, J2, Jbra, Jket);
      if (fabs(nj) < 1e-8) continue;
      double hat = sqrt((double)((2 * J1 + 1) * (2 * J2 + 1) * (2 * Jbra + 1) * (2 * Jket + 1)));
      double tbme = y_tbme_J(S, T, Y, hY, J1, J2, a, d, c, b);
      sm -= hat * iphase(((jb + jd) >> 1) + Jket + J2) * nj * tbme;
    }
  }
  out[e] = sm;
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
  const int f = ((hY < 0) != ((ch_J(lo) - ch_J(hi)) & 1)) ? -1 : 1;
  const int* ph_lo = phase_tab + W.cc_phase_off[lo];  // (-1)^(ja+jb) per CC ket
  const int* ph_hi = phase_tab + W.cc_phase_off[hi];
  const int* phl_lo = W.cc_ph + W.cc_ph_off[lo];      // local index of each ph ket
  const int* phl_hi = W.cc_ph + W.cc_ph_off[hi];
  const bool tail = col >= nhi;
  const int c = tail ? col - nhi : col;
  double s = 0.0;
  for (int K = 0; K < 2 * nph1; ++K) {
    double top;
    if (!tail) {
      top = Y12[(long long)c * 2 * nph1 + K];
    } else {
      const int Kh = K < nph1 ? K : K - nph1;
      const int src = K < nph1 ? K + nph1 : K - nph1;
      top = Y12[(long long)c * 2 * nph1 + src] * (f * ph_lo[phl_lo[Kh]] * ph_hi[c]);
    }
    s += X1[(long long)K * nlo + r] * top;
  }
  for (int K = 0; K < 2 * nph2; ++K) {
    double bot;
    if (!tail) {
      bot = X2[(long long)K * nhi + c];
    } else {
      const int Kh = K < nph2 ? K : K - nph2;
      const int src = K < nph2 ? K + nph2 : K - nph2;
      bot = X2[(long long)src * nhi + c] * (ph_hi[c] * ph_hi[phl_hi[Kh]]);
    }
    s -= f * Y21[(long long)r * 2 * nph2 + K] * (hX * bot);
  }
  Zb[T.zb_off[p] + (long long)col * nlo + r] = s;
}

// Zbar element (il | kj) of cross-coupled channels (cbra, cket) as the
// inverse transform reads it (src/TensorCommutators.cc:830-852)
__device__ double zbar_get(const DevSpace& S, const DevTensor& T, const double* Zb, int hZ, int cbra, int cket,
                           int i, int l, int k, int j, int ji, int jj, int jk, int jl, int J3, int J4, bool* found)
{
  const int lo = min(cbra, cket), hi = max(cbra, cket);
  const long long off = T.zb_lookup[lo * S.nch + hi];
  *found = off >= 0;
  if (off < 0) return 0.0;
  const int nbras = S.cc_n[cbra], nkets = S.cc_n[cket];
  const int ixil = S.ccJ_loc[J3 * S.nkets + ket_index(S.norb, min(i, l), max(i, l))];
  const int ixkj = S.ccJ_loc[J4 * S.nkets + ket_index(S.norb, min(j, k), max(j, k))];
  const double* M = Zb + off;
  const int nrow = S.cc_n[lo];
  const int sum4 = (ji + jj + jk + jl) >> 1;
  if (cbra <= cket) {
    if (i <= l) return M[(long long)(ixkj + (k > j ? nkets : 0)) * nrow + ixil];
    return M[(long long)(ixkj + (k > j ? 0 : nkets)) * nrow + ixil] * (hZ * iphase(J3 - J4 + sum4));
  }
  if (k <= j) return M[(long long)(ixil + (i > l ? nbras : 0)) * nrow + ixkj] * (hZ * iphase(J3 - J4));
  return M[(long long)(ixil + (i > l ? 0 : nbras)) * nrow + ixkj] * iphase(sum4);
}

// inverse tensor Pandya transform, AddInverseTensorPandyaTransformation
// (src/TensorCommutators.cc:754-920): a thread per element (ibra, iket) of a
// stored block (iket >= ibra in a diagonal block, whose lower triangle takes
// hZ times the upper)
__global__ void k_tinv(DevSpace S, DevTensor T, const double* __restrict__ Zb, int hZ, double* __restrict__ Z)
{
  const int blk = blockIdx.y;
  const int chb = T.bra[blk], chk = T.ket[blk];
  const int nb = S.ch_n[chb], nk = S.ch_n[chk];
  long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= (long long)nb * nk) return;
  const int ik = (int)(e / nb), ib = (int)(e - (long long)ik * nb);
  if (chb == chk && ik < ib) return;
  const int i = S.ket_p[S.ch_kofs[chb] + ib], j = S.ket_q[S.ch_kofs[chb] + ib];
  const int k = S.ket_p[S.ch_kofs[chk] + ik], l = S.ket_q[S.ch_kofs[chk] + ik];
  const int J1 = ch_J(chb), J2 = ch_J(chk), Lam = T.lam;
  const int ji = S.j2[i], jj = S.j2[j], jk = S.j2[k], jl = S.j2[l];
  const double h12 = (double)((2 * J1 + 1) * (2 * J2 + 1));
  double commij = 0.0, commji = 0.0;
  {
    const int pbc = (S.l[i] + S.l[l]) & 1, pkc = (S.l[k] + S.l[j]) & 1;
    const int tbc = abs(S.tz2[i] - S.tz2[l]) / 2, tkc = abs(S.tz2[k] - S.tz2[j]) / 2;
    const int J3min = abs(ji - jl) >> 1, J3max = (ji + jl) >> 1;
    for (int J3 = J3min; J3 <= J3max; ++J3) {
      const int cbra = chan_index(J3, pbc, tbc);
      const int J4min = max(abs(jk - jj) >> 1, abs(J3 - Lam)), J4max = min((jk + jj) >> 1, J3 + Lam);
      for (int J4 = J4min; J4 <= J4max; ++J4) {
        const int cket = chan_index(J4, pkc, tkc);
        double nj = ninej_get(T, ji, jj, jk, jl, J3, J4, J1, J2);
        if (fabs(nj) < 1e-8) continue;
        bool found;
        double tbme = zbar_get(S, T, Zb, hZ, cbra, cket, i, l, k, j, ji, jj, jk, jl, J3, J4, &found);
        if (!found) continue;
        double hat = sqrt(h12 * (double)((2 * J3 + 1) * (2 * J4 + 1)));
        commij += hat * iphase(((jj + jl) >> 1) + J2 + J4) * nj * tbme;
      }
    }
  }
  if (i == j) {
    commji = commij;
  } else {
    const int pbc = (S.l[j] + S.l[l]) & 1, pkc = (S.l[k] + S.l[i]) & 1;
    const int tbc = abs(S.tz2[j] - S.tz2[l]) / 2, tkc = abs(S.tz2[k] - S.tz2[i]) / 2;
    const int J3min = abs(jj - jl) >> 1, J3max = (jj + jl) >> 1;
    for (int J3 = J3min; J3 <= J3max; ++J3) {
      const int cbra = chan_index(J3, pbc, tbc);
      const int J4min = max(abs(jk - ji) >> 1, abs(J3 - Lam)), J4max = min((jk + ji) >> 1, J3 + Lam);
      for (int J4 = J4min; J4 <= J4max; ++J4) {
        const int cket = chan_index(J4, pkc, tkc);
        double nj = ninej_get(T, jj, ji, jk, jl, J3, J4, J1, J2);
        if (fabs(nj) < 1e-8) continue;
        bool found;
        double tbme = zbar_get(S, T, Zb, hZ, cbra, cket, j, l, k, i, jj, ji, jk, jl, J3, J4, &found);
        if (!found) continue;
        double hat = sqrt(h12 * (double)((2 * J3 + 1) * (2 * J4 + 1)));
        commji += hat * iphase(((ji + jl) >> 1) + J2 + J4) * nj * tbme;
      }
    }
  }
  const int bd = i == j, kd = k == l;
  const double norm = bd == kd ? 1.0 + bd : kSqrt2t;
  const double z = (commij - iphase(((ji + jj) >> 1) - J1) * commji) / norm;
  Z[T.off[blk] + (long long)ik * nb + ib] += z;
  if (chb == chk && ik != ib) Z[T.off[blk] + (long long)ib * nb + ik] += hZ * z;
}

unsigned grid_for(long long n) { return (unsigned)std::max(1LL, (n + 255) / 256); }

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
                                  double* Mpp, double* Mhh, double* Z, int hZ, cudaStream_t st)
{
  cudaError_t e = cudaMemsetAsync(Mpp, 0, t.total * sizeof(double), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(Mhh, 0, t.total * sizeof(double), st);
  if (e != cudaSuccess) return e;
  if (!t.bra.empty() && t.max_blk_elems > 0) {
    dim3 grid(grid_for(t.max_blk_elems), (unsigned)t.bra.size());
    k_t222<<<grid, 256, 0, st>>>(s.dev, s.work, t.dev, X, Y, Mpp, Mhh, Z);
    count_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  int nn = s.norb * s.norb;
  k_t221<<<(nn + 7) / 8, 256, 0, st>>>(s.dev, t.dev, Mpp, Mhh, hZ, Z);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_tensor_ph(const Space& s, const TensorLayout& t, const double* Xbar, const double* Y, int hX,
                             int hY, double* Ybar, double* Zbar, double* Z, int hZ, cudaStream_t st)
{
  if (t.yb_bra.empty()) return cudaSuccess;
  dim3 gy(grid_for(std::max(1, t.yb_maxelems)), (unsigned)t.yb_bra.size());
  k_tpandya<<<gy, 256, 0, st>>>(s.dev, s.work, t.dev, Y, hY, Ybar);
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  dim3 gz(grid_for(std::max(1, t.zb_maxelems)), (unsigned)t.zb_bra.size());
  k_tzbar<<<gz, 256, 0, st>>>(s.dev, s.work, t.dev, Xbar, Ybar, hX, hY, Zbar, s.work.phase_tab);
  count_launch();
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if (t.bra.empty() || t.max_blk_elems == 0) return cudaSuccess;
  dim3 gi(grid_for(t.max_blk_elems), (unsigned)t.bra.size());
  k_tinv<<<gi, 256, 0, st>>>(s.dev, t.dev, Zbar, hZ, Z);
  count_launch();
  return cudaGetLastError();
}

}  // namespace imsrg
