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
// The element Z(ij, kl) of block (chb, chk) is a sum over the bra's
// partners and a sum over the ket's partners (src/TensorCommutators.cc:
// 158-312 with the reference's i == j and k == l shortcuts):
//   bra side:  sum_a X1(a,i) Y(aj, kl) + X1(a,j) Y(ia, kl)   (Y rows: chb kets)
//            + hat (-1)^.. 6j Y1(a,i) X(aj, kl) ...          (X rows: chk kets)
//   ket side: -sum_a X1(k,a) Y(ij, al) + ...                 (Y columns: chk kets)
//            + hat (-1)^.. 6j Y1(k,a) X(ij, la) ...          (X columns: chb kets)
// Each side is a list of (partner ket, coefficient) per bra or per ket,
// built once per block tile in shared memory; every element is then one FMA
// per list entry.  The pair normalisation factorises as (1/sqrt2)^(i==j)
// (1/sqrt2)^(k==l) and cancels the fixed side's sqrt(2), so each side carries
// its own factor.  Bra-side values are read as Y^T (the block transposed) and
// X^T = hX X (symmetry) so that lanes over kets read consecutive addresses.
struct T122Lists {
  int* yrow;
  double* ycoef;
  int* xrow;
  double* xcoef;
  int* ny;
  int* nx;
  int LY, LX;
};

// carve the lists of 32 bras (or kets) out of dynamic shared memory
__device__ __forceinline__ T122Lists t122_lists(unsigned char* smem, int LY, int LX)
{
  T122Lists L;
  L.ycoef = (double*)smem;
  L.xcoef = L.ycoef + 32 * LY;
  L.yrow = (int*)(L.xcoef + 32 * LX);
  L.xrow = L.yrow + 32 * LY;
  L.ny = L.xrow + 32 * LX;
  L.nx = L.ny + 32;
  L.LY = LY;
  L.LX = LX;
  return L;
}

// Entries of one bra (side 0: p = i, q = j; J, J' = J1, J2; Y rows in chb,
// X rows in chk) or one ket (side 1: p = k, q = l; Y columns in chk, X
// columns in chb), the lanes of a warp over the candidate partners, compacted
// by ballot into slot s of the lists.
__device__ void t122_build(const DevSpace& S, const DevTensor& T, const double* X, const double* Y, int side, int p,
                           int q, int chb, int chk, int hX, int s, T122Lists& L)
{
  const int lane = threadIdx.x & 31, N = S.norb, Lam = T.lam;
  const int J1 = ch_J(chb), J2 = ch_J(chk);
  const int jp = S.j2[p], jq = S.j2[q];
  const bool same = p == q;
  const double* X1 = X + 32;
  const double* Y1 = Y + 32;
  const int n1 = S.ob_count[p], n2 = same ? 0 : S.ob_count[q];
  const int n3 = T.tob_off[p + 1] - T.tob_off[p], n4 = same ? 0 : T.tob_off[q + 1] - T.tob_off[q];
  const int ntot = n1 + n2 + n3 + n4;
  const double hat = T.hat2[J1 * T.NJ + J2];
  const double fnorm = same ? kInvSqrt2 : 1.0;
  // the two X-side phases (odd1, odd2 for a bra; odd3, odd4 for a ket)
  const int oddA = side == 0 ? ((jp + jq) >> 1) + J2 + Lam : J1 - J2 + Lam;
  const int oddB = side == 0 ? J1 - J2 + Lam : ((jp + jq) >> 1) - J1 + Lam;
  int ny = 0, nx = 0;
  for (int c0 = 0; c0 < ntot; c0 += 32) {
    const int t = c0 + lane;
    int row = -1;
    double coef = 0.0;
    bool isx = false;
    if (t < n1 + n2) {
      // X one-body, Y two-body
      const bool first = t < n1;
      const int a = first ? S.ob_list[S.ob_start[p] + t] : S.ob_list[S.ob_start[q] + t - n1];
      const int ja = S.j2[a];
      if (side == 0) {
        // bra (a, q) or (p, a) in chb: coefficient X1(a, p) or X1(a, q)
        const int u = first ? a : p, v = first ? q : a;
        row = ket_in(S, chb, u, v);
        coef = X1[(long long)a * N + (first ? p : q)];
        coef = flip(coef, u > v ? ((S.j2[u] + S.j2[v]) >> 1) + 1 + J1 : 0);
        if (u == v) coef *= kSqrt2t;
        if (same) coef *= 2.0;
      } else {
        // ket (a, q) or (p, a) in chk: coefficient -X1(p, a) or -X1(q, a)
        const int u = first ? a : p, v = first ? q : a;
        row = ket_in(S, chk, u, v);
        coef = -X1[(long long)(first ? p : q) * N + a];
        coef = flip(coef, u > v ? ((S.j2[u] + S.j2[v]) >> 1) + 1 + J2 : 0);
        if (u == v) coef *= kSqrt2t;
        if (same) coef *= 2.0;
      }
      (void)ja;
      coef *= fnorm;
    } else if (t < ntot) {
      // Y one-body, X two-body
      isx = true;
      const bool first = t < n1 + n2 + n3;
      const int a = first ? T.tob_list[T.tob_off[p] + t - n1 - n2] : T.tob_list[T.tob_off[q] + t - n1 - n2 - n3];
      const int ja = S.j2[a];
      double sg;
      if (side == 0) {
        // bra (a, q) or (a, p) of chk, X rows: -6j{J2 J1 lam; jp ja jq} Y1(a, p), +6j{..; jq ja jp} Y1(a, q)
        const int u = a, v = first ? q : p;
        row = ket_in(S, chk, u, v);
        coef = first ? -sixjA(T, J2, J1, jp, ja, jq) * Y1[(long long)a * N + p]
                     : sixjA(T, J2, J1, jq, ja, jp) * Y1[(long long)a * N + q];
        coef = flip(coef, u > v ? ((S.j2[u] + S.j2[v]) >> 1) + 1 + J2 : 0);
        if (u == v) coef *= kSqrt2t;
      } else {
        // ket (q, a) or (p, a) of chb, X columns: -6j{J1 J2 lam; jp ja jq} Y1(p, a), +6j{..; jq ja jp} Y1(q, a)
        const int u = first ? q : p, v = a;
        row = ket_in(S, chb, u, v);
        coef = first ? -sixjA(T, J1, J2, jp, ja, jq) * Y1[(long long)p * N + a]
                     : sixjA(T, J1, J2, jq, ja, jp) * Y1[(long long)q * N + a];
        coef = flip(coef, u > v ? ((S.j2[u] + S.j2[v]) >> 1) + 1 + J1 : 0);
        if (u == v) coef *= kSqrt2t;
      }
      // hat (-1)^odd; for p == q the partner list repeats with the opposite
      // sign, which folds into (-1)^oddA - (-1)^oddB
      if (same)
        sg = (double)(iphase(oddA) - iphase(oddB));
      else
        sg = (double)iphase(first ? oddA : oddB);
      coef *= hat * sg * fnorm;
      if (side == 0 && hX < 0) coef = -coef;  // X^T = hX X
    }
    const bool vy = row >= 0 && !isx && coef != 0.0, vx = row >= 0 && isx && coef != 0.0;
    const unsigned my = __ballot_sync(0xffffffffu, vy), mx = __ballot_sync(0xffffffffu, vx);
    const unsigned below = (1u << lane) - 1;
    if (vy) {
      const int pos = ny + __popc(my & below);
      L.yrow[s * L.LY + pos] = row;
      L.ycoef[s * L.LY + pos] = coef;
    }
    if (vx) {
      const int pos = nx + __popc(mx & below);
      L.xrow[s * L.LX + pos] = row;
      L.xcoef[s * L.LX + pos] = coef;
    }
    ny += __popc(my);
    nx += __popc(mx);
  }
  if (lane == 0) {
    L.ny[s] = ny;
    L.nx[s] = nx;
  }
}

// bra side: a block per (32 bras, block); warp w builds the lists of bras
// w, w + 8, ...; then for each 32-ket chunk the warps take 4 bras each, lanes
// over kets (reads of Y^T and X^T rows), results through a shared tile so the
// Z update is coalesced over bras
__global__ void __launch_bounds__(256) k_t122_bra(DevSpace S, DevTensor T, const double* __restrict__ X,
                                                  const double* __restrict__ Y, const double* __restrict__ YT, int hX,
                                                  double* __restrict__ Z, int LY, int LX)
{
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ double tile[32][33];
  const int blk = blockIdx.y;
  const int chb = T.bra[blk], chk = T.ket[blk];
  const int nb = S.ch_n[chb], nk = S.ch_n[chk];
  const int ib0 = blockIdx.x * 32;
  if (ib0 >= nb) return;
  T122Lists L = t122_lists(smem, LY, LX);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int b = warp; b < 32; b += 8) {
    const int ib = ib0 + b;
    if (ib < nb)
      t122_build(S, T, X, Y, 0, S.ket_p[S.ch_kofs[chb] + ib], S.ket_q[S.ch_kofs[chb] + ib], chb, chk, hX, b, L);
    else if (lane == 0)
      L.ny[b] = L.nx[b] = 0;
  }
  __syncthreads();
  const double* yt = YT + T.off[blk];         // nb x nk transposed: yt[row nk + ik]
  const double* xk = X + S.ch_off[chk];        // symmetric: X(row, ik) = hX xk[row nk + ik]
  for (int k0 = 0; k0 < nk; k0 += 32) {
    const int ik = k0 + lane;
    for (int b = warp; b < 32; b += 8) {
      double z = 0.0;
      if (ik < nk) {
        const int ny = L.ny[b], nx = L.nx[b];
        for (int e = 0; e < ny; ++e) z = fma(L.ycoef[b * LY + e], yt[(long long)L.yrow[b * LY + e] * nk + ik], z);
        for (int e = 0; e < nx; ++e) z = fma(L.xcoef[b * LX + e], xk[(long long)L.xrow[b * LX + e] * nk + ik], z);
      }
      tile[b][lane] = z;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 32 * 32; e += 256) {
      const int kk = e >> 5, b = e & 31;
      if (ib0 + b < nb && k0 + kk < nk) Z[T.off[blk] + (long long)(k0 + kk) * nb + ib0 + b] += tile[b][kk];
    }
    __syncthreads();
  }
}

// ket side: a block per (32 kets, block); lists per ket, then warps take 4
// kets each, lanes over bras (reads of Y's and X's columns), Z += directly
__global__ void __launch_bounds__(256) k_t122_ket(DevSpace S, DevTensor T, const double* __restrict__ X,
                                                  const double* __restrict__ Y, int hX, double* __restrict__ Z,
                                                  int LY, int LX)
{
  extern __shared__ __align__(16) unsigned char smem[];
  const int blk = blockIdx.y;
  const int chb = T.bra[blk], chk = T.ket[blk];
  const int nb = S.ch_n[chb], nk = S.ch_n[chk];
  const int ik0 = blockIdx.x * 32;
  if (ik0 >= nk) return;
  T122Lists L = t122_lists(smem, LY, LX);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int c = warp; c < 32; c += 8) {
    const int ik = ik0 + c;
    if (ik < nk)
      t122_build(S, T, X, Y, 1, S.ket_p[S.ch_kofs[chk] + ik], S.ket_q[S.ch_kofs[chk] + ik], chb, chk, hX, c, L);
    else if (lane == 0)
      L.ny[c] = L.nx[c] = 0;
  }
  __syncthreads();
  const double* yb = Y + T.off[blk];   // nb x nk: yb[col nb + ib]
  const double* xb = X + S.ch_off[chb];  // nb x nb: xb[col nb + ib]
  for (int c = warp; c < 32; c += 8) {
    const int ik = ik0 + c;
    if (ik >= nk) continue;
    const int ny = L.ny[c], nx = L.nx[c];
    for (int ib = lane; ib < nb; ib += 32) {
      double z = 0.0;
      for (int e = 0; e < ny; ++e) z = fma(L.ycoef[c * LY + e], yb[(long long)L.yrow[c * LY + e] * nb + ib], z);
      for (int e = 0; e < nx; ++e) z = fma(L.xcoef[c * LX + e], xb[(long long)L.xrow[c * LX + e] * nb + ib], z);
      Z[T.off[blk] + (long long)ik * nb + ib] += z;
    }
  }
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
  if (!nj.p) return 0.0;
  // the row's J1 window is this sum's J3 range (both |ja - jl| .. ja + jl),
  // and J4 - J3 + lam stays in [0, w): every slot below is in the table
  const int J3min = abs(ja - jl) >> 1, J3max = (ja + jl) >> 1;
  const int J4lo = abs(jk - jb) >> 1, J4hi = (jk + jb) >> 1;
  const long long st = nj.stride;
  double acc = 0.0;
  for (int J3 = J3min; J3 <= J3max; ++J3) {
    const int J4min = max(J4lo, abs(J3 - Lam)), J4max = min(J4hi, J3 + Lam);
    if (J4min > J4max) continue;
    long long k9 = ((long long)(J3 - J3min) * w + (J4min - J3 + Lam)) * st;
    int e = (J3 - J3min) * w + (J4min - J3 + Lam);
    int odd = ((jb + jl) >> 1) + J2 + J4min;
    // the table's zeros (the reference's skipped terms) add exactly 0: no
    // branch, so the loads of consecutive terms can be in flight together
    for (int J4 = J4min; J4 <= J4max; ++J4, k9 += st, ++e, ++odd) acc = fma(flip(nj.p[k9], odd), in[e], acc);
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

__global__ void __launch_bounds__(32 * kTqWarps, 6) k_tinv_q(DevSpace S, DevTensor T, const double* __restrict__ Zb,
                                                         int hZ, double* __restrict__ Z,
                                                         const int2* __restrict__ tq, long long nq, int slots)
{
  extern __shared__ double s_in[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long qi = blockIdx.x * (long long)kTqWarps + warp;
  if (qi >= nq) return;
  // per warp: the two sums' gathered values, then the owned output slots
  double* in1 = s_in + (size_t)warp * 3 * slots;
  double* in2 = in1 + slots;
  int* own = reinterpret_cast<int*>(in2 + slots);
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
  // the slots this quadruple owns, compacted (ballot) so every lane of the
  // sums below has one
  int nown = 0;
  for (int c0 = 0; c0 < nJ1 * w; c0 += 32) {
    const int t = c0 + lane;
    bool ok = false;
    if (t < nJ1 * w) {
      const int J1 = J1min + t / w, J2 = J1 - Lam + t % w;
      if (J2 >= J2lo && J2 <= J2hi && J1 < S.NJ && J2 < S.NJ) {
        const int ib = S.ketJ_loc[J1 * S.nkets + kb], ik = S.ketJ_loc[J2 * S.nkets + kk];
        const int chb = chan_index(J1, pb, tb), chk = chan_index(J2, pk, tk);
        ok = ib >= 0 && ik >= 0 && !(chb > chk || (chb == chk && ik < ib)) && T.lookup[chb * S.nch + chk] >= 0;
      }
    }
    const unsigned m = __ballot_sync(0xffffffffu, ok);
    if (ok) own[nown + __popc(m & ((1u << lane) - 1))] = t;
    nown += __popc(m);
  }
  __syncwarp();
  for (int x = lane; x < nown; x += 32) {
    const int t = own[x];
    const int J1 = J1min + t / w, J2 = J1 - Lam + t % w;
    const int ib = S.ketJ_loc[J1 * S.nkets + kb], ik = S.ketJ_loc[J2 * S.nkets + kk];
    const int chb = chan_index(J1, pb, tb), chk = chan_index(J2, pk, tk);
    const int blk = T.lookup[chb * S.nch + chk];
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
  // slots bounds a sum's gathered values and the output slots alike
  const int slots = t.tq_max_j3 * (2 * t.lam + 1);
  const size_t smem = (size_t)kTqWarps * 3 * slots * sizeof(double);
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

cudaError_t launch_tensor_122(const Space& s, const TensorLayout& t, const double* X, const double* Y, int hX,
                              double* YT, double* Z, cudaStream_t st)
{
  if (t.bra.empty() || t.max_blk_elems == 0) return cudaSuccess;
  cudaError_t e;
  // Y^T for the bra side
  k_ttranspose<<<dim3((unsigned)t.max_tiles32, (unsigned)t.bra.size()), dim3(32, 8), 0, st>>>(s.dev, t.dev, Y, YT);
  count_launch();
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  const int LY = std::max(1, 2 * t.max_ob), LX = std::max(1, 2 * t.max_tob);
  const size_t smem = (size_t)32 * (LY + LX) * (sizeof(double) + sizeof(int)) + 64 * sizeof(int);
  if (smem > 40 * 1024) {
    if ((e = cudaFuncSetAttribute(k_t122_bra, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) !=
            cudaSuccess ||
        (e = cudaFuncSetAttribute(k_t122_ket, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess)
      return e;
  }
  int maxn = 0;
  for (int c = 0; c < s.nch; ++c) maxn = std::max(maxn, s.ch[c].n());
  const dim3 grid((unsigned)((maxn + 31) / 32), (unsigned)t.bra.size());
  k_t122_bra<<<grid, 256, smem, st>>>(s.dev, t.dev, X, Y, YT, hX, Z, LY, LX);
  count_launch();
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  k_t122_ket<<<grid, 256, smem, st>>>(s.dev, t.dev, X, Y, hX, Z, LY, LX);
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

// Operator::Norm of a tensor operator: blocks 0 .. n2-1 sum their chunk's
// squares times its weight; block n2 sums the weighted one-body squares
__global__ void k_tnorm(const double* __restrict__ A, const long long* __restrict__ off,
                        const int* __restrict__ len, const double* __restrict__ w2, int n2,
                        const int* __restrict__ idx1, const double* __restrict__ w1, int n1,
                        double* __restrict__ partial)
{
  __shared__ double red[32];
  const int c = blockIdx.x;
  double s = 0.0;
  if (c < n2) {
    const double* p = A + off[c];
    for (int t = threadIdx.x; t < len[c]; t += blockDim.x) s = fma(p[t], p[t], s);
  } else {
    for (int t = threadIdx.x; t < n1; t += blockDim.x) {
      const double v = A[idx1[t]];
      s = fma(v * v, w1[t], s);
    }
  }
  s = wsum(s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    v = wsum(v);
    if (threadIdx.x == 0) partial[c] = c < n2 ? v * w2[c] : v;
  }
}

cudaError_t launch_tensor_norm(const TensorLayout& t, const double* A, double* partial, cudaStream_t st)
{
  const int n2 = (int)t.nrm2_off.size();
  k_tnorm<<<n2 + 1, 256, 0, st>>>(A, t.d_nrm2_off, t.d_nrm2_len, t.d_nrm2_w, n2, t.d_nrm1_idx, t.d_nrm1_w,
                                  (int)t.nrm1_idx.size(), partial);
  count_launch();
  return cudaGetLastError();
}

}  // namespace imsrg
