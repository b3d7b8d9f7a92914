// FP64 kernels of the scalar IMSRG(2) commutator terms other than the dense
// channel products: comm110ss, comm111ss, comm220ss, comm121ss, the one-body
// part of comm221ss, comm122ss, the forward and inverse Pandya
// transformations of comm222_phss, and the operator algebra of the BCH series.
// Each kernel states the reference lines it reproduces.
#include <cuda_runtime.h>

#include <algorithm>

#include "dfloat.cuh"
#include "kernels.cuh"
#include "prof.hpp"

namespace imsrg {

static constexpr double kSqrt2 = 1.4142135623730950488;

// grouped launches over several pairs of the same structure (batches): the
// pair is blockIdx.z and its operands sit at byte offsets zo[z * kZRoles +
// role] from the pointers the launch passes (zo null: one pair, no shift)
template <class T>
__device__ __forceinline__ T* zsh(T* p, const long long* zo, int role)
{
  return zo ? (T*)((char*)p + zo[blockIdx.z * kZRoles + role]) : p;
}
static constexpr int kMaxChannels = 6 * 64;  // 2b / CC channels: 6 (j2max + 1), j2max <= 63

__device__ __forceinline__ double warp_sum(double v)
{
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ---------------------------------------------------------------- 111 + 110
// Z1 += X1 Y1 - Y1 X1  (comm111ss, src/Commutator.cc:644-649) and
// Z0 += sum_a (2j_a+1) n_a (X1 Y1 - Y1 X1)_aa over holes (comm110ss, :564-581)
__global__ void k_comm111_110(DevSpace S, const double* __restrict__ X, const double* __restrict__ Y,
                              double* __restrict__ Z, int do111, int do110, const long long* __restrict__ zo)
{
  X = zsh(X, zo, ZR_X);
  Y = zsh(Y, zo, ZR_Y);
  Z = zsh(Z, zo, ZR_Z);
  int N = S.norb;
  int i = blockIdx.x;
  const double* X1 = X + 32;
  const double* Y1 = Y + 32;
  for (int j = threadIdx.x; j < N; j += blockDim.x) {
    double xy = 0.0, yx = 0.0;
    for (int b = 0; b < N; ++b) {
      xy = fma(X1[(size_t)b * N + i], Y1[(size_t)j * N + b], xy);
      yx = fma(Y1[(size_t)b * N + i], X1[(size_t)j * N + b], yx);
    }
    double v = xy - yx;
    if (do111) Z[32 + (size_t)j * N + i] += v;
    if (do110 && j == i) {
      double oc = S.occ[i];
      if (oc >= 1e-6) atomicAdd(Z, (S.j2[i] + 1) * oc * v);
    }
  }
}

// ---------------------------------------------------------------------- 220
// Z0 += 2 sum_ch (2J+1) sum_{h in hh} n_h n_h' (X_{h,nbar} (nbar nbar) Y_{nbar,h})
// (comm220ss, src/Commutator.cc:601-631); one warp per hh ket.
__global__ void k_comm220(DevSpace S, DevWork W, const double* __restrict__ X, const double* __restrict__ Y,
                          double* __restrict__ Z, int hX, const long long* __restrict__ zo)
{
  X = zsh(X, zo, ZR_X);
  Y = zsh(Y, zo, ZR_Y);
  Z = zsh(Z, zo, ZR_Z);
  int item = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  int lane = threadIdx.x & 31;
  if (item >= W.n220) return;
  int ch = W.items220[2 * item], h = W.items220[2 * item + 1];
  int n = S.ch_n[ch];
  long long off = S.ch_off[ch];
  const double* xc = X + off + (long long)h * n;  // X(h,k) = hX X(k,h)
  const double* yc = Y + off + (long long)h * n;  // Y(k,h)
  const double* w = W.ket_wpp + S.ch_kofs[ch];
  double d = 0.0;
  for (int k = lane; k < n; k += 32) d = fma(xc[k] * w[k], yc[k], d);
  d = warp_sum(d);
  if (lane == 0) {
    int J = ch / 6;
    double nn = W.ket_nn[S.ch_kofs[ch] + h];
    atomicAdd(Z, 2.0 * (2 * J + 1) * hX * d * nn);
  }
}

// ---------------------------------------------------------------------- 121
// TwoBodyME::GetTBMEmonopole (src/TwoBodyME.cc:615-682)
__device__ double dev_monopole(const DevSpace& S, const double* op, int a, int b, int c, int d)
{
  int pab = (S.l[a] + S.l[b]) & 1, pcd = (S.l[c] + S.l[d]) & 1;
  if (pab != pcd) return 0.0;
  if (S.tz2[a] + S.tz2[b] != S.tz2[c] + S.tz2[d]) return 0.0;
  int ja = S.j2[a], jb = S.j2[b];
  int jmin = abs(ja - jb) / 2, jmax = (ja + jb) / 2;
  double mon = 0.0;
  for (int J = jmin; J <= jmax; ++J) mon += (2 * J + 1) * dev_tbme_J_norm(S, op, J, a, b, c, d);
  mon /= (double)((ja + 1) * (jb + 1));
  if (a == b) mon *= kSqrt2;
  if (c == d) mon *= kSqrt2;
  return mon;
}

// comm121ss, src/Commutator.cc:670-728: one warp per (i <= j) pair, lanes over
// (hole a, b in the one-body channel of a).
__global__ void k_comm121(DevSpace S, DevWork W, const int* __restrict__ holes, int nholes,
                          const double* __restrict__ X, const double* __restrict__ Y, double* __restrict__ Z, int hZ,
                          const long long* __restrict__ zo)
{
  X = zsh(X, zo, ZR_X);
  Y = zsh(Y, zo, ZR_Y);
  Z = zsh(Z, zo, ZR_Z);
  int item = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  int lane = threadIdx.x & 31;
  if (item >= W.npairs1b) return;
  int i = W.pairs1b[2 * item], j = W.pairs1b[2 * item + 1];
  int N = S.norb;
  const double* X1 = X + 32;
  const double* Y1 = Y + 32;
  double z = 0.0;
  // enumerate (a, b) pairs: a = holes[ia], b = ob_list[ob_start[a] + ib]
  int total = 0;
  for (int ia = 0; ia < nholes; ++ia) total += S.ob_count[holes[ia]];
  for (int t = lane; t < total; t += 32) {
    int ia = 0, rem = t;
    while (rem >= S.ob_count[holes[ia]]) {
      rem -= S.ob_count[holes[ia]];
      ++ia;
    }
    int a = holes[ia];
    int b = S.ob_list[S.ob_start[a] + rem];
    double nanb = S.occ[a] * (1.0 - S.occ[b]);
    if (fabs(nanb) < 1e-6) continue;
    int jja = S.j2[a], jjb = S.j2[b];
    double ybiaj = dev_monopole(S, Y, b, i, a, j);
    double yaibj = dev_monopole(S, Y, a, i, b, j);
    z += (jjb + 1) * nanb * X1[(size_t)b * N + a] * ybiaj;
    z -= (jja + 1) * nanb * X1[(size_t)a * N + b] * yaibj;
    z -= (jjb + 1) * nanb * Y1[(size_t)b * N + a] * dev_monopole(S, X, b, i, a, j);
    z += (jja + 1) * nanb * Y1[(size_t)a * N + b] * dev_monopole(S, X, a, i, b, j);
  }
  z = warp_sum(z);
  if (lane == 0) {
    Z[32 + (size_t)j * N + i] += z;
    if (i != j) Z[32 + (size_t)i * N + j] += hZ * z;
  }
}

// -------------------------------------------------------------- 221 (1b)
// One-body part of comm222_pp_hh_221ss / comm221ss (src/Commutator.cc:1250-1294):
// Z1_ij += 1/(2j_i+1) sum_c sum_J (2J+1) [n_c Mpp^J_{ci,cj} + nbar_c Mhh^J_{ci,cj}],
// with the needed elements of the symmetrised intermediates
// Mpp = X P Y + hZ (X P Y)^T, Mhh = X (nn) Y + hZ (...)^T (ConstructScalarMpp_Mhh,
// src/Commutator.cc:1170-1194) evaluated as dot products.  One warp per (i, j, c).
__device__ __forceinline__ double warp_dot_w(const double* a, const double* b, const double* w, int n, int lane)
{
  double d = 0.0;
  for (int k = lane; k < n; k += 32) d = fma(a[k] * w[k], b[k], d);
  return warp_sum(d);
}

__device__ __forceinline__ double warp_dot_list(const double* a, const double* b, const double* w, const int* idx,
                                                int m, int lane)
{
  double d = 0.0;
  for (int t = lane; t < m; t += 32) {
    int k = idx[t];
    d = fma(a[k] * w[k], b[k], d);
  }
  return warp_sum(d);
}

// With Mz != nullptr, Mz holds the two-body blocks of Mpp - Mhh (symmetrised),
// i.e. exactly what the ladder product added to a zeroed Z, and
// Mpp = Mz + Mhh needs only the short hh dot products.
__global__ void k_comm221_1b(DevSpace S, DevWork W, const double* __restrict__ X, const double* __restrict__ Y,
                             double* __restrict__ Z, int hX, int hZ, const double* __restrict__ Mz)
{
  int item = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  int lane = threadIdx.x & 31;
  if (item >= W.n221) return;
  int i = W.items221[3 * item], j = W.items221[3 * item + 1], c = W.items221[3 * item + 2];
  int N = S.norb;
  double nc = S.occ[c], nbarc = 1.0 - nc;
  int jc = S.j2[c], ji = S.j2[i], jj = S.j2[j];
  int Jmin = max(abs(jc - ji), abs(jc - jj)) / 2;
  int Jmax = (jc + min(ji, jj)) / 2;
  int par = (S.l[c] + S.l[i]) & 1, tz = (S.tz2[c] + S.tz2[i]) / 2;
  int kci = ket_index(N, min(c, i), max(c, i)), kcj = ket_index(N, min(c, j), max(c, j));
  double z = 0.0;
  for (int J = Jmin; J <= Jmax; ++J) {
    int r = S.ketJ_loc[J * S.nkets + kci], s = S.ketJ_loc[J * S.nkets + kcj];
    if (r < 0 || s < 0) continue;
    int ch = chan_index(J, par, tz);
    int n = S.ch_n[ch];
    long long off = S.ch_off[ch];
    const double* xr = X + off + (long long)r * n;
    const double* xs = X + off + (long long)s * n;
    const double* yr = Y + off + (long long)r * n;
    const double* ys = Y + off + (long long)s * n;
    double ph = 1.0;
    if (c > i) ph *= iphase((jc + ji) / 2 + 1 + J);
    if (c > j) ph *= iphase((jc + jj) / 2 + 1 + J);
    double nrm = 1.0;
    if (c == i) nrm *= kSqrt2;
    if (c == j) nrm *= kSqrt2;
    double fac = (2 * J + 1) * ph * nrm;
    const bool need_pp = fabs(nc) > 1e-9, need_hh = fabs(nbarc) > 1e-9;
    double mhh = 0.0;
    if (need_hh || (need_pp && Mz)) {
      const double* w = W.ket_nn + S.ch_kofs[ch];
      const int* hh = W.hh_list + W.hh_off[ch];
      int nhh = W.hh_off[ch + 1] - W.hh_off[ch];
      double m_rs = hX * warp_dot_list(xr, ys, w, hh, nhh, lane);
      double m_sr = (r == s) ? m_rs : hX * warp_dot_list(xs, yr, w, hh, nhh, lane);
      mhh = m_rs + hZ * m_sr;
    }
    if (need_pp) {
      double mpp;
      if (Mz) {
        mpp = Mz[off + (long long)s * n + r] + mhh;
      } else {
        const double* w = W.ket_wpp + S.ch_kofs[ch];
        double m_rs = hX * warp_dot_w(xr, ys, w, n, lane);
        double m_sr = (r == s) ? m_rs : hX * warp_dot_w(xs, yr, w, n, lane);
        mpp = m_rs + hZ * m_sr;
      }
      z += fac * nc * mpp;
    }
    if (need_hh) z += fac * nbarc * mhh;
  }
  if (lane == 0 && z != 0.0) {
    double v = z / (ji + 1.0);
    atomicAdd(Z + 32 + (size_t)j * N + i, v);
    if (i != j) atomicAdd(Z + 32 + (size_t)i * N + j, hZ * v);
  }
}

// double-float arithmetic: dfloat.cuh

// FP64 arena -> (hi, lo) pairs, integer instructions only
__global__ void k_to_ff(const double* __restrict__ src, float2* __restrict__ dst, long long n,
                        const long long* __restrict__ zo, int rsrc, int rdst)
{
  src = zsh(src, zo, rsrc);
  dst = zsh(dst, zo, rdst);
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long stride = (long long)gridDim.x * blockDim.x;
  // four loads in flight per thread, then the conversions and stores
  for (; i + 3 * stride < n; i += 4 * stride) {
    double v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) v[u] = src[i + u * stride];
#pragma unroll
    for (int u = 0; u < 4; ++u) dst[i + u * stride] = d2ff(v[u]);
  }
  for (; i < n; i += stride) dst[i] = d2ff(src[i]);
}

// ---------------------------------------------------------------------- 122
// comm122ss, src/Commutator.cc:837-932.  W2(:, ij) = sum_items f (Y2(:,loc) X1(a,src)
// - X2(:,loc) Y1(a,src)); one block per column, threads over rows, in
// double-float arithmetic from (hi, lo) copies of X2 and Y2; W2 is stored as
// (hi, lo) pairs.
__global__ void __launch_bounds__(128) k_comm122_w_df(DevSpace S, DevWork W, const double* __restrict__ X,
                                                      const double* __restrict__ Y, const float2* __restrict__ Xf,
                                                      const float2* __restrict__ Yf, float2* __restrict__ W2,
                                                      const long long* __restrict__ zo)
{
  X = zsh(X, zo, ZR_X);
  Y = zsh(Y, zo, ZR_Y);
  Xf = zsh(Xf, zo, ZR_XF);
  Yf = zsh(Yf, zo, ZR_YF);
  W2 = zsh(W2, zo, ZR_W2);
  __shared__ float2 cx[32], cy[32];
  __shared__ int cl[32];
  int col = blockIdx.x;
  if (col >= W.ncols122) return;
  int ch = W.cols122[4 * col], ij = W.cols122[4 * col + 1];
  int first = W.cols122[4 * col + 2], cnt = min(W.cols122[4 * col + 3], 32);
  int n = S.ch_n[ch];
  long long off = S.ch_off[ch];
  int N = S.norb;
  if (threadIdx.x < cnt) {
    int t = threadIdx.x;
    int a = W.it122_a[first + t], src = W.it122_src[first + t];
    double f = W.it122_f[first + t];
    cx[t] = d2ff(X[32 + (size_t)src * N + a] * f);   //  X1(a,src) f multiplies Y2
    cy[t] = d2ff(-Y[32 + (size_t)src * N + a] * f);  // -Y1(a,src) f multiplies X2
    cl[t] = W.it122_loc[first + t];
  }
  __syncthreads();
  // two rows per thread and pass (r and r + blockDim.x): the item's
  // coefficients and column address are read once for both
  for (int r0 = threadIdx.x; r0 < n; r0 += 2 * blockDim.x) {
    const int r1 = r0 + blockDim.x;
    const bool two = r1 < n;
    float s0 = 0.f, c0 = 0.f, s1 = 0.f, c1 = 0.f;
    for (int t = 0; t < cnt; ++t) {
      const long long e = off + (long long)cl[t] * n + r0;
      const float2 ax = cx[t], ay = cy[t];
      df_fma(ax, Yf[e], s0, c0);
      df_fma(ay, Xf[e], s0, c0);
      if (two) {
        df_fma(ax, Yf[e + blockDim.x], s1, c1);
        df_fma(ay, Xf[e + blockDim.x], s1, c1);
      }
    }
    float hi = __fadd_rn(s0, c0);
    float lo = __fsub_rn(c0, __fsub_rn(hi, s0));
    W2[off + (long long)ij * n + r0] = make_float2(hi, lo);
    if (two) {
      hi = __fadd_rn(s1, c1);
      lo = __fsub_rn(c1, __fsub_rn(hi, s1));
      W2[off + (long long)ij * n + r1] = make_float2(hi, lo);
    }
  }
}

// Z2 -= W2 + hZ W2^T with W2 in (hi, lo) pairs, per channel in 32x32 tiles:
// the pair sum in double-float, converted with integer instructions, so the
// only FP64 instruction per element is the subtraction from Z2
__global__ void k_sym_subtract_ff(DevSpace S, const float2* __restrict__ W2, double* __restrict__ Z, int hZ,
                                  const int* __restrict__ tiles, int ntiles, const long long* __restrict__ zo)
{
  W2 = zsh(W2, zo, ZR_W2);
  Z = zsh(Z, zo, ZR_Z);
  __shared__ float2 tt[32][33];
  int t = blockIdx.x;
  if (t >= ntiles) return;
  int ch = tiles[3 * t], ti = tiles[3 * t + 1], tj = tiles[3 * t + 2];
  int n = S.ch_n[ch];
  long long off = S.ch_off[ch];
  int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (int yy = ty; yy < 32; yy += 8) {
    int r = tj * 32 + tx, c = ti * 32 + yy;
    float2 v = make_float2(0.f, 0.f);
    if (r < n && c < n) v = W2[off + (long long)c * n + r];
    tt[yy][tx] = v;
  }
  // the direct W2 values and the old Z values of this thread's four
  // elements are all requested before the first store (loads in flight
  // together; the kernel is bound by their latency)
  float2 w[4];
  double zo4[4];
  const int r = ti * 32 + tx;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int c = tj * 32 + ty + 8 * k;
    w[k] = make_float2(0.f, 0.f);
    zo4[k] = 0.0;
    if (r < n && c < n) {
      w[k] = W2[off + (long long)c * n + r];
      zo4[k] = Z[off + (long long)c * n + r];
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int yy = ty + 8 * k, c = tj * 32 + yy;
    if (r < n && c < n) {
      float2 u = tt[tx][yy];
      if (hZ < 0) {
        u.x = -u.x;
        u.y = -u.y;
      }
      float hi, lo;
      df_add(w[k].x, w[k].y, u.x, u.y, hi, lo);
      Z[off + (long long)c * n + r] = zo4[k] - ff2d(hi, lo);
    }
  }
}

// Same one-body part when Mpp - Mhh is already in Mz (the ladder product added
// to a zeroed Z): one block of 128 threads per (i <= j) pair, threads over c;
// each thread forms the short Mhh dot products (hh kets only) itself, and the
// block reduces once.  (A warp per pair left 5% of the warps of the GPU
// active: there are only a few hundred pairs.)
__global__ void k_comm221_1b_mz(DevSpace S, DevWork W, const double* __restrict__ X, const double* __restrict__ Y,
                                double* __restrict__ Z, int hX, int hZ, const double* __restrict__ Mz,
                                const long long* __restrict__ zo)
{
  X = zsh(X, zo, ZR_X);
  Y = zsh(Y, zo, ZR_Y);
  Z = zsh(Z, zo, ZR_Z);
  Mz = zsh(Mz, zo, ZR_Z);
  __shared__ double red[4];
  const int item = blockIdx.x;
  const int lane = threadIdx.x & 31;
  if (item >= W.npairs1b) return;
  const int i = W.pairs1b[2 * item], j = W.pairs1b[2 * item + 1];
  const int N = S.norb;
  const int ji = S.j2[i], jj = S.j2[j];
  double z = 0.0;
  for (int c = threadIdx.x; c < N; c += blockDim.x) {
    const double nc = S.occ[c], nbarc = 1.0 - nc;
    const bool need_pp = fabs(nc) > 1e-9, need_hh = fabs(nbarc) > 1e-9;
    const int jc = S.j2[c];
    const int Jmin = max(abs(jc - ji), abs(jc - jj)) / 2;
    const int Jmax = (jc + min(ji, jj)) / 2;
    const int par = (S.l[c] + S.l[i]) & 1, tz = (S.tz2[c] + S.tz2[i]) / 2;
    const int kci = ket_index(N, min(c, i), max(c, i)), kcj = ket_index(N, min(c, j), max(c, j));
    for (int J = Jmin; J <= Jmax; ++J) {
      int r = S.ketJ_loc[J * S.nkets + kci], s = S.ketJ_loc[J * S.nkets + kcj];
      if (r < 0 || s < 0) continue;
      int ch = chan_index(J, par, tz);
      int n = S.ch_n[ch];
      long long off = S.ch_off[ch];
      const double* xr = X + off + (long long)r * n;
      const double* xs = X + off + (long long)s * n;
      const double* yr = Y + off + (long long)r * n;
      const double* ys = Y + off + (long long)s * n;
      const double* w = W.ket_nn + S.ch_kofs[ch];
      const int* hh = W.hh_list + W.hh_off[ch];
      const int nhh = W.hh_off[ch + 1] - W.hh_off[ch];
      double m_rs = 0.0, m_sr = 0.0;
      for (int t = 0; t < nhh; ++t) {
        int k = hh[t];
        double wk = w[k];
        m_rs = fma(xr[k] * wk, ys[k], m_rs);
        m_sr = fma(xs[k] * wk, yr[k], m_sr);
      }
      if (r == s) m_sr = m_rs;
      double mhh = hX * (m_rs + hZ * m_sr);
      double ph = 1.0;
      if (c > i) ph *= iphase((jc + ji) / 2 + 1 + J);
      if (c > j) ph *= iphase((jc + jj) / 2 + 1 + J);
      double nrm = 1.0;
      if (c == i) nrm *= kSqrt2;
      if (c == j) nrm *= kSqrt2;
      double fac = (2 * J + 1) * ph * nrm;
      if (need_pp) z += fac * nc * (Mz[off + (long long)s * n + r] + mhh);
      if (need_hh) z += fac * nbarc * mhh;
    }
  }
  z = warp_sum(z);
  if (lane == 0) red[threadIdx.x >> 5] = z;
  __syncthreads();
  if (threadIdx.x == 0) {
    z = red[0] + red[1] + red[2] + red[3];
    double v = z / (ji + 1.0);
    Z[32 + (size_t)j * N + i] += v;
    if (i != j) Z[32 + (size_t)i * N + j] += hZ * v;
  }
}

// ---------------------------------------------------------------------- 122
// comm122ss, src/Commutator.cc:837-932.  W2(:, ij) = sum_items f (Y2(:,loc) X1(a,src)
// - X2(:,loc) Y1(a,src)); one block per column, threads over rows (FP64).
__global__ void k_comm122_w(DevSpace S, DevWork W, const double* __restrict__ X, const double* __restrict__ Y,
                            double* __restrict__ W2, const long long* __restrict__ zo)
{
  X = zsh(X, zo, ZR_X);
  Y = zsh(Y, zo, ZR_Y);
  W2 = zsh(W2, zo, ZR_W2);
  int col = blockIdx.x;
  if (col >= W.ncols122) return;
  int ch = W.cols122[4 * col], ij = W.cols122[4 * col + 1];
  int first = W.cols122[4 * col + 2], cnt = W.cols122[4 * col + 3];
  int n = S.ch_n[ch];
  long long off = S.ch_off[ch];
  int N = S.norb;
  for (int r = threadIdx.x; r < n; r += blockDim.x) {
    double w = 0.0;
    for (int t = 0; t < cnt; ++t) {
      int loc = W.it122_loc[first + t];
      int a = W.it122_a[first + t], src = W.it122_src[first + t];
      double f = W.it122_f[first + t];
      double x1 = X[32 + (size_t)src * N + a] * f;
      double y1 = Y[32 + (size_t)src * N + a] * f;
      w = fma(Y[off + (long long)loc * n + r], x1, w);
      w = fma(-X[off + (long long)loc * n + r], y1, w);
    }
    W2[off + (long long)ij * n + r] = w;
  }
}

// Z2 -= W2 + hZ W2^T, per channel in 32x32 tiles
__global__ void k_sym_subtract(DevSpace S, const double* __restrict__ W2, double* __restrict__ Z, int hZ,
                               const int* __restrict__ tiles, int ntiles, const long long* __restrict__ zo)
{
  W2 = zsh(W2, zo, ZR_W2);
  Z = zsh(Z, zo, ZR_Z);
  __shared__ double tt[32][33];
  int t = blockIdx.x;
  if (t >= ntiles) return;
  int ch = tiles[3 * t], ti = tiles[3 * t + 1], tj = tiles[3 * t + 2];
  int n = S.ch_n[ch];
  long long off = S.ch_off[ch];
  int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  // load W2 tile (tj, ti) transposed: rows tj*32+.., cols ti*32+..
  for (int yy = ty; yy < 32; yy += 8) {
    int r = tj * 32 + tx, c = ti * 32 + yy;
    tt[yy][tx] = (r < n && c < n) ? W2[off + (long long)c * n + r] : 0.0;
  }
  __syncthreads();
  for (int yy = ty; yy < 32; yy += 8) {
    int r = ti * 32 + tx, c = tj * 32 + yy;
    if (r < n && c < n) {
      // W2^T(r, c) = W2(c, r) = tt[r - ti*32][c - tj*32] stored as tt[col=(r)][row=(c)]
      double wt = tt[tx][yy];
      Z[off + (long long)c * n + r] -= W2[off + (long long)c * n + r] + hZ * wt;
    }
  }
}

// ------------------------------------------------------------ Pandya forward
// DoPandyaTransformation_SingleChannel_XandY (src/Commutator.cc:1392-1485) plus the
// flipped Ybar of comm222_phss (src/Commutator.cc:1766-1788).  Outputs, per CC
// channel, three n_cc x 2nph column-major panels:
//   Xb(ik, t)  = Xbar(ik, t) * normfactor * (n_a - n_b)
//   Yt(ik, t)  = Ybar(t, ik) * normfactor
//   Yf(ik, t') = Ybar(t, ik) * normfactor * phi_bra phi_ik hY, t' = t with halves swapped
// One thread per (ik, t), from the space's descriptors (build_pandya_fwd,
// space.cpp): the J sum is one gather of X and of Y and two FMAs per term.
// DF: the J sums in double-float on the FP32 pipe (the split form, whose
// Z-bar product takes 42-bit digits of these panels); otherwise FP64.
template <bool DF>
__global__ void __launch_bounds__(256) k_pandya_fwd(DevWork W, const double* __restrict__ X,
                                                    const double* __restrict__ Y, int hY, double* __restrict__ Xb,
                                                    double* __restrict__ Yt, double* __restrict__ Yf,
                                                    const long long* __restrict__ zo)
{
  X = zsh(X, zo, ZR_X);
  Y = zsh(Y, zo, ZR_Y);
  Xb = zsh(Xb, zo, ZR_XB);
  Yt = zsh(Yt, zo, ZR_YT);
  Yf = zsh(Yf, zo, ZR_YFL);
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= W.n_pfout) return;
  const PfOut m = W.pf_out[o];
  const int nterm = (int)(m.code & 0xFFFFu), nsq = (int)((m.code >> 16) & 3u);
  // normfactor as the reference forms it: 1, sqrt 2 or sqrt 2 * sqrt 2
  const double ys = nsq == 0 ? 1.0 : nsq == 1 ? kSqrt2 : kSqrt2 * kSqrt2;
  const double yfs = (m.code >> 18) & 1u ? -1.0 : 1.0;
  double xbar = 0.0, ybar = 0.0;
  if (DF) {
    float sx = 0.f, cx = 0.f, sy = 0.f, cy = 0.f;
    for (int k = m.beg; k < m.beg + nterm; ++k) {
      const int e = __ldg(W.pf_e + k);
      const float2 w = __ldg(W.pf_wf + k);
      df_fma(w, d2ff(X[e]), sx, cx);
      df_fma(w, d2ff(Y[e]), sy, cy);
    }
    float hi = __fadd_rn(sx, cx);
    xbar = ff2d(hi, __fsub_rn(cx, __fsub_rn(hi, sx)));
    hi = __fadd_rn(sy, cy);
    ybar = ff2d(hi, __fsub_rn(cy, __fsub_rn(hi, sy)));
  } else {
    for (int k = m.beg; k < m.beg + nterm; ++k) {
      const int e = __ldg(W.pf_e + k);
      const double w = __ldg(W.pf_w + k);
      xbar = fma(w, X[e], xbar);
      ybar = fma(w, Y[e], ybar);
    }
  }
  // the FP64 pipe is this kernel's bound: factors of +-1 (every phase, the
  // usual normfactor and occupation difference) are sign flips, not
  // multiplies; the results are the same numbers
  const double xs = m.xs;
  Xb[m.dest] = (xs == 1.0 || xs == -1.0) ? dneg_if(xbar, xs < 0.0) : xbar * xs;
  const double yv = dneg_if(nsq == 0 ? ybar : ybar * ys, hY < 0);
  Yt[m.dest] = yv;
  Yf[m.dest + m.dyf] = dneg_if(yv, (yfs < 0.0) != (hY < 0));
}

// ------------------------------------------------------------ Pandya inverse
// AddInversePandyaTransformation (src/Commutator.cc:1501-1616): for every
// (ibra <= iket) element of every 2b channel block, the two J' sums over Zbar.
//
// Access pattern: a block owns a 32 (bras) x 32 (kets) tile; lanes run over
// kets, so for one bra (i,j) consecutive lanes share k and step through l.
// The first sum reads Zbar(il, kj): one column kj, consecutive rows il.  The
// second sum needs Zbar(ik, lj), which would be one row and scattered
// columns; it is read through the symmetry of the symmetrised Zbar instead,
//   head:  Zbar(r, c) = hZ Zbar(c, r),
//   tail:  Zbar(r, n + c) = phi_r phi_c Zbar(c, n + r),
// i.e. as Zbar(lj, ik): again one column, consecutive rows.  Results go
// through shared memory so both the Z(ibra, iket) and the mirrored
// Z(iket, ibra) updates are coalesced.
__global__ void __launch_bounds__(256) k_pandya_inv(DevSpace S, DevWork W, const double* __restrict__ Zb,
                                                    double* __restrict__ Z, int hZ, const int* __restrict__ tiles,
                                                    int ntiles)
{
  __shared__ double T[32][33];
  __shared__ int s_ccn[kMaxChannels];
  __shared__ long long s_zboff[kMaxChannels];
  int tix = blockIdx.x;
  if (tix >= ntiles) return;
  for (int c = threadIdx.x; c < S.nch; c += blockDim.x) {
    s_ccn[c] = S.cc_n[c];
    s_zboff[c] = W.zb_off[c];
  }
  __syncthreads();
  const int ch = tiles[3 * tix], tb = tiles[3 * tix + 1], tk = tiles[3 * tix + 2];
  const int n = S.ch_n[ch];
  const int J = ch / 6;
  const int kofs = S.ch_kofs[ch];
  const int N = S.norb;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int iket = tk * 32 + lane;
  int k = 0, l = 0, jjk = 0, jjl = 0;
  if (iket < n) {
    k = S.ket_p[kofs + iket];
    l = S.ket_q[kofs + iket];
    jjk = S.j2[k];
    jjl = S.j2[l];
  }
  for (int bb = warp; bb < 32; bb += 8) {
    const int ibra = tb * 32 + bb;
    double z = 0.0;
    const bool valid = ibra < n && iket < n && (hZ == 1 ? iket >= ibra : iket > ibra);
    if (valid) {
      const int i = S.ket_p[kofs + ibra], j = S.ket_q[kofs + ibra];
      const int jji = S.j2[i], jjj = S.j2[j];
      double commij = 0.0, commji = 0.0;
      {
        int par = (S.l[i] + S.l[l]) & 1;
        int tz = abs(S.tz2[i] - S.tz2[l]) / 2;
        int Jpmin = max(abs(jji - jjl), abs(jjk - jjj)) / 2;
        int Jpmax = min(jji + jjl, jjk + jjj) / 2;
        int kil = ket_index(N, min(i, l), max(i, l)), kkj = ket_index(N, min(j, k), max(j, k));
        // (2J'+1) 6j for consecutive J' sit in consecutive table slots
        const double* wrow = S.sixj_wval + sixj_slot(S.d1, S.sixj_base, jji, jjj, J, jjk, jjl, Jpmin) - Jpmin;
#pragma unroll 2
        for (int Jp = Jpmin; Jp <= Jpmax; ++Jp) {
          double w = __ldg(wrow + Jp);
          if (dzero(w)) continue;
          int cc = chan_index(Jp, par, tz);
          int ncc = s_ccn[cc];
          int il = __ldg(S.ccJ_loc + Jp * S.nkets + kil) + (i > l ? ncc : 0);
          int kj = __ldg(S.ccJ_loc + Jp * S.nkets + kkj) + (k > j ? ncc : 0);
          commij = fma(-w, Zb[s_zboff[cc] + (long long)kj * ncc + il], commij);
        }
      }
      if (k == l) {
        commji = commij;
      } else if (i == j) {
        commji = iphase((jji + jjj + jjk + jjl) / 2) * commij;
      } else {
        int par = (S.l[i] + S.l[k]) & 1;
        int tz = abs(S.tz2[i] - S.tz2[k]) / 2;
        int Jpmin = max(abs(jjj - jjl), abs(jjk - jji)) / 2;
        int Jpmax = min(jjj + jjl, jjk + jji) / 2;
        int kik = ket_index(N, min(i, k), max(i, k)), klj = ket_index(N, min(l, j), max(l, j));
        // i <= k always (ibra <= iket), so ik is a row of the head/tail blocks
        const int tsign = (l > j) ? iphase((jji + jjk + jjl + jjj) / 2) : hZ;
        double acc = 0.0;
        const double* wrow = S.sixj_wval + sixj_slot(S.d1, S.sixj_base, jjj, jji, J, jjk, jjl, Jpmin) - Jpmin;
#pragma unroll 2
        for (int Jp = Jpmin; Jp <= Jpmax; ++Jp) {
          double w = __ldg(wrow + Jp);
          if (dzero(w)) continue;
          int cc = chan_index(Jp, par, tz);
          int ncc = s_ccn[cc];
          int ik = __ldg(S.ccJ_loc + Jp * S.nkets + kik);
          int lj = __ldg(S.ccJ_loc + Jp * S.nkets + klj);
          // Zbar(ik, lj[+n]) read as its symmetric partner Zbar(lj, ik[+n])
          long long e = s_zboff[cc] + (long long)(ik + (l > j ? ncc : 0)) * ncc + lj;
          acc = fma(-w, Zb[e], acc);
        }
        commji = dneg_if(acc, tsign < 0);
      }
      // z = -(commij - (-1)^(jk+jl-J) commji) / norm
      int bd = (i == j), kd = (k == l);
      double inv_norm = bd == kd ? (bd ? 0.5 : 1.0) : 0.70710678118654752440;
      double d = commij - dneg_if(commji, iphase((jjk + jjl) / 2 - J) < 0);
      z = dneg_if(d, true);
      if (bd || kd) z *= inv_norm;
    }
    T[bb][lane] = z;
  }
  __syncthreads();
  const long long off = S.ch_off[ch];
  // Z(ibra, iket) += z : threads run over bras (column-major rows)
  for (int e = threadIdx.x; e < 1024; e += 256) {
    int bb = e & 31, kk = e >> 5;
    int ibra = tb * 32 + bb, ik2 = tk * 32 + kk;
    if (ibra < n && ik2 < n && (hZ == 1 ? ik2 >= ibra : ik2 > ibra)) Z[off + (long long)ik2 * n + ibra] += T[bb][kk];
  }
  // Z(iket, ibra) += hZ z for ibra != iket : threads run over kets
  for (int e = threadIdx.x; e < 1024; e += 256) {
    int kk = e & 31, bb = e >> 5;
    int ibra = tb * 32 + bb, ik2 = tk * 32 + kk;
    if (ibra < n && ik2 < n && ik2 > ibra) Z[off + (long long)ibra * n + ik2] += hZ * T[bb][kk];
  }
}

// ------------------------------------------- Pandya inverse, by orbit quadruple
// Split form of AddInversePandyaTransformation (src/Commutator.cc:1501-1616),
// reorganised around orbit quadruples: the element Z_J(ij, kl) of every J is
// a small recoupling of the same Zbar_J'(il, kj) and Zbar_J'(ik, lj) values,
// so a block loads those values once for all J instead of once per J.
//
// A block owns one (i, k, class of j) group of quadruples (see
// build_invq_tasks), laid out as a jn x ln rectangle of (j, l) pairs:
//   1. per-pair counts and a block scan give each pair its slots in shared
//      memory: n1 + n2 staged Zbar values and nJ result slots, in order of
//      (2j_j, 2j_l) so neighbouring slots share loop lengths;
//   2. staging, a thread per value slot (four loads in flight): Zbar values
//      -> (hi, lo) float pairs;
//   3. a thread per result slot (pair, J): the two J' sums in double-float on
//      the FP32 pipe, then Z(ij, kl) += z and Z(kl, ij) += hZ z.  The rows
//      (i, j) and columns (k, l) of the block in channel J are runs of
//      consecutive kets, so a ket's index is its run's first plus its rank.
// FP64 appears only in the final Z += z.  Values are carried with 48-bit
// significands (double-float), far inside the split form's 1e-10 tolerance;
// magnitudes below the FP32 normal range (1.2e-38) are flushed to zero.

constexpr int kInvqThreads = 256;

// the r-th set position of the first n predicate values (n <= 64) of a warp,
// written to out[]: a ballot compaction; returns the count
// (and, with rank, each value's position: rank[x] = r)
__device__ __forceinline__ int warp_compact64(bool v0, bool v1, unsigned char x0, unsigned char x1, unsigned char* out,
                                              unsigned char* rank = nullptr)
{
  const int lane = threadIdx.x & 31;
  const unsigned m0 = __ballot_sync(0xffffffffu, v0), m1 = __ballot_sync(0xffffffffu, v1);
  const unsigned below = (1u << lane) - 1;
  const int r0 = __popc(m0 & below), r1 = __popc(m0) + __popc(m1 & below);
  if (v0) {
    out[r0] = x0;
    if (rank) rank[x0] = (unsigned char)r0;
  }
  if (v1) {
    out[r1] = x1;
    if (rank) rank[x1] = (unsigned char)r1;
  }
  return __popc(m0) + __popc(m1);
}

// floor(r / n) for 0 <= r <= 4096, 1 <= n <= 64, with rcp = 1.0f / n: the exact
// quotient's fractional part stays >= 1/128 from an integer, far above the
// product's rounding error (2^-11)
__device__ __forceinline__ int small_div(int r, float rcp) { return __float2int_rz(__fmul_rn((float)r + 0.5f, rcp)); }

// (four blocks per SM: the shared-memory budget admits four, and the register
// bound that fits them measured 3% faster than the compiler's own choice;
// smaller or larger budgets measured slower)
__global__ void __launch_bounds__(kInvqThreads, 4) k_pandya_inv_ff(DevSpace S, DevWork W, const double* __restrict__ Zb,
                                                             double* __restrict__ Z, int hZ,
                                                             const int4* __restrict__ tasks,
                                                             const int* __restrict__ clist,
                                                             const int* __restrict__ coff,
                                                             const unsigned char* __restrict__ csort,
                                                             const long long* __restrict__ zo)
{
  Zb = zsh(Zb, zo, ZR_ZB);
  Z = zsh(Z, zo, ZR_Z);
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int s_j[kInvqMaxOrb], s_l[kInvqMaxOrb], s_jj[kInvqMaxOrb], s_jl[kInvqMaxOrb];
  __shared__ int s_kkj[kInvqMaxOrb];       // global index of the ket (k, j) / (j, k)
  __shared__ unsigned char s_jperm[kInvqMaxOrb], s_lperm[kInvqMaxOrb];
  __shared__ unsigned char s_jv[kInvqMaxJ][kInvqMaxOrb], s_lv[kInvqMaxJ][kInvqMaxOrb];  // per J: valid j, l
  __shared__ unsigned char s_jrk[kInvqMaxJ][kInvqMaxOrb], s_lrk[kInvqMaxJ][kInvqMaxOrb];  // per J: their ranks
  __shared__ int s_wbk[kInvqMaxJ][3];      // per J: first bra, first ket, channel size
  __shared__ long long s_woff[kInvqMaxJ];  // per J: arena offset of the channel
  __shared__ int s_cn[2][kInvqMaxJ];       // per J': CC channel size, sums 1 and 2
  __shared__ long long s_coff[2][kInvqMaxJ];
  __shared__ int s_cik[kInvqMaxJ];         // per J': local index of the CC ket (i, k)
  __shared__ unsigned long long s_wsum[kInvqThreads / 32];
  __shared__ int s_red[6];                 // unions over the block: J' of sum 1, J' of sum 2, J

  const int4 tk = tasks[blockIdx.x];
  const int i = tk.x & 0xFFFF, k = tk.x >> 16;
  const int cj = tk.y & 0xFF, cl = (tk.y >> 8) & 0xFF;
  const int jf = tk.z & 0xFFFF, jn = tk.z >> 16, lf = tk.w & 0xFFFF, ln = tk.w >> 16;
  const int P = jn * ln;
  const float rln = 1.0f / ln;  // pair p = jx ln + lx: jx = small_div(p, rln)
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int N = S.norb, nk = S.nkets;
  if (tid < jn) {
    int o = clist[coff[cj] + jf + tid];
    s_j[tid] = o;
    s_jj[tid] = S.j2[o];
    s_kkj[tid] = ket_index(N, min(k, o), max(k, o));
  }
  if (tid >= 64 && tid - 64 < ln) {
    int o = clist[coff[cl] + lf + tid - 64];
    s_l[tid - 64] = o;
    s_jl[tid - 64] = S.j2[o];
  }
  if (tid < 6) s_red[tid] = (tid & 1) ? -1 : (1 << 20);
  if (warp == 4 || warp == 5) {
    // slot order: the block's j (warp 4) and l (warp 5) by (2j, orbit), from
    // the class's sorted positions, so neighbouring slots have equal loop lengths
    const int c = warp == 4 ? cj : cl, f = warp == 4 ? jf : lf, n = warp == 4 ? jn : ln;
    const int nc = coff[c + 1] - coff[c];
    const int x0 = lane < nc ? csort[coff[c] + lane] - f : -1;
    const int x1 = lane + 32 < nc ? csort[coff[c] + lane + 32] - f : -1;
    warp_compact64(x0 >= 0 && x0 < n, x1 >= 0 && x1 < n, (unsigned char)x0, (unsigned char)x1,
                   warp == 4 ? s_jperm : s_lperm);
  }
  __syncthreads();
  const int ji = S.j2[i], jk = S.j2[k];

  // 1. per pair p = jx ln + lx: counts n1 | n2 << 5 | nJ << 10, slot offsets of
  //    its staged values (off1, off2) and results (offO), assigned in slot order
  unsigned short* cnt = (unsigned short*)smem;
  unsigned short* off1 = cnt + P;
  unsigned short* off2 = off1 + P;
  unsigned short* offO = off2 + P;
  float2* zs = (float2*)(smem + ((8 * P + 15) & ~15));
  unsigned long long carry = 0;
  for (int base = 0; base < P; base += kInvqThreads) {
    const int sidx = base + tid;
    unsigned long long v = 0;
    int p = 0;
    int r0 = 1 << 20, r1 = -1, r2 = 1 << 20, r3 = -1, r4 = 1 << 20, r5 = -1;
    if (sidx < P) {
      const int jsx = small_div(sidx, rln);
      const int jx = s_jperm[jsx], lx = s_lperm[sidx - jsx * ln];
      p = jx * ln + lx;
      int n1, n2, nJ, Jlo, lo1, lo2;
      if (invq_counts(i, s_j[jx], k, s_l[lx], ji, s_jj[jx], jk, s_jl[lx], hZ, n1, n2, nJ, Jlo, lo1, lo2)) {
        v = (unsigned long long)n1 | ((unsigned long long)n2 << 21) | ((unsigned long long)nJ << 42);
        if (n1) {
          r0 = lo1;
          r1 = lo1 + n1 - 1;
        }
        if (n2) {
          r2 = lo2;
          r3 = lo2 + n2 - 1;
        }
        const bool ev = (i == s_j[jx]) || (k == s_l[lx]);
        r4 = Jlo;
        r5 = Jlo + (ev ? 2 : 1) * (nJ - 1);
      }
      cnt[p] = (unsigned short)((v & 31) | (((v >> 21) & 31) << 5) | (((v >> 42) & 31) << 10));
    }
    r0 = __reduce_min_sync(0xffffffffu, r0);
    r1 = __reduce_max_sync(0xffffffffu, r1);
    r2 = __reduce_min_sync(0xffffffffu, r2);
    r3 = __reduce_max_sync(0xffffffffu, r3);
    r4 = __reduce_min_sync(0xffffffffu, r4);
    r5 = __reduce_max_sync(0xffffffffu, r5);
    if (lane == 0) {
      atomicMin(&s_red[0], r0);
      atomicMax(&s_red[1], r1);
      atomicMin(&s_red[2], r2);
      atomicMax(&s_red[3], r3);
      atomicMin(&s_red[4], r4);
      atomicMax(&s_red[5], r5);
    }
    unsigned long long x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      unsigned long long t = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += t;
    }
    if (lane == 31) s_wsum[warp] = x;
    __syncthreads();
    unsigned long long wpre = 0, tot = 0;
#pragma unroll
    for (int w = 0; w < kInvqThreads / 32; ++w) {
      unsigned long long t = s_wsum[w];
      if (w < warp) wpre += t;
      tot += t;
    }
    if (sidx < P) {
      unsigned long long e = carry + wpre + x - v;
      off1[p] = (unsigned short)(e & 0x1FFFFF);
      off2[p] = (unsigned short)((e >> 21) & 0x1FFFFF);
      offO[p] = (unsigned short)(e >> 42);
    }
    carry += tot;
    __syncthreads();
  }
  const int tot1 = (int)(carry & 0x1FFFFF), tot2 = (int)((carry >> 21) & 0x1FFFFF), totO = (int)(carry >> 42);
  const int tot12 = tot1 + tot2;
  // regions: sum-1 values [0, tot1), sum-2 values [tot1, tot12), then the
  // owner of each value slot and of each result slot (tot12 + e);
  // owner[slot] = its pair
  unsigned short* owner = (unsigned short*)(zs + tot12);
  for (int p = tid; p < P; p += kInvqThreads) {
    const int c = cnt[p];
    off2[p] = (unsigned short)(off2[p] + tot1);
    const int n1 = c & 31, n2 = (c >> 5) & 31, nJ = c >> 10;
    for (int x = 0; x < n1; ++x) owner[off1[p] + x] = (unsigned short)p;
    for (int x = 0; x < n2; ++x) owner[off2[p] + x] = (unsigned short)p;
    for (int x = 0; x < nJ; ++x) owner[tot12 + offO[p] + x] = (unsigned short)p;
  }

  // per-J' CC channels of both sums (a thread each) and per-J output
  // rectangles (a warp each); empty unions (no sum-2 pairs, or no pair at all
  // when Z is anti-hermitian and the block's only pair is diagonal) count 0
  const int u1 = s_red[0], u2 = s_red[2], uJ = s_red[4];
  const int n1u = max(0, s_red[1] - u1 + 1), n2u = max(0, s_red[3] - u2 + 1), nJu = max(0, s_red[5] - uJ + 1);
  const int pl = cl & 1, tzl = (cl & 2) ? 1 : -1;
  const int pj = cj & 1, tzj = (cj & 2) ? 1 : -1;
  if (tid < n1u) {
    const int cc = chan_index(u1 + tid, (S.l[i] + pl) & 1, abs(S.tz2[i] - tzl) / 2);
    s_cn[0][tid] = S.cc_n[cc];
    s_coff[0][tid] = W.zb_off[cc];
  } else if (tid >= 32 && tid - 32 < n2u) {
    const int t = tid - 32, Jp = u2 + t;
    const int cc = chan_index(Jp, (S.l[i] + S.l[k]) & 1, abs(S.tz2[i] - S.tz2[k]) / 2);
    s_cn[1][t] = S.cc_n[cc];
    s_coff[1][t] = W.zb_off[cc];
    s_cik[t] = S.ccJ_loc[(size_t)Jp * nk + ket_index(N, i, k)];
  }
  for (int t = warp; t < nJu; t += kInvqThreads / 32) {
    // rows (i, j) and columns (k, l) of channel J: consecutive kets
    const int J = uJ + t;
    bool v0 = false, v1 = false;
    if (lane < jn) {
      const int jj = s_jj[lane];
      v0 = abs(ji - jj) <= 2 * J && ji + jj >= 2 * J && !(s_j[lane] == i && (J & 1));
    }
    if (lane + 32 < jn) {
      const int jj = s_jj[lane + 32];
      v1 = abs(ji - jj) <= 2 * J && ji + jj >= 2 * J && !(s_j[lane + 32] == i && (J & 1));
    }
    const int nr = warp_compact64(v0, v1, (unsigned char)lane, (unsigned char)(lane + 32), s_jv[t], s_jrk[t]);
    v0 = v1 = false;
    if (lane < ln) {
      const int jl = s_jl[lane];
      v0 = abs(jk - jl) <= 2 * J && jk + jl >= 2 * J && !(s_l[lane] == k && (J & 1));
    }
    if (lane + 32 < ln) {
      const int jl = s_jl[lane + 32];
      v1 = abs(jk - jl) <= 2 * J && jk + jl >= 2 * J && !(s_l[lane + 32] == k && (J & 1));
    }
    const int nc = warp_compact64(v0, v1, (unsigned char)lane, (unsigned char)(lane + 32), s_lv[t], s_lrk[t]);
    __syncwarp();
    if (lane == 0) {
      if (nr && nc) {
        const int ch = chan_index(J, (S.l[i] + pj) & 1, (S.tz2[i] + tzj) / 2);
        s_wbk[t][0] = S.ketJ_loc[(size_t)J * nk + ket_index(N, i, s_j[s_jv[t][0]])];
        s_wbk[t][1] = S.ketJ_loc[(size_t)J * nk + ket_index(N, k, s_l[s_lv[t][0]])];
        s_wbk[t][2] = S.ch_n[ch];
        s_woff[t] = S.ch_off[ch];
      }
    }
  }
  __syncthreads();

  // 2. staging, a thread per slot: Zbar values as (hi, lo) pairs, batches of
  //    four slots with their loads in flight together
  //    sum 1: Zbar_J'(il, kj); sum 2: Zbar_J'(ik, lj), read as its symmetric
  //    partner Zbar_J'(lj, ik[+n]) (head: hZ, tail: phi phi; the sign is
  //    applied with the sum)
  {
    const int kk = ket_index(N, i, 0);  // ket (i, l) = kk + l
    for (int e0 = tid; e0 < tot12; e0 += 4 * kInvqThreads) {
      double v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int e = e0 + u * kInvqThreads;
        v[u] = 0.0;
        if (e >= tot12) continue;
        const int p = owner[e];
        const int jx = small_div(p, rln), lx = p - jx * ln;
        const int j = s_j[jx], l = s_l[lx], jj = s_jj[jx], jl = s_jl[lx];
        if (e < tot1) {
          const int Jp = (max(abs(ji - jl), abs(jk - jj)) >> 1) + e - off1[p], t = Jp - u1;
          const int ncc = s_cn[0][t];
          const int* cmap = S.ccJ_loc + (size_t)Jp * nk;
          const int il = __ldg(cmap + kk + l);
          const int kj = __ldg(cmap + s_kkj[jx]) + (k > j ? ncc : 0);
          v[u] = __ldg(Zb + s_coff[0][t] + (long long)kj * ncc + il);
        } else {
          const int Jp = (max(abs(jj - jl), abs(jk - ji)) >> 1) + e - off2[p], t = Jp - u2;
          const int ncc = s_cn[1][t];
          const int lj = __ldg(S.ccJ_loc + (size_t)Jp * nk + ket_index(N, min(l, j), max(l, j)));
          v[u] = __ldg(Zb + s_coff[1][t] + (long long)(s_cik[t] + (l > j ? ncc : 0)) * ncc + lj);
        }
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int e = e0 + u * kInvqThreads;
        if (e < tot12) zs[e] = d2ff(v[u]);
      }
    }
  }
  __syncthreads();

  // 3. the J' sums, a thread per result slot (pair, J)
  {
    const int d1 = S.d1;
    const int a6 = (ji - 1) >> 1, c6 = (jk - 1) >> 1;
    for (int e = tid; e < totO; e += kInvqThreads) {
      const int p = owner[tot12 + e];
      const int t = e - offO[p];
      const int jx = small_div(p, rln), lx = p - jx * ln;
      const int j = s_j[jx], l = s_l[lx], jj = s_jj[jx], jl = s_jl[lx];
      const int c = cnt[p];
      const int n1 = c & 31, n2 = (c >> 5) & 31;
      const bool ev = (i == j) || (k == l);
      int Jlo = max(abs(ji - jj), abs(jk - jl)) >> 1;
      if (ev) Jlo += Jlo & 1;
      const int J = Jlo + (ev ? 2 * t : t);
      const int J3min = abs(ji - jj) >> 1;
      const int b6 = (jj - 1) >> 1, e6 = (jl - 1) >> 1;
      const float2* wr = S.sixj_wf + __ldg(S.sixj_base + ((a6 * d1 + b6) * d1 + c6) * d1 + e6) + (J - J3min) * n1;
      const float2* z1 = zs + off1[p];
      // two accumulators halve the dependency chain
      float s1 = 0.f, c1 = 0.f, s1b = 0.f, c1b = 0.f;
      int x = 0;
      for (; x + 1 < n1; x += 2) {
        df_fma(__ldg(wr + x), z1[x], s1, c1);
        df_fma(__ldg(wr + x + 1), z1[x + 1], s1b, c1b);
      }
      if (x < n1) df_fma(__ldg(wr + x), z1[x], s1, c1);
      float hi, lo;
      df_add(s1, c1, s1b, c1b, s1, c1);
      const int phJ = iphase((jk + jl) / 2 - J);
      if (ev) {
        // z = (1 - phJ [ph4]) A1: 0 or 2 A1
        const int f = (k == l) ? phJ : phJ * iphase((ji + jj + jk + jl) / 2);
        hi = f > 0 ? 0.f : __fmul_rn(s1, 2.f);
        lo = f > 0 ? 0.f : __fmul_rn(c1, 2.f);
      } else {
        const float2* wq = S.sixj_wf + __ldg(S.sixj_base + ((b6 * d1 + a6) * d1 + c6) * d1 + e6) + (J - J3min) * n2;
        const float2* z2 = zs + off2[p];
        float s2 = 0.f, c2 = 0.f, s2b = 0.f, c2b = 0.f;
        x = 0;
        for (; x + 1 < n2; x += 2) {
          df_fma(__ldg(wq + x), z2[x], s2, c2);
          df_fma(__ldg(wq + x + 1), z2[x + 1], s2b, c2b);
        }
        if (x < n2) df_fma(__ldg(wq + x), z2[x], s2, c2);
        df_add(s2, c2, s2b, c2b, s2, c2);
        // z = A1 - phJ tsign A2
        const int tsign = (l > j) ? iphase((ji + jj + jk + jl) / 2) : hZ;
        if (phJ * tsign > 0) {
          s2 = -s2;
          c2 = -c2;
        }
        df_add(s1, c1, s2, c2, hi, lo);
      }
      double z = ff2d(hi, lo);
      if (i == j && k == l) z *= 0.5;
      else if (ev) z *= 0.70710678118654752440;
      // Z(ij, kl) += z and Z(kl, ij) += hZ z: bra (i, j) and ket (k, l) are
      // consecutive kets of channel J, found by their ranks among the block's
      // rows and columns of that channel
      const int tJ = J - uJ;
      const int ib = s_wbk[tJ][0] + s_jrk[tJ][jx], ik = s_wbk[tJ][1] + s_lrk[tJ][lx], n = s_wbk[tJ][2];
      double* Zc = Z + s_woff[tJ];
      Zc[(long long)ik * n + ib] += z;
      if (ib != ik) Zc[(long long)ib * n + ik] += dneg_if(z, hZ < 0);
    }
  }
}

// -------------------------------------------------- single-operator Pandya
// Commutator::DoPandyaTransformation (src/Commutator.cc:1319-1390, 1487-1497):
// for cross-coupled channel ch (blockIdx.y), bras are its hh then ph kets (a,b)
// in both orders (rows ib and ib + nph), kets (c,d) all its kets, and
//   Xbar = - sum_J (2J+1) {ja jb Jcc; jc jd J} Z^J_{ad,cb}   (|6j| < 1e-8 skipped)
// normal: 2nph x ncc column-major, Xbar; transpose: ncc x 2nph, herm (na-nb) Xbar.
// One thread per element, in output order, so the writes coalesce.
__global__ void k_pandya_single(DevSpace S, DevWork W, const double* __restrict__ Z, int herm, int transpose,
                                double* __restrict__ out)
{
  int ch = blockIdx.y;
  int ncc = S.cc_n[ch], nph = W.cc_nph[ch];
  long long tot = 2LL * nph * ncc;
  long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= tot) return;
  int row, ik;
  if (transpose) {
    row = (int)(e / ncc);
    ik = (int)(e - (long long)row * ncc);
  } else {
    ik = (int)(e / (2 * nph));
    row = (int)(e - (long long)ik * 2 * nph);
  }
  const int second = row >= nph;
  const int kb = W.cc_ph[W.cc_ph_off[ch] + row - second * nph];
  const int kofs = S.cc_kofs[ch];
  const int p = S.cc_p[kofs + kb], q = S.cc_q[kofs + kb];
  const int a = second ? q : p, b = second ? p : q;
  const int c = S.cc_p[kofs + ik], d = S.cc_q[kofs + ik];
  const int ja = S.j2[a], jb = S.j2[b], jc = S.j2[c], jd = S.j2[d];
  const int Jcc = ch / 6;
  int t1 = abs(ja - jd), t2 = abs(jc - jb);
  const int jmin = (t1 > t2 ? t1 : t2) >> 1;
  const int jmax = ((ja + jd) < (jc + jb) ? ja + jd : jc + jb) >> 1;
  double nrm = 1.0;
  if (a == d) nrm *= kSqrt2;
  if (c == b) nrm *= kSqrt2;
  double xbar = 0.0;
  for (int J = jmin; J <= jmax; ++J) {
    double w = dev_sixj_w(S, ja, jb, Jcc, jc, jd, J);
    if (w == 0.0) continue;
    xbar -= w * (nrm * dev_tbme_J_norm(S, Z, J, a, d, c, b));
  }
  double* o = out + W.xb_off[ch];
  if (transpose)
    o[e] = herm * xbar * (S.occ[a] - S.occ[b]);
  else
    o[e] = xbar;
}

// ------------------------------------------------------------------ generator
// Generator::Update -> ConstructGenerator_SingleRef (src/Generator.cc:32-76,
// 236-297) for a single-reference space, whose core is the set of occupied
// orbits: Eta is zero except <i|Eta|a> (i outside, a inside the core) and
// <ij|Eta|kl> (i, j outside, k, l inside), each the generator function of the
// matching element of H and its energy denominator, antisymmetrised.
constexpr double kGenOccCut = 1e-6;  // ModelSpace::OCC_CUT (src/ModelSpace.cc:14)

// the generator functions of src/Generator.cc:12-15
// the reference's q-transfer generators (src/Generator.cc:18, :63-69):
// atan(2 Hod / d) / 2 times (|d| M_N / (hbar c)^2)^(n/2), with the reference's
// constants (src/PhysicalConstants.hh: hbar c = 197.3269718 MeV fm, M_N the
// mean of 938.2720813 and 939.5654133 MeV)
constexpr double kHbarc = 197.3269718;
constexpr double kMNucleon = (938.2720813 + 939.5654133) / 2.0;

__device__ __forceinline__ double eta_value(int type, double hod, double den)
{
  if (type > GEN_QTRANSFER_BASE)
    return pow(fabs(den) * kMNucleon / kHbarc / kHbarc, 0.5 * (type - GEN_QTRANSFER_BASE)) *
           (0.5 * atan(2 * hod / den));
  switch (type) {
    case GEN_ATAN: return 0.5 * atan(2 * hod / den);
    case GEN_WEGNER: return hod * den;
    case GEN_IMAGINARY_TIME: return hod * (double)((den > 0) - (den < 0));
    default: return hod / den;
  }
}

// M[a * N + b] = GetTBMEmonopole(a, b, a, b): the monopoles the Epstein-Nesbet
// denominators add (src/Generator.cc:116-119, 172-180)
__global__ void k_gen_monopoles(DevSpace S, const double* __restrict__ H, double* __restrict__ M)
{
  int N = S.norb;
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= N * N) return;
  int a = idx / N, b = idx - a * N;
  M[idx] = dev_monopole(S, H, a, b, a, b);
}

// one-body part; Generator::Get1bDenominator, src/Generator.cc:110-139
__global__ void k_gen_onebody(DevSpace S, const double* __restrict__ H, const double* __restrict__ M,
                              double* __restrict__ Eta, GenParams p)
{
  int N = S.norb;
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= N * N) return;
  int a = idx / N, i = idx - a * N;  // column a (core), row i (outside the core)
  double na = S.occ[a], ni = S.occ[i];
  if (na < kGenOccCut || ni >= kGenOccCut) return;
  const double* H1 = H + 32;
  double d = H1[(long long)i * N + i] - H1[(long long)a * N + a];
  if (p.partitioning == DENOM_EPSTEIN_NESBET) d += (ni - na) * M[(long long)i * N + a];
  if (p.delta_index == kDeltaAll || i == p.delta_index || a == p.delta_index) d += p.delta;
  if (fabs(d) < p.cutoff) d = p.cutoff;
  double e = eta_value(p.type, H1[(long long)a * N + i], d);
  Eta[32 + (long long)a * N + i] = e;
  Eta[32 + (long long)i * N + a] = -e;
}

// two-body part, one block per channel: columns are the channel's hh kets,
// threads run over the bra kets; Generator::Get2bDenominator,
// src/Generator.cc:142-188
__global__ void k_gen_twobody(DevSpace S, DevWork W, const double* __restrict__ H, const double* __restrict__ M,
                              double* __restrict__ Eta, GenParams p)
{
  int ch = blockIdx.x;
  int n = S.ch_n[ch];
  int h0 = W.hh_off[ch], h1 = W.hh_off[ch + 1];
  if (n == 0 || h0 == h1) return;
  int N = S.norb;
  long long off = S.ch_off[ch];
  int kofs = S.ch_kofs[ch];
  const double* H1 = H + 32;
  const bool en = p.partitioning == DENOM_EPSTEIN_NESBET;
  for (int h = h0; h < h1; ++h) {
    int ik = W.hh_list[h];
    int k = S.ket_p[kofs + ik], l = S.ket_q[kofs + ik];
    double nk = S.occ[k], nl = S.occ[l];
    double fk = H1[(long long)k * N + k], fl = H1[(long long)l * N + l];
    for (int ib = threadIdx.x; ib < n; ib += blockDim.x) {
      int i = S.ket_p[kofs + ib], j = S.ket_q[kofs + ib];
      double ni = S.occ[i], nj = S.occ[j];
      if (ni >= kGenOccCut || nj >= kGenOccCut) continue;
      double d = H1[(long long)i * N + i] + H1[(long long)j * N + j] - fk - fl;
      if (p.delta_index == kDeltaAll) d += p.delta;
      if (en) {
        d += (1 - ni - nj) * M[(long long)i * N + j];
        d -= (1 - nk - nl) * M[(long long)k * N + l];
        d += (ni - nk) * M[(long long)i * N + k];
        d += (ni - nl) * M[(long long)i * N + l];
        d += (nj - nk) * M[(long long)j * N + k];
        d += (nj - nl) * M[(long long)j * N + l];
      }
      if (fabs(d) < p.cutoff) d = p.cutoff;
      double e = eta_value(p.type, H[off + (long long)ik * n + ib], d);
      Eta[off + (long long)ik * n + ib] = e;
      Eta[off + (long long)ib * n + ik] = -e;
    }
  }
}

// ------------------------------------------------------------ operator algebra
__global__ void k_axpy(double* __restrict__ y, const double* __restrict__ x, double a, long long n)
{
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  long long stride = (long long)gridDim.x * blockDim.x;
  for (; i < n; i += stride) y[i] = fma(a, x[i], y[i]);
}

__global__ void k_scale(double* __restrict__ y, double a, long long n)
{
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  long long stride = (long long)gridDim.x * blockDim.x;
  for (; i < n; i += stride) y[i] *= a;
}

// Operator::Norm pieces: chunk c of the norm list sums weight * v^2 over its
// range; partial[c] is written (no atomics, deterministic).
__global__ void k_norm_chunks(const double* __restrict__ A, const long long* __restrict__ chunk_off,
                              const int* __restrict__ chunk_len, const double* __restrict__ chunk_w,
                              double* __restrict__ partial, int nchunks)
{
  __shared__ double red[32];
  int c = blockIdx.x;
  if (c >= nchunks) return;
  const double* p = A + chunk_off[c];
  int len = chunk_len[c];
  double s = 0.0;
  for (int t = threadIdx.x; t < len; t += blockDim.x) s = fma(p[t], p[t], s);
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    v = warp_sum(v);
    if (threadIdx.x == 0) partial[c] = v * chunk_w[c];
  }
}

// y += a x together with the pieces of x's norm (the BCH loop adds each
// nested commutator and tests its norm): block c < nchunks does norm chunk c
// of the two-body blocks, block nchunks the zero- and one-body parts.  x is a
// commutator result, whose padding between blocks is zero, so those words of
// y are left as they are.
__global__ void k_axpy_norm(DevSpace S, double* __restrict__ y, const double* __restrict__ x, double a,
                            const long long* __restrict__ chunk_off, const int* __restrict__ chunk_len,
                            const double* __restrict__ chunk_w, double* __restrict__ partial, int nchunks)
{
  __shared__ double red[32];
  const int c = blockIdx.x;
  double s = 0.0;
  if (c < nchunks) {
    const long long off = chunk_off[c];
    const int len = chunk_len[c];
    int t = threadIdx.x;
    // four elements' loads in flight per thread
    for (; t + 3 * (int)blockDim.x < len; t += 4 * blockDim.x) {
      double v[4], w[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        v[u] = x[off + t + u * blockDim.x];
        w[u] = y[off + t + u * blockDim.x];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        y[off + t + u * blockDim.x] = fma(a, v[u], w[u]);
        s = fma(v[u], v[u], s);
      }
    }
    for (; t < len; t += blockDim.x) {
      const double v = x[off + t];
      y[off + t] = fma(a, v, y[off + t]);
      s = fma(v, v, s);
    }
  } else {
    const int N = S.norb;
    if (threadIdx.x == 0) y[0] = fma(a, x[0], y[0]);
    for (int t = threadIdx.x; t < N * N; t += blockDim.x) {
      const int p = t % N, q = t / N;
      const double v = x[32 + t];
      y[32 + t] = fma(a, v, y[32 + t]);
      if (S.l[p] == S.l[q] && S.j2[p] == S.j2[q] && S.tz2[p] == S.tz2[q]) s += v * v * (S.j2[p] + 1);
    }
  }
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    v = warp_sum(v);
    if (threadIdx.x == 0) partial[c] = c < nchunks ? v * chunk_w[c] : v;
  }
}

// one-body norm: sum over p, q in one channel of (2 j_p + 1) O_pq^2
__global__ void k_norm_onebody(DevSpace S, const double* __restrict__ A, double* __restrict__ out)
{
  __shared__ double red[32];
  int N = S.norb;
  double s = 0.0;
  for (int t = threadIdx.x; t < N * N; t += blockDim.x) {
    int p = t % N, q = t / N;
    if (S.l[p] == S.l[q] && S.j2[p] == S.j2[q] && S.tz2[p] == S.tz2[q]) {
      double v = A[32 + t];
      s += v * v * (S.j2[p] + 1);
    }
  }
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    v = warp_sum(v);
    if (threadIdx.x == 0) *out = v;
  }
}

// ------------------------------------------------------------------ launchers
cudaError_t launch_comm111_110(const Space& s, const double* X, const double* Y, double* Z, bool do111, bool do110,
                               cudaStream_t st, const long long* zo, int nz)
{
  int threads = s.norb <= 128 ? 128 : 256;
  k_comm111_110<<<dim3(s.norb, 1, nz), threads, 0, st>>>(s.dev, X, Y, Z, do111, do110, zo);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_comm220(const Space& s, const double* X, const double* Y, double* Z, int hX, cudaStream_t st,
                           const long long* zo, int nz)
{
  if (s.work.n220 == 0) return cudaSuccess;
  int wpb = 8;
  k_comm220<<<dim3((s.work.n220 + wpb - 1) / wpb, 1, nz), 32 * wpb, 0, st>>>(s.dev, s.work, X, Y, Z, hX, zo);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_comm121(const Space& s, const int* dev_holes, const double* X, const double* Y, double* Z,
                           int hZ, cudaStream_t st, const long long* zo, int nz)
{
  if (s.work.npairs1b == 0) return cudaSuccess;
  int wpb = 4;
  k_comm121<<<dim3((s.work.npairs1b + wpb - 1) / wpb, 1, nz), 32 * wpb, 0, st>>>(
      s.dev, s.work, dev_holes, (int)s.holes.size(), X, Y, Z, hZ, zo);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_comm221_1b(const Space& s, const double* X, const double* Y, double* Z, int hX, int hZ,
                              const double* Mz, cudaStream_t st, const long long* zo, int nz)
{
  if (s.work.n221 == 0) return cudaSuccess;
  int wpb = 8;
  if (Mz) {
    // no other kernel writes Z1 concurrently: plain stores per (i, j) pair
    k_comm221_1b_mz<<<dim3(s.work.npairs1b, 1, nz), 128, 0, st>>>(s.dev, s.work, X, Y, Z, hX, hZ, Mz, zo);
    count_launch();
    return cudaGetLastError();
  }
  k_comm221_1b<<<(s.work.n221 + wpb - 1) / wpb, 32 * wpb, 0, st>>>(s.dev, s.work, X, Y, Z, hX, hZ, Mz);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_comm122(const Space& s, const double* X, const double* Y, double* Z, double* W2, int hZ,
                           const int* sym_tiles, int nsym_tiles, cudaStream_t st, const long long* zo, int nz, bool sym)
{
  if (s.work.ncols122 == 0) return cudaSuccess;
  k_comm122_w<<<dim3(s.work.ncols122, 1, nz), 128, 0, st>>>(s.dev, s.work, X, Y, W2, zo);
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || !sym) return e;
  k_sym_subtract<<<dim3(nsym_tiles, 1, nz), 256, 0, st>>>(s.dev, W2, Z, hZ, sym_tiles, nsym_tiles, zo);
  count_launch();
  return cudaGetLastError();
}

cudaError_t load_comm122_kernels()
{
  // cudaFuncGetAttributes loads a kernel's module under lazy module loading
  cudaFuncAttributes a;
  cudaError_t e = cudaFuncGetAttributes(&a, k_comm122_w);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, k_sym_subtract);
  return e;
}

// grid of a grid-stride elementwise kernel over n elements: at most cap blocks
// (a few waves at emax >= 8), fewer for small arenas, so that small operators
// do not fill the GPU with idle blocks (commutators of different spaces run
// side by side in a batch)
static unsigned stride_grid(long long n, unsigned cap)
{
  long long b = (n + 255) / 256;
  return (unsigned)std::max(1LL, std::min<long long>(b, cap));
}

cudaError_t launch_to_ff(const Space& s, const double* A, float2* Af, cudaStream_t st, const long long* zo, int nz,
                         int rsrc, int rdst)
{
  k_to_ff<<<dim3(stride_grid(s.arena, 2432), 1, nz), 256, 0, st>>>(A, Af, s.arena, zo, rsrc, rdst);
  count_launch();
  return cudaGetLastError();
}

// comm122ss in the split form without the W2 round trip: one block per pair
// of 32 x 32 tiles (a, b), a <= b, of a channel block.  It forms W2's tile
// (rows a, columns b) and, for a != b, its tile (rows b, columns a) in shared
// memory -- each element the same double-float sum over the column's gather
// list as k_comm122_w_df -- and subtracts
//   Z(a, b) -= W2(a, b) + hZ W2(b, a)^T,  Z(b, a) -= W2(b, a) + hZ W2(a, b)^T
// directly (src/Commutator.cc:837-932; the symmetrisation of :927-929).
__global__ void __launch_bounds__(256) k_comm122_fused_df(DevSpace S, DevWork W, const double* __restrict__ X,
                                                          const double* __restrict__ Y,
                                                          const float2* __restrict__ Xf,
                                                          const float2* __restrict__ Yf, double* __restrict__ Z,
                                                          int hZ, const int* __restrict__ tiles, int ntiles,
                                                          const long long* __restrict__ zo)
{
  X = zsh(X, zo, ZR_X);
  Y = zsh(Y, zo, ZR_Y);
  Xf = zsh(Xf, zo, ZR_XF);
  Yf = zsh(Yf, zo, ZR_YF);
  Z = zsh(Z, zo, ZR_Z);
  __shared__ float2 cx[32][32], cy[32][32];  // per column of the tile being formed: coefficients
  __shared__ int cl[32][32], ccnt[32];       // and source columns
  __shared__ float2 wab[32][33], wba[32][33];
  const int t = blockIdx.x;
  if (t >= ntiles) return;
  const int ch = tiles[3 * t], ta = tiles[3 * t + 1], tb = tiles[3 * t + 2];
  const int n = S.ch_n[ch];
  const long long off = S.ch_off[ch];
  const int N = S.norb;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int col0 = S.ch_kofs[ch];  // the channel's first entry in the column list
  // one tile of W2: rows from tile tr, columns from tile tc, into w
  auto form = [&](int tr, int tc, float2 (*w)[33]) {
    // gather lists of the tile's columns (a warp per 4 columns, a lane per item)
    for (int cc = warp; cc < 32; cc += 8) {
      const int c = tc * 32 + cc;
      int cnt = 0, first = 0;
      if (c < n) {
        first = W.cols122[4 * (col0 + c) + 2];
        cnt = min(W.cols122[4 * (col0 + c) + 3], 32);
      }
      if (lane < cnt) {
        const int a = W.it122_a[first + lane], src = W.it122_src[first + lane];
        const double f = W.it122_f[first + lane];
        cx[cc][lane] = d2ff(X[32 + (size_t)src * N + a] * f);   //  X1(a, src) f multiplies Y2
        cy[cc][lane] = d2ff(-Y[32 + (size_t)src * N + a] * f);  // -Y1(a, src) f multiplies X2
        cl[cc][lane] = W.it122_loc[first + lane];
      }
      if (lane == 0) ccnt[cc] = cnt;
    }
    __syncthreads();
    const int r = tr * 32 + lane;
    for (int cc = warp; cc < 32; cc += 8) {
      float s = 0.f, e = 0.f;
      if (r < n) {
        const int cnt = ccnt[cc];
        for (int k = 0; k < cnt; ++k) {
          const long long el = off + (long long)cl[cc][k] * n + r;
          df_fma(cx[cc][k], Yf[el], s, e);
          df_fma(cy[cc][k], Xf[el], s, e);
        }
      }
      w[lane][cc] = make_float2(s, e);  // w[row][column]
    }
    __syncthreads();
  };
  form(ta, tb, wab);
  if (ta != tb) form(tb, ta, wba);
  const float2(*wt)[33] = ta != tb ? wba : wab;  // the tile holding W2(b-rows, a-columns)
  // Z(a, b) -= W2(a, b) + hZ W2(b, a)^T: lanes over rows of tile a
  for (int cc = warp; cc < 32; cc += 8) {
    const int r = ta * 32 + lane, c = tb * 32 + cc;
    if (r < n && c < n) {
      const float2 w = wab[lane][cc];
      float2 u = wt[cc][lane];
      if (hZ < 0) {
        u.x = -u.x;
        u.y = -u.y;
      }
      float hi, lo;
      df_add(w.x, w.y, u.x, u.y, hi, lo);
      Z[off + (long long)c * n + r] -= ff2d(hi, lo);
    }
  }
  if (ta == tb) return;
  // Z(b, a) -= W2(b, a) + hZ W2(a, b)^T: lanes over rows of tile b
  for (int cc = warp; cc < 32; cc += 8) {
    const int r = tb * 32 + lane, c = ta * 32 + cc;
    if (r < n && c < n) {
      const float2 w = wba[lane][cc];
      float2 u = wab[cc][lane];
      if (hZ < 0) {
        u.x = -u.x;
        u.y = -u.y;
      }
      float hi, lo;
      df_add(w.x, w.y, u.x, u.y, hi, lo);
      Z[off + (long long)c * n + r] -= ff2d(hi, lo);
    }
  }
}

cudaError_t launch_comm122_fused_df(const Space& s, const double* X, const double* Y, double* Z, const float2* Xf,
                                    const float2* Yf, int hZ, const int* tiles, int ntiles, cudaStream_t st,
                                    const long long* zo, int nz)
{
  if (ntiles == 0) return cudaSuccess;
  k_comm122_fused_df<<<dim3(ntiles, 1, nz), 256, 0, st>>>(s.dev, s.work, X, Y, Xf, Yf, Z, hZ, tiles, ntiles, zo);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_comm122_df(const Space& s, const double* X, const double* Y, double* Z, const float2* Xf,
                              const float2* Yf, float2* W2, int hZ, const int* sym_tiles, int nsym_tiles,
                              cudaStream_t st, const long long* zo, int nz, bool sym)
{
  if (s.work.ncols122 == 0) return cudaSuccess;
  k_comm122_w_df<<<dim3(s.work.ncols122, 1, nz), 128, 0, st>>>(s.dev, s.work, X, Y, Xf, Yf, W2, zo);
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || !sym) return e;
  k_sym_subtract_ff<<<dim3(nsym_tiles, 1, nz), 256, 0, st>>>(s.dev, W2, Z, hZ, sym_tiles, nsym_tiles, zo);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_pandya_fwd(const Space& s, const double* X, const double* Y, int hY, double* Xb, double* Yt,
                              double* Yf, bool df, cudaStream_t st, const long long* zo, int nz)
{
  if (s.work.n_pfout == 0) return cudaSuccess;
  auto kern = df ? k_pandya_fwd<true> : k_pandya_fwd<false>;
  kern<<<dim3((s.work.n_pfout + 255) / 256, 1, nz), 256, 0, st>>>(s.work, X, Y, hY, Xb, Yt, Yf, zo);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_pandya_inv(const Space& s, const double* Zb, double* Z, int hZ, const int* tiles, int ntiles,
                              cudaStream_t st)
{
  if (ntiles == 0) return cudaSuccess;
  k_pandya_inv<<<ntiles, 256, 0, st>>>(s.dev, s.work, Zb, Z, hZ, tiles, ntiles);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_pandya_inv_ff(const Space& s, const double* Zb, double* Z, int hZ, const int* tasks, int ntasks,
                                 const int* clist, const int* coff, const unsigned char* csort, int smem,
                                 cudaStream_t st, const long long* zo, int nz)
{
  if (ntasks == 0) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(k_pandya_inv_ff, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  k_pandya_inv_ff<<<dim3(ntasks, 1, nz), kInvqThreads, smem, st>>>(s.dev, s.work, Zb, Z, hZ, (const int4*)tasks,
                                                                     clist, coff, csort, zo);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_pandya_single(const Space& s, const double* Z, int herm, int transpose, double* out,
                                 cudaStream_t st)
{
  cudaError_t e = cudaMemsetAsync(out, 0, std::max<int64_t>(1, s.xb_total) * sizeof(double), st);
  if (e != cudaSuccess) return e;
  long long most = 0;
  for (int c = 0; c < s.nch; ++c) most = std::max(most, 2LL * s.cc_nph[c] * s.cc[c].n());
  if (most == 0) return cudaSuccess;
  dim3 grid((unsigned)((most + 255) / 256), (unsigned)s.nch);
  k_pandya_single<<<grid, 256, 0, st>>>(s.dev, s.work, Z, herm, transpose, out);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_generator(const Space& s, const double* H, double* Eta, double* mono, const GenParams& p,
                             cudaStream_t st)
{
  cudaError_t e = cudaMemsetAsync(Eta, 0, s.arena * sizeof(double), st);
  if (e != cudaSuccess) return e;
  int nn = s.norb * s.norb;
  int blocks = (nn + 255) / 256;
  if (p.partitioning == DENOM_EPSTEIN_NESBET) {
    k_gen_monopoles<<<blocks, 256, 0, st>>>(s.dev, H, mono);
    count_launch();
  }
  k_gen_onebody<<<blocks, 256, 0, st>>>(s.dev, H, mono, Eta, p);
  count_launch();
  k_gen_twobody<<<s.nch, 256, 0, st>>>(s.dev, s.work, H, mono, Eta, p);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_axpy(double* y, const double* x, double a, long long n, cudaStream_t st)
{
  k_axpy<<<stride_grid(n, 1216), 256, 0, st>>>(y, x, a, n);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_scale(double* y, double a, long long n, cudaStream_t st)
{
  k_scale<<<stride_grid(n, 1216), 256, 0, st>>>(y, a, n);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_axpy_norm(const Space& s, double* y, const double* x, double a, const long long* chunk_off,
                             const int* chunk_len, const double* chunk_w, int nchunks, double* partial,
                             cudaStream_t st)
{
  // the one-body block first: it is the longest
  k_axpy_norm<<<nchunks + 1, 256, 0, st>>>(s.dev, y, x, a, chunk_off, chunk_len, chunk_w, partial, nchunks);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_norm(const Space& s, const double* A, const long long* chunk_off, const int* chunk_len,
                        const double* chunk_w, int nchunks, double* partial, cudaStream_t st)
{
  k_norm_onebody<<<1, 256, 0, st>>>(s.dev, A, partial + nchunks);
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || nchunks == 0) return e;
  k_norm_chunks<<<nchunks, 256, 0, st>>>(A, chunk_off, chunk_len, chunk_w, partial, nchunks);
  count_launch();
  return cudaGetLastError();
}

}  // namespace imsrg
