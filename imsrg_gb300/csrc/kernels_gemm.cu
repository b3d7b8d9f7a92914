// FP64 "symmetrised channel product" on CUDA cores:
//     Out (+)= P + sign * phi_i phi_j * P^T,   P = A B^T,
// evaluated on tile pairs (I <= J) so the transpose-add of the reference is
// fused into the epilogue (no intermediate M / Zbar-before-symmetrisation in
// HBM).  Two users:
//   * the pp/hh ladder of comm222_pp_hhss (ConstructScalarMpp_Mhh,
//     src/Commutator.cc:1170-1194, then Z += Mpp - Mhh, :1237-1238):
//     A(i,t) = X(i, k_t) = hX X(k_t, i), B(j,t) = hY w_t Y(j, k_t),
//     Out = Z2 block (accumulate), sign = hZ;
//   * the Pandya-space product of comm222_phss (src/Commutator.cc:1789-1805):
//     A = Xbar, B = Ybar^T (head, sign = hZ) or Yflip^T (tail, sign = +1 and
//     phases phi), Out = Zbar (overwrite).
// 64 x 64 tiles, 256 threads, each thread a 4 x 4 register block per tile.
#include <cuda_runtime.h>

#include "kernels.cuh"
#include "prof.hpp"

namespace imsrg {

namespace {
constexpr int TM = 64;
constexpr int TK = 16;
constexpr int LDS = TM + 1;
}  // namespace

__global__ void __launch_bounds__(256) k_symgemm_fp64(const GemmJobDev* __restrict__ jobs,
                                                      const int* __restrict__ pairs, int npairs,
                                                      const double* __restrict__ Abase,
                                                      const double* __restrict__ B0, const double* __restrict__ B1,
                                                      double* __restrict__ Obase, const int* __restrict__ kidx,
                                                      const double* __restrict__ kw, const int* __restrict__ phase,
                                                      int gsign, double gbscale)
{
  extern __shared__ double smem[];
  int pid = blockIdx.x;
  if (pid >= npairs) return;
  const GemmJobDev jb = jobs[pairs[3 * pid]];
  const int ti = pairs[3 * pid + 1], tj = pairs[3 * pid + 2];
  const bool diag = (ti == tj);
  const int m = jb.m, K = jb.K;
  const double* A = Abase + jb.a_off;
  const double* B = (jb.bsel ? B1 : B0) + jb.b_off;
  const int* kx = jb.kidx_off >= 0 ? kidx + jb.kidx_off : nullptr;
  const double* w = jb.w_off >= 0 ? kw + jb.w_off : nullptr;

  double* AsI = smem;             // [TK][TM]
  double* AsJ = AsI + TK * TM;
  double* BsI = AsJ + TK * TM;
  double* BsJ = BsI + TK * TM;

  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  double acc1[4][4], acc2[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc1[a][b] = acc2[a][b] = 0.0;

  const int I0 = ti * TM, J0 = tj * TM;
  for (int k0 = 0; k0 < K; k0 += TK) {
    // each thread loads 4 elements of each of the four tiles
#pragma unroll
    for (int rep = 0; rep < 4; ++rep) {
      int e = tid + rep * 256;  // 0..1023
      int kk = e >> 6, r = e & 63;
      int t = k0 + kk;
      double aI = 0, aJ = 0, bI = 0, bJ = 0;
      if (t < K) {
        int col = kx ? kx[t] : t;
        double sc = jb.bscale * gbscale * (w ? w[t] : 1.0);
        const double* ac = A + (long long)col * jb.lda;
        const double* bc = B + (long long)col * jb.ldb;
        if (I0 + r < m) {
          aI = ac[I0 + r];
          bI = sc * bc[I0 + r];
        }
        if (J0 + r < m) {
          aJ = ac[J0 + r];
          bJ = sc * bc[J0 + r];
        }
      }
      AsI[kk * TM + r] = aI;
      AsJ[kk * TM + r] = aJ;
      BsI[kk * TM + r] = bI;
      BsJ[kk * TM + r] = bJ;
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < TK; ++kk) {
      double ra[4], rb[4], ra2[4], rb2[4];
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        ra[a] = AsI[kk * TM + ty * 4 + a];
        rb[a] = BsJ[kk * TM + tx * 4 + a];
        ra2[a] = AsJ[kk * TM + ty * 4 + a];
        rb2[a] = BsI[kk * TM + tx * 4 + a];
      }
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          acc1[a][b] = fma(ra[a], rb[b], acc1[a][b]);
          if (!diag) acc2[a][b] = fma(ra2[a], rb2[b], acc2[a][b]);
        }
    }
    __syncthreads();
  }

  // epilogue: S1 = P(I,J), S2 = P(J,I) in shared memory
  double* S1 = smem;
  double* S2 = smem + TM * LDS;
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      S1[(ty * 4 + a) * LDS + tx * 4 + b] = acc1[a][b];
      if (!diag) S2[(ty * 4 + a) * LDS + tx * 4 + b] = acc2[a][b];
    }
  __syncthreads();
  const int* ph = jb.phase_off >= 0 ? phase + jb.phase_off : nullptr;
  double* O = Obase + jb.out_off;
  const double sgn = (double)(jb.sign != 0 ? jb.sign : gsign);
  for (int e = tid; e < TM * TM; e += 256) {
    int r = e & 63, c = e >> 6;  // r fastest -> coalesced column-major stores
    int i = I0 + r, j = J0 + c;
    if (i < m && j < m) {
      double p = diag ? S1[c * LDS + r] : S2[c * LDS + r];  // P(j,i)
      double f = ph ? (double)(ph[i] * ph[j]) : 1.0;
      double v = S1[r * LDS + c] + sgn * f * p;
      long long o = (long long)j * jb.ldo + i;
      O[o] = jb.accumulate ? O[o] + v : v;
    }
    if (!diag) {
      // Out(J, I): rows from J, cols from I
      int i2 = J0 + r, j2 = I0 + c;
      if (i2 < m && j2 < m) {
        double f = ph ? (double)(ph[i2] * ph[j2]) : 1.0;
        double v = S2[r * LDS + c] + sgn * f * S1[c * LDS + r];
        long long o = (long long)j2 * jb.ldo + i2;
        O[o] = jb.accumulate ? O[o] + v : v;
      }
    }
  }
}

size_t symgemm_fp64_smem() { return (size_t)2 * TM * LDS * sizeof(double); }
int symgemm_fp64_tile() { return TM; }

cudaError_t launch_symgemm_fp64(const GemmJobDev* jobs, const int* pairs, int npairs, const double* A,
                                const double* B0, const double* B1, double* O, const int* kidx, const double* kw,
                                const int* phase, int gsign, double gbscale, cudaStream_t st)
{
  if (npairs == 0) return cudaSuccess;
  static bool attr = false;
  size_t sm = symgemm_fp64_smem();
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_symgemm_fp64, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  k_symgemm_fp64<<<npairs, 256, sm, st>>>(jobs, pairs, npairs, A, B0, B1, O, kidx, kw, phase, gsign, gbscale);
  count_launch();
  return cudaGetLastError();
}

}  // namespace imsrg
