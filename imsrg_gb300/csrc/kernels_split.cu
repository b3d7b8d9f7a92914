// Split-precision symmetrised channel products on the Blackwell tensor cores.
//
// Computes, for every job (a channel block), the same quantity as
// k_symgemm_fp64 (kernels_gemm.cu):
//     Out (+)= P + s phi_i phi_j P^T,   P = A B^T,   A, B: m x K FP64
// as an Ozaki-style sum of exact BF16 digit products:
//
//  * Digits.  Each row i gets one exponent a_i for its A row and b_i = a_i + c
//    for its B row (c is one per job), chosen so both rows fit below the
//    exponent.  Every element is rounded to an integer q = v * 2^(beta*S - e)
//    (|q| <= 2^(beta*S)) and split into S balanced base-2^beta digits
//    (|d_1| <= 2^beta, |d_s| <= 2^(beta-1)), all exact in BF16.  Only integer
//    instructions are used (FP64 runs at 1/57 of the FP32 rate on this part).
//  * Symmetrisation folded into K.  With the shared-exponent choice both
//    A_i.B_j and B_i.A_j carry the scale 2^(a_i + a_j + c), so
//        Out(i,j) = sum_t [A(i,t) | s phi_i B(i,t)] . [B(j,t) | phi_j A(j,t)]
//    is one product with K doubled; only tiles of the upper triangle are
//    computed and each is written together with its mirror (no transpose
//    pass, no extra flops over P alone).
//  * Products.  The digit products with s + t <= S + 1 are issued as
//    tcgen05.mma kind::f16 (BF16 in, FP32 accumulate in tensor memory), one
//    TMEM accumulator per weight group T = s + t.  beta is chosen from K so
//    that the FP32 sums of the leading groups stay exact integers.
//  * Recombination.  The epilogue reads the S group sums (tcgen05.ld), merges
//    them exactly as int64, converts once to FP64 and applies the power-of-two
//    scale by exponent arithmetic.  Tensor memory is a ring of accumulator
//    blocks, so the next tile's products run while the epilogue drains a tile.
//  * Plain jobs (nosym): Out (+)= A B^T with A m x K, B n x K, each row of A
//    and of B with its own exponent, K not doubled, every tile of the m x n
//    output (the rectangular products of the scalar-tensor commutator).
//
// Kernel layout (persistent, one CTA per SM, 320 threads):
//   warp 0: TMA producer (cp.async.bulk.tensor, 64B swizzle, mbarrier pipeline;
//           one 3-D box per operand and stage, holding every digit plane)
//   warp 1: TMEM allocator + single-thread MMA issuer
//   warps 2-9: epilogue (two warps per TMEM lane quarter, each on half the columns)
// Every mbarrier wait is bounded; a timeout sets the status word and the CTA
// drains and exits.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <vector>

#include "kernels.cuh"
#include "prof.hpp"

namespace imsrg {

namespace {

constexpr int KB = 32;          // K elements (bf16) per pipeline stage: one 64-byte swizzle row
constexpr int TILE_M = 128;     // rows per tile (UMMA M)
constexpr int MAX_S = 7;
constexpr int EPI_COLS = 8;     // TMEM columns read per tcgen05.ld
// bounded spin: every mbarrier wait gives up after WAIT_LIMIT try_wait rounds.
// One round (try_wait's own suspend plus the nanosleep backoff) measured
// about 8000 SM cycles on GB300 (imsrg_space_wait_selftest), so the bound is
// about 2 s at 2 GHz; the longest wait of a healthy launch (one tile's MMAs)
// is microseconds
constexpr unsigned WAIT_LIMIT = 1u << 19;
constexpr int EXP_NONE = -100000;          // exponent of an all-zero row

struct SplitJob {
  long long a_off, b_off, out_off;
  int m, K, lda, ldb, ldo;
  int kidx_off, w_off, phase_off;
  int bsel, sign, accumulate;
  double bscale;
  // slice layout: digit s of row i of this job is row exp_base + i of digit
  // plane s (every slice array is S planes of the same row count)
  long long exp_base;  // first row of this job in the exponent arrays and in each digit plane
  int m_pad, K_pad, nkb;
  int nosym, n;        // plain product: B rows (n = m for the symmetrised form)
  int nkt;             // K blocks per tile: nkb (plain) or 2 nkb (K doubled)
};

struct SplitTile {
  int job, I, J, diag;
};

}  // namespace

struct SplitPlan {
  int family = 0;
  int S = 6, beta = 6;
  int K_stride = 0;
  long long total_exp_rows = 0;   // rows of one digit plane (and of the exponent arrays)
  int njobs = 0, ntiles = 0;
  std::vector<SplitJob> jobs;
  SplitJob* d_jobs = nullptr;
  SplitTile* d_tiles = nullptr;
  __nv_bfloat16* arr[4] = {nullptr, nullptr, nullptr, nullptr};  // alpha, beta, gamma, delta
  int* d_rexpA = nullptr;   // raw row exponent of A rows
  int* d_rexpB = nullptr;
  int* d_jobmax = nullptr;  // [2 * njobs]: max exponent of A, of B
  int* d_flags = nullptr;   // [2 * njobs]: gamma used, delta used (set per launch)
  int4* d_rblk = nullptr;   // exponent blocks (job, 32-row group, 256-column chunk)
  int4* d_dblk = nullptr;   // digit blocks (job, 32-row group, KB-column chunk), jobs in reverse order
  int n_rblk = 0, n_dblk = 0;
  // 3-D maps (K, plane row, digit): A-operand role (TILE_M-row boxes) of
  // alpha, beta, gamma, then B-operand role (tn-row boxes) of alpha, beta, delta
  CUtensorMap maps[6];
  int grid = 0;
  size_t smem = 0;
  int nstages = 0;
  int accum_override = -1;
  int mirror = 1;  // 0: symmetrised jobs write only their upper triangle
  int tn = 64, nacc = 1, epiw = 4;  // tile columns, tuning label of the tile (64 x 1 or 32 x 2), epilogue warps
  int stages_opt = 0, sched = 0;    // requested pipeline stages (0: most that fit), tile schedule
  int* d_cta = nullptr;             // [grid + 1]: each CTA's tiles are tiles[d_cta[b] .. d_cta[b + 1])
  bool shared_gd = false;           // gamma / delta alias beta / alpha (plain jobs only)
  bool plain = false;               // every job is a plain product (a plan holds one kind)
};

// ----------------------------------------------------------------- device
namespace {

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned a, unsigned count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned a, unsigned bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(unsigned a)
{
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(a) : "memory");
}

__device__ __forceinline__ bool mbar_try(unsigned a, unsigned parity)
{
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(a), "r"(parity)
      : "memory");
  return ok != 0;
}

// bounded wait: false on timeout
__device__ __forceinline__ bool mbar_wait(unsigned a, unsigned parity, unsigned limit = WAIT_LIMIT)
{
  for (unsigned it = 0; it < limit; ++it) {
    if (mbar_try(a, parity)) return true;
    if (it > 64) __nanosleep(it > 4096 ? 256 : 32);
  }
  return false;
}

// one box of all S digit planes: coordinates (K element, plane row, digit 0)
__device__ __forceinline__ void tma_load_3d(unsigned dst, const CUtensorMap* map, int x, int y, unsigned bar)
{
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(dst),
      "l"((unsigned long long)map), "r"(x), "r"(y), "r"(0), "r"(bar)
      : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tc_mma(unsigned d_tmem, unsigned long long adesc, unsigned long long bdesc,
                                       unsigned idesc, unsigned accumulate)
{
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void tc_commit(unsigned bar)
{
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// UMMA shared-memory descriptor: K-major operand, 64-byte swizzle
// (8 rows x 64 bytes per swizzle atom, 512 bytes between 8-row groups).
__device__ __forceinline__ unsigned long long sdesc_sw64(unsigned addr)
{
  unsigned long long d = 0;
  d |= (unsigned long long)((addr >> 4) & 0x3FFF);
  d |= (unsigned long long)1 << 16;             // leading byte offset (unused for swizzled K-major)
  d |= (unsigned long long)(512 >> 4) << 32;    // stride byte offset
  d |= (unsigned long long)1 << 46;             // descriptor version (sm_100 family)
  d |= (unsigned long long)4 << 61;             // layout: 64-byte swizzle
  return d;
}

// instruction descriptor, kind::f16: BF16 x BF16 -> F32, both K-major
// (bit 13, set by the caller where needed, negates the A operand)
__host__ __device__ constexpr unsigned idesc_bf16(int M, int N)
{
  return (1u << 4)                   // D format F32
         | (1u << 7)                 // A format BF16
         | (1u << 10)                // B format BF16
         | ((unsigned)(N >> 3) << 17)  // N / 8
         | ((unsigned)(M >> 4) << 24); // M / 16
}

__device__ __forceinline__ void tmem_ld8(unsigned taddr, unsigned (&r)[8])
{
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ void set_status(int* st, int code)
{
  if (st) atomicCAS(st, 0, code);
}

// biased exponent field of a double (0 for zero / subnormal)
__device__ __forceinline__ int dexp(double v) { return (int)((__double_as_longlong(v) >> 52) & 0x7FF); }

// q = round(v * 2^(P - e)) for |v| < 2^e, P = beta*S <= 42; integer only
__device__ __forceinline__ long long to_fixed(double v, int e, int P)
{
  long long bits = __double_as_longlong(v);
  int E = (int)((bits >> 52) & 0x7FF);
  if (E == 0) return 0;
  long long M = (bits & 0xFFFFFFFFFFFFFll) | 0x10000000000000ll;
  int r = 1075 - E - P + e;  // right shift, >= 11 since |v| < 2^e
  if (r >= 64 || r <= 0) return 0;  // r >= 11 whenever |v| < 2^e
  long long q = (M + (1ll << (r - 1))) >> r;
  return bits < 0 ? -q : q;
}

// ------------------------------------------------------------ column scales
// The B operand is taken with a per-column scale (job scale x launch scale x
// ladder weight).  A scale that is a signed power of two, as every weight of
// a closed-shell reference is, is applied by exponent arithmetic and a sign
// (integer instructions); any other scale by an FP64 multiply.
constexpr int SC_GENERAL = 0x40000000;

// code of a scale: (k << 1) | sign for +-2^k, SC_GENERAL otherwise
__device__ __forceinline__ int scale_code(double sc)
{
  const long long b = __double_as_longlong(sc);
  const int E = (int)((b >> 52) & 0x7FF);
  if ((b & 0xFFFFFFFFFFFFFll) != 0 || E == 0 || E == 0x7FF) return SC_GENERAL;
  return ((E - 1023) << 1) | (int)((unsigned long long)b >> 63);
}

// biased exponent of v * scale (0 for zero / subnormal)
__device__ __forceinline__ int dexp_scaled(double v, int code, double sc)
{
  if (code == SC_GENERAL) return dexp(v * sc);
  const int e = dexp(v);
  if (e == 0) return 0;
  const int es = e + (code >> 1);
  return es < 1 ? 0 : es;
}

// ------------------------------------------------------------ exponents
// raw row exponents (max biased exponent over the row) of A and B, and the
// per-job maxima.  One block per listed (job, 32-row group, 256-column chunk):
// 32 rows x 8 column lanes; partial maxima combine through atomicMax (the
// arrays are zeroed first).  The exponent of B includes the column scale so
// the B digits are taken of the scaled values.
// (PLAIN: a plan of plain jobs, whose A rows (i < m) and B rows (i < n) are
// counted separately; the symmetrised form keeps its single row test)
template <bool PLAIN>
__global__ void __launch_bounds__(256) k_split_rowexp(const SplitJob* __restrict__ jobs, const int4* __restrict__ blocks,
                                                      const double* __restrict__ Abase,
                                                      const double* __restrict__ B0, const double* __restrict__ B1,
                                                      const int* __restrict__ kidx, const double* __restrict__ kw,
                                                      double gbscale, int* __restrict__ rexpA,
                                                      int* __restrict__ rexpB, int* __restrict__ jobmax)
{
  __shared__ int sa[8][33], sb[8][33];
  __shared__ int s_col[256], s_code[256];
  __shared__ double s_sc[256];
  const int4 bk = blocks[blockIdx.x];
  const int job = bk.x;
  const SplitJob jb = jobs[job];
  const int r = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int i = bk.y * 32 + r;
  const int t0 = bk.z * 256;
  const int tend = min(jb.K, t0 + 256);
  {
    // column indices and scales of this chunk, once per block
    const int* kx = jb.kidx_off >= 0 ? kidx + jb.kidx_off : nullptr;
    const double* w = jb.w_off >= 0 ? kw + jb.w_off : nullptr;
    const double sc0 = jb.bscale * gbscale;
    const int t = t0 + threadIdx.x;
    if (t < tend) {
      const double sc = w ? sc0 * w[t] : sc0;
      s_col[threadIdx.x] = kx ? kx[t] : t;
      s_sc[threadIdx.x] = sc;
      s_code[threadIdx.x] = scale_code(sc);
    }
  }
  __syncthreads();
  int ea = 0, eb = 0;
  const double* A = Abase + jb.a_off;
  const double* B = (jb.bsel ? B1 : B0) + jb.b_off;
  if (!PLAIN) {
    if (i < jb.m) {
      // four columns' loads in flight per thread (the pass is bound by them)
      int t = t0 + ty;
      for (; t + 24 < tend; t += 32) {
        double a[4], b[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int col = s_col[t + 8 * u - t0];
          a[u] = A[(long long)col * jb.lda + i];
          b[u] = B[(long long)col * jb.ldb + i];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          ea = max(ea, dexp(a[u]));
          eb = max(eb, dexp_scaled(b[u], s_code[t + 8 * u - t0], s_sc[t + 8 * u - t0]));
        }
      }
      for (; t < tend; t += 8) {
        const int col = s_col[t - t0];
        ea = max(ea, dexp(A[(long long)col * jb.lda + i]));
        eb = max(eb, dexp_scaled(B[(long long)col * jb.ldb + i], s_code[t - t0], s_sc[t - t0]));
      }
    }
  } else {
    if (i < jb.m)
      for (int t = t0 + ty; t < tend; t += 8) ea = max(ea, dexp(A[(long long)s_col[t - t0] * jb.lda + i]));
    if (i < jb.n)
      for (int t = t0 + ty; t < tend; t += 8)
        eb = max(eb, dexp_scaled(B[(long long)s_col[t - t0] * jb.ldb + i], s_code[t - t0], s_sc[t - t0]));
  }
  sa[ty][r] = ea;
  sb[ty][r] = eb;
  __syncthreads();
  if (ty == 0) {
    for (int y = 1; y < 8; ++y) {
      ea = max(ea, sa[y][r]);
      eb = max(eb, sb[y][r]);
    }
    if (ea) atomicMax(rexpA + jb.exp_base + i, ea);
    if (eb) atomicMax(rexpB + jb.exp_base + i, eb);
    int wa = ea, wb = eb;
    for (int o = 16; o > 0; o >>= 1) {
      wa = max(wa, __shfl_xor_sync(0xffffffffu, wa, o));
      wb = max(wb, __shfl_xor_sync(0xffffffffu, wb, o));
    }
    if (r == 0) {
      if (wa) atomicMax(jobmax + 2 * job, wa);
      if (wb) atomicMax(jobmax + 2 * job + 1, wb);
    }
  }
}

// signed 64-bit integer times 2^X as a double, integer instructions only
// (round to nearest even); 0 on underflow of the exponent range.
__device__ __forceinline__ double i64_ldexp(long long v, int X)
{
  if (v == 0) return 0.0;
  unsigned long long sgn = v < 0 ? (1ull << 63) : 0ull;
  unsigned long long u = v < 0 ? (unsigned long long)(-v) : (unsigned long long)v;
  int lz = __clzll((long long)u);
  unsigned long long m = u << lz;            // leading one at bit 63
  unsigned long long mant = m >> 11;         // 53 bits
  unsigned long long rest = m & 0x7FFull;
  if (rest > 0x400ull || (rest == 0x400ull && (mant & 1ull))) {
    ++mant;
    if (mant >> 53) {
      mant >>= 1;
      --lz;
    }
  }
  int e = (63 - lz) + 1023 + X;
  if (e <= 0) return 0.0;
  if (e >= 2047) return __longlong_as_double((long long)(sgn | (0x7FFull << 52)));
  return __longlong_as_double((long long)(sgn | ((unsigned long long)e << 52) | (mant & 0xFFFFFFFFFFFFFull)));
}

// exponent of row i (A side) from the raw exponents: a_i = max(eA, eB - c)
__device__ __forceinline__ int row_exp(int eA, int eB, int c)
{
  int a = eA > 0 ? eA - 1022 : EXP_NONE;
  int b = eB > 0 ? eB - 1022 - c : EXP_NONE;
  return max(a, b);
}

// exponent of a row of a plain job's A or B from its raw exponent
__device__ __forceinline__ int own_exp(int e) { return e > 0 ? e - 1022 : EXP_NONE; }

__device__ __forceinline__ int job_c(const int* jobmax, int job)
{
  int ma = jobmax[2 * job], mb = jobmax[2 * job + 1];
  if (ma == 0 || mb == 0) return 0;
  return mb - ma;
}

// ---------------------------------------------------------------- digits
// One block per listed (job, 32-row group, KB-column group): digits of A and
// B rows into shared memory, then coalesced 16-byte stores of the four slice
// arrays
//   alpha = A digits, beta = B digits, gamma = s phi_i B digits, delta = phi_i A digits
// (gamma / delta written only when they differ from beta / alpha).
template <int S, bool PLAIN>
__global__ void __launch_bounds__(256) k_split_digits(const SplitJob* __restrict__ jobs, const int4* __restrict__ blocks,
                                                     const double* __restrict__ Abase,
                                                     const double* __restrict__ B0, const double* __restrict__ B1,
                                                     const int* __restrict__ kidx, const double* __restrict__ kw,
                                                     const int* __restrict__ phase, double gbscale, int gsign,
                                                     const int* __restrict__ rexpA, const int* __restrict__ rexpB,
                                                     const int* __restrict__ jobmax, const int* __restrict__ flags,
                                                     int beta, int K_stride, long long plane_rows,
                                                     __nv_bfloat16* __restrict__ alpha, __nv_bfloat16* __restrict__ bet,
                                                     __nv_bfloat16* __restrict__ gam, __nv_bfloat16* __restrict__ del)
{
  // rows of KB + 2 digits = 17 words: the 32 rows a warp writes at once fall
  // in 32 different banks
  constexpr int RW = (KB + 2) / 2;
  __shared__ unsigned dA[S][32][RW];
  __shared__ unsigned dB[S][32][RW];
  __shared__ int rowA[32], rowB[32], rowsg[32], rowph[32];
  __shared__ int s_col[KB], s_code[KB];
  __shared__ double s_sc[KB];
  const int4 bk = blocks[blockIdx.x];
  const int job = bk.x;
  const SplitJob jb = jobs[job];
  const int r0 = bk.y * 32;
  const int t0 = bk.z * KB;
  const int c = PLAIN ? 0 : job_c(jobmax, job);
  const int sign = jb.sign != 0 ? jb.sign : gsign;
  const int* ph = jb.phase_off >= 0 ? phase + jb.phase_off : nullptr;
  if (threadIdx.x < 32) {
    const int i = r0 + threadIdx.x;
    if (PLAIN) {
      rowA[threadIdx.x] = own_exp(rexpA[jb.exp_base + i]);
      rowB[threadIdx.x] = own_exp(rexpB[jb.exp_base + i]);
    } else {
      const int a = row_exp(rexpA[jb.exp_base + i], rexpB[jb.exp_base + i], c);
      rowA[threadIdx.x] = a;
      rowB[threadIdx.x] = a + c;
    }
    const int p = (ph && i < jb.m) ? ph[i] : 1;
    rowph[threadIdx.x] = p;
    rowsg[threadIdx.x] = sign * p;
  } else if (threadIdx.x < 32 + KB) {
    const int tt = threadIdx.x - 32, t = t0 + tt;
    if (t < jb.K) {
      const double sc = jb.w_off >= 0 ? jb.bscale * gbscale * kw[jb.w_off + t] : jb.bscale * gbscale;
      s_col[tt] = jb.kidx_off >= 0 ? kidx[jb.kidx_off + t] : t;
      s_sc[tt] = sc;
      s_code[tt] = scale_code(sc);
    }
  }
  __syncthreads();
  const double* A = Abase + jb.a_off;
  const double* B = (jb.bsel ? B1 : B0) + jb.b_off;
  const int P = beta * S;
  const long long half = 1ll << (beta - 1), mask = (1ll << beta) - 1;
  long long bias = 0;
#pragma unroll
  for (int s = 1; s < S; ++s) bias += half << (beta * (S - 1 - s));
  // column pair (tt, tt + 1) of row r: thread layout r fastest (coalesced
  // column reads), the two digits of a pair packed in one 32-bit word.  Every
  // operand value of the thread's pairs is requested before the first is
  // converted (the pass is bound by those loads)
  constexpr int NIT = 32 * (KB / 2) / 256;
  double va[NIT][2], vb[NIT][2];
#pragma unroll
  for (int u = 0; u < NIT; ++u) {
    const int e = threadIdx.x + u * 256;
    const int r = e & 31, tp = e >> 5;
    const int i = r0 + r;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int tt = 2 * tp + h, t = t0 + tt;
      va[u][h] = 0.0;
      vb[u][h] = 0.0;
      if (!PLAIN ? (i < jb.m && t < jb.K) : (t < jb.K && (i < jb.m || i < jb.n))) {
        const int col = s_col[tt];
        if (!PLAIN || i < jb.m) va[u][h] = A[(long long)col * jb.lda + i];
        if (!PLAIN || i < jb.n) vb[u][h] = B[(long long)col * jb.ldb + i];
      }
    }
  }
#pragma unroll
  for (int u = 0; u < NIT; ++u) {
    const int e = threadIdx.x + u * 256;
    const int r = e & 31, tp = e >> 5;
    long long qa2[2], qb2[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int tt = 2 * tp + h, t = t0 + tt;
      long long qa = 0, qb = 0;
      if (t < jb.K) {  // the values outside the job are 0.0 and give 0
        const int code = s_code[tt];
        qa = to_fixed(va[u][h], rowA[r], P);
        if (code == SC_GENERAL) {
          qb = to_fixed(vb[u][h] * s_sc[tt], rowB[r], P);
        } else {
          qb = to_fixed(vb[u][h], rowB[r] - (code >> 1), P);
          if (code & 1) qb = -qb;
        }
      }
      // balanced digits by one biased add: the lower digits are the beta-bit
      // fields of q + bias minus half, the top digit the arithmetic shift of
      // the rest (bias = half * sum_{s >= 1} 2^(beta (S-1-s)), so the digits
      // still sum to q): |d| <= 2^(beta-1) below the top digit,
      // |d_1| <= 2^beta + 1
      qa2[h] = qa + bias;
      qb2[h] = qb + bias;
    }
    // small integer -> bf16 bits (exact): the float 1.5*2^23 + x minus
    // 1.5*2^23, whose upper 16 bits are the bf16 of x; for a lower digit the
    // "- half" rides in the magic constant.  The two columns' upper halves
    // are packed into one word by a byte permute.
    unsigned wa[S], wb[S];
#pragma unroll
    for (int s = 0; s < S; ++s) {
      const int sh = beta * (S - 1 - s);
      const int mg = s == 0 ? 0x4B400000 : 0x4B400000 - (int)half;
      float fa[2], fb[2];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int xa = s == 0 ? (int)(qa2[h] >> sh) : (int)((unsigned)(qa2[h] >> sh) & (unsigned)mask);
        const int xb = s == 0 ? (int)(qb2[h] >> sh) : (int)((unsigned)(qb2[h] >> sh) & (unsigned)mask);
        fa[h] = __int_as_float(mg + xa) - 12582912.0f;
        fb[h] = __int_as_float(mg + xb) - 12582912.0f;
      }
      wa[s] = __byte_perm(__float_as_uint(fa[0]), __float_as_uint(fa[1]), 0x7632);
      wb[s] = __byte_perm(__float_as_uint(fb[0]), __float_as_uint(fb[1]), 0x7632);
    }
#pragma unroll
    for (int s = 0; s < S; ++s) {
      dA[s][r][tp] = wa[s];
      dB[s][r][tp] = wb[s];
    }
  }
  __syncthreads();
  const bool need_g = flags[2 * job] == 1, need_d = flags[2 * job + 1] != 0;
  // stores: each thread one 16-byte vector (8 digits) of one row of one slice
  for (int e = threadIdx.x; e < S * 32 * (KB / 8); e += 256) {
    const int v = e % (KB / 8), r = (e / (KB / 8)) & 31, s = e / (32 * (KB / 8));
    const long long row = (long long)s * plane_rows + jb.exp_base + r0 + r;
    const long long o = row * K_stride + t0 + v * 8;
    const unsigned* qa = &dA[s][r][v * 4];
    const unsigned* qb = &dB[s][r][v * 4];
    const uint4 va = make_uint4(qa[0], qa[1], qa[2], qa[3]);
    const uint4 vb = make_uint4(qb[0], qb[1], qb[2], qb[3]);
    *(uint4*)(alpha + o) = va;
    *(uint4*)(bet + o) = vb;
    if (need_g) {
      uint4 vg = vb;
      if (rowsg[r] < 0) {
        vg.x ^= 0x80008000u; vg.y ^= 0x80008000u; vg.z ^= 0x80008000u; vg.w ^= 0x80008000u;
      }
      *(uint4*)(gam + o) = vg;
    }
    if (need_d) {
      uint4 vd = va;
      if (rowph[r] < 0) {
        vd.x ^= 0x80008000u; vd.y ^= 0x80008000u; vd.z ^= 0x80008000u; vd.w ^= 0x80008000u;
      }
      *(uint4*)(del + o) = vd;
    }
  }
}

// --------------------------------------------------------------- the GEMM
struct GemmArgs {
  const SplitJob* jobs;
  const SplitTile* tiles;
  const int* cta_first;  // [gridDim.x + 1]: the CTA's run of tiles
  int ntiles;
  const int* rexpA;
  const int* rexpB;
  const int* jobmax;
  const int* flags;   // [2*job]: second-half A operand (0 beta, 1 gamma, 2 beta negated by the MMA); [2*job+1]: delta used
  const int* phase;
  double* out;
  int* status;
  int S, beta, nstages, gsign;
  int accum;  // -1: each job's flag; 0: overwrite; 1: accumulate
  int nomirror;  // 1: symmetrised jobs skip the mirror (lower-triangle) stores
};

// Accumulators in tensor memory: NB = 512 / TN blocks of TN columns, one
// block per weight group (S groups a tile).  Even tiles (counted per CTA)
// keep group g in block g, odd tiles in block NB - S + g, so consecutive
// tiles share OV = 2S - NB blocks (none when 2S <= NB): the last OV groups of
// an even tile, the first OV groups of an odd one.  The epilogue folds those
// groups into a per-column int64 partial sum first and releases them, and the
// next tile's MMAs run under the rest of the epilogue.
template <int S, int TN>
struct AccPair {
  static constexpr int NB = 512 / TN;
  static constexpr int OV = 2 * S - NB > 0 ? 2 * S - NB : 0;
  static_assert(S <= NB, "a tile's groups exceed tensor memory");
  __device__ static unsigned base(int tc) { return (unsigned)((tc & 1) ? TN * (NB - S) : 0); }
  // first group the next tile overwrites (the early ones: [early_lo, early_lo + OV))
  __device__ static int early_lo(int tc) { return (tc & 1) ? 0 : S - OV; }
};

// TN: tile columns (UMMA N); EPIW: epilogue warps (4 or 8; with 8, two warps
// share a TMEM lane quarter and split the columns).
// The maps: the A-operand role (TILE_M-row boxes) of alpha, beta, gamma and
// the B-operand role (TN-row boxes) of alpha, beta, delta; each box holds all
// S digit planes, so one stage is two TMA loads.
// Registers are capped at 128 a thread (41k for the CTA), so the kernels of
// a second stream still fit beside the product on every SM; uncapped, the
// epilogue's per-column partial sums take it to 168 and the commutator's two
// streams stop overlapping.
template <int S, int TN, int EPIW>
__global__ void __maxnreg__(128) k_split_gemm(const __grid_constant__ CUtensorMap mAlphaA,
                                                                 const __grid_constant__ CUtensorMap mBetaA,
                                                                 const __grid_constant__ CUtensorMap mGammaA,
                                                                 const __grid_constant__ CUtensorMap mAlphaB,
                                                                 const __grid_constant__ CUtensorMap mBetaB,
                                                                 const __grid_constant__ CUtensorMap mDeltaB,
                                                                 GemmArgs g)
{
  using Acc = AccPair<S, TN>;
  constexpr int OV = Acc::OV;
  static_assert(TILE_M % TN == 0 && TN % 16 == 0, "tile shape");
  constexpr int EPI_T = 32 * EPIW;          // epilogue threads
  constexpr int COLS_W = TN / (EPIW / 4);   // columns per epilogue warp
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // 1024-byte aligned base
  unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const int NST = g.nstages;
  const unsigned A_SLICE = TILE_M * KB * 2;  // 8 KB
  const unsigned B_SLICE = TN * KB * 2;
  const unsigned STAGE = S * (A_SLICE + B_SLICE);
  unsigned long long* bars = (unsigned long long*)(smem + NST * STAGE);
  // bars: full[NST], empty[NST], acc_full[2], done[2], early[1]; then the tmem slot
  unsigned* tmem_slot = (unsigned*)(bars + 2 * NST + 5);
  __shared__ int s_err_;
  __shared__ int s_colexp[2][TN];  // indexed by tile parity: warps run at most one tile apart
  __shared__ int s_colph[2][TN];
  __shared__ int s_epi_err_;
  volatile int& s_err = s_err_;
  volatile int& s_epi_err = s_epi_err_;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const unsigned sbase = smem_u32(smem);
  const unsigned bar0 = smem_u32(bars);
  auto full_bar = [&](int s) { return bar0 + 8u * s; };
  auto empty_bar = [&](int s) { return bar0 + 8u * (NST + s); };
  auto acc_full = [&](int b) { return bar0 + 8u * (2 * NST + b); };
  auto acc_done = [&](int b) { return bar0 + 8u * (2 * NST + 2 + b); };  // epilogue finished the tile
  const unsigned acc_early = bar0 + 8u * (2 * NST + 4);                  // shared blocks read

  if (threadIdx.x == 0) {
    s_err = 0;
    s_epi_err = 0;
    for (int s = 0; s < NST; ++s) {
      mbar_init(full_bar(s), 1);
      mbar_init(empty_bar(s), 1);
    }
    mbar_init(acc_full(0), 1);
    mbar_init(acc_full(1), 1);
    mbar_init(acc_done(0), EPI_T);
    mbar_init(acc_done(1), EPI_T);
    mbar_init(acc_early, EPI_T);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(512)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const unsigned tmem = *tmem_slot;

  if (warp == 0) {
    // ------------------------------------------------ TMA producer
    if (lane == 0) {
      int it = 0;
      const int tend = g.cta_first[blockIdx.x + 1];
      for (int tix = g.cta_first[blockIdx.x]; tix < tend && !s_err; ++tix) {
        const SplitTile tl = g.tiles[tix];
        // the job's fields are copied to registers: the TMA and MMA asm
        // statements clobber memory, which would reload them from global
        const SplitJob* jp = g.jobs + tl.job;
        const long long exp_base = jp->exp_base;
        const int nkt = jp->nkt, nkb = jp->nkb;
        const bool useG = g.flags[2 * tl.job] == 1, useD = g.flags[2 * tl.job + 1] != 0;
        const CUtensorMap* mA2 = useG ? &mGammaA : &mBetaA;
        const CUtensorMap* mB2 = useD ? &mDeltaB : &mAlphaB;
        const int rowA = (int)(exp_base + tl.I * TILE_M);
        const int rowB = (int)(exp_base + tl.J * TN);
        for (int kb = 0; kb < nkt; ++kb, ++it) {
          int st = it % NST;
          unsigned ph = (unsigned)((it / NST) & 1);
          if (!mbar_wait(empty_bar(st), ph ^ 1u)) {
            set_status(g.status, 101);
            s_err = 1;
            break;
          }
          mbar_expect_tx(full_bar(st), STAGE);
          const bool second = kb >= nkb;
          const int k = (second ? kb - nkb : kb) * KB;
          const CUtensorMap* ma = second ? mA2 : &mAlphaA;
          const CUtensorMap* mb = second ? mB2 : &mBetaB;
          // digit plane s of a box lands s slices after the box start: the A
          // digit tiles at sA + s A_SLICE, the B digit tiles at sB + t B_SLICE
          const unsigned sA = sbase + st * STAGE;
          const unsigned sB = sA + S * A_SLICE;
          tma_load_3d(sA, ma, k, rowA, full_bar(st));
          tma_load_3d(sB, mb, k, rowB, full_bar(st));
        }
      }
    }
  } else if (warp == 1) {
    // ------------------------------------------------ MMA issuer
    if (lane == 0) {
      constexpr int MAXT = 256 / TN;  // B digit tiles per MMA (UMMA N <= 256)
      int it = 0, tc = 0;
      const int tend = g.cta_first[blockIdx.x + 1];
      for (int tix = g.cta_first[blockIdx.x]; tix < tend && !s_err; ++tix, ++tc) {
        const int job = g.tiles[tix].job;
        const int nkt = g.jobs[job].nkt, nkb = g.jobs[job].nkb;
        const unsigned neg2 = g.flags[2 * job] == 2 ? (1u << 13) : 0u;  // negate A in the second K half
        // the blocks of this tile are free: the tile before last is done, and
        // the shared blocks of the previous tile have been read (the
        // epilogue works through the tiles in order, so the second implies
        // the first)
        const bool waited = OV > 0 ? mbar_wait(acc_early, (unsigned)((tc & 1) ^ 1))
                                   : mbar_wait(acc_done(tc & 1), (unsigned)(((tc >> 1) & 1) ^ 1));
        if (!waited) {
          set_status(g.status, 102);
          s_err = 1;
          break;
        }
        tc_fence_after();
        const unsigned dbase = tmem + Acc::base(tc);
        bool ok = true;
        for (int kb = 0; kb < nkt; ++kb, ++it) {
          int st = it % NST;
          unsigned ph = (unsigned)((it / NST) & 1);
          if (!mbar_wait(full_bar(st), ph)) {
            set_status(g.status, 103);
            s_err = 1;
            ok = false;
            break;
          }
          tc_fence_after();
          // descriptors of this stage: a base each, every operand tile a
          // compile-time offset from it (the start-address field is addr >> 4,
          // and the stage never crosses its 14 bits); each group is written
          // (not accumulated) by the first K16 step of the tile, whose s = 0
          // products are the first ones issued into every group
          const unsigned sA = sbase + st * STAGE;
          const unsigned long long a0 = sdesc_sw64(sA), b0 = sdesc_sw64(sA + S * A_SLICE);
          const unsigned first = kb == 0 ? 0u : 1u;
          const unsigned neg = kb >= nkb ? neg2 : 0u;
          // The products (s, t) of one A digit s go to the weight groups s + t,
          // which are consecutive TN-column blocks of tensor memory, and the B
          // digit tiles t are consecutive TN-row blocks of shared memory with
          // the same 512-byte swizzle-atom stride: so the products of one s
          // over a run of t are one MMA with N = (run length) x TN, up to 256
#pragma unroll
          for (int sub = 0; sub < KB / 16; ++sub) {
#pragma unroll
            for (int s = 0; s < S; ++s) {
              const unsigned long long ad = a0 + (unsigned long long)((s * A_SLICE + sub * 32) >> 4);
#pragma unroll
              for (int t0 = 0; t0 < S - s; t0 += MAXT) {
                const int nt = (S - s - t0) < MAXT ? (S - s - t0) : MAXT;
                const unsigned long long bd = b0 + (unsigned long long)((t0 * B_SLICE + sub * 32) >> 4);
                tc_mma(dbase + (s + t0) * TN, ad, bd, idesc_bf16(TILE_M, nt * TN) | neg, (sub == 0 && s == 0) ? first : 1u);
              }
            }
          }
          tc_commit(empty_bar(st));
        }
        if (!ok) break;
        tc_commit(acc_full(tc & 1));
      }
    }
  } else {
    // ------------------------------------------------ epilogue (warps 2 .. 1+EPIW)
    const int q = warp & 3;                  // TMEM lane quarter of this warp
    const int cbeg = ((warp - 2) >> 2) * COLS_W;  // first column of this warp
    const int et = threadIdx.x - 64;         // 0 .. EPI_T-1
    int tc = 0;
    const int tend = g.cta_first[blockIdx.x + 1];
    for (int tix = g.cta_first[blockIdx.x]; tix < tend; ++tix, ++tc) {
      const SplitTile tl = g.tiles[tix];
      // the job's fields in registers (a reference would be re-read after
      // every store to the output, which the compiler cannot tell apart)
      const SplitJob* jp = g.jobs + tl.job;
      const int jm = jp->m, jn = jp->n, ldo = jp->ldo, nosym = jp->nosym, phase_off = jp->phase_off;
      const int jsign = jp->sign, jacc = jp->accumulate;
      const long long exp_base = jp->exp_base, out_off = jp->out_off;
      // the tile's row and column exponents and phases come from the
      // exponent pass (before this kernel), not from the MMAs: they are read
      // while the tile's products still run.  (s_colexp[tc & 1] was last read
      // for tile tc - 2, which every epilogue warp finished before the
      // barrier of tile tc - 1.)
      const int c = nosym ? 0 : job_c(g.jobmax, tl.job);
      const int* ph = phase_off >= 0 ? g.phase + phase_off : nullptr;
      // column exponents and phases of this tile (a plain job's columns are
      // B rows with their own exponents)
      if (et < TN) {
        const int j = tl.J * TN + et;
        const bool ok = j < jn;
        s_colexp[tc & 1][et] = !ok ? EXP_NONE
                               : nosym ? own_exp(g.rexpB[exp_base + j])
                                          : row_exp(g.rexpA[exp_base + j], g.rexpB[exp_base + j], c);
        s_colph[tc & 1][et] = (ph && ok) ? ph[j] : 1;
      }
      const int sign = jsign != 0 ? jsign : g.gsign;
      const int i = tl.I * TILE_M + q * 32 + lane;
      const bool rowok = i < jm;
      const int ai = !rowok   ? EXP_NONE
                     : nosym ? own_exp(g.rexpA[exp_base + i])
                                : row_exp(g.rexpA[exp_base + i], g.rexpB[exp_base + i], c);
      const int phi_i = (ph && rowok) ? ph[i] : 1;
      // the epilogue warps decide together (named barrier 1), so a timeout
      // never leaves one of them waiting at a barrier alone
      if (!mbar_wait(acc_full(tc & 1), (unsigned)((tc >> 1) & 1))) {
        set_status(g.status, 104);
        s_epi_err = 1;
      }
      asm volatile("bar.sync 1, %0;" ::"r"(EPI_T) : "memory");
      if (s_epi_err) {
        s_err = 1;
        break;
      }
      tc_fence_after();
      double* O = g.out + out_off;
      const int Xi = ai + c - g.beta * (S + 1);
      const bool accumulate = g.accum > 0 || (g.accum < 0 && jacc);
      const unsigned lane_base = tmem + ((unsigned)(q * 32) << 16) + Acc::base(tc);
      // exact merge of the weight groups: Horner in base 2^beta, per column,
      // in two parts.  The groups the next tile overwrites (e0 .. e0+OV-1)
      // are read first for all this warp's columns into P, then released;
      // per chunk of columns the other groups (l0 .. l0+S-OV-1) give the rest:
      //   odd tile  (e0 = 0, the leading groups):  I = P 2^(beta (S-OV)) + L
      //   even tile (e0 = S-OV, the trailing ones): I = L 2^(beta OV) + P
      const int e0 = Acc::early_lo(tc);
      const int l0 = (tc & 1) ? OV : 0;
      const long long mulP = (tc & 1) ? (1ll << (g.beta * (S - OV))) : 1ll;
      const long long mulL = (tc & 1) ? 1ll : (1ll << (g.beta * OV));
      long long P[COLS_W];
#pragma unroll
      for (int cc = 0; cc < COLS_W; ++cc) P[cc] = 0;
      if (OV > 0) {
#pragma unroll
        for (int c0 = 0; c0 < COLS_W; c0 += EPI_COLS) {
          unsigned r[OV > 0 ? OV : 1][EPI_COLS];
#pragma unroll
          for (int gi = 0; gi < OV; ++gi)
            tmem_ld8(lane_base + (unsigned)((e0 + gi) * TN + cbeg + c0), r[gi]);
          tmem_wait_ld();
#pragma unroll
          for (int gi = 0; gi < OV; ++gi)
#pragma unroll
            for (int cc = 0; cc < EPI_COLS; ++cc)
              P[c0 + cc] = P[c0 + cc] * (1ll << g.beta) + __float2int_rn(__uint_as_float(r[gi][cc]));
        }
        tc_fence_before();
        mbar_arrive(acc_early);
      }
#pragma unroll
      for (int c0 = 0; c0 < COLS_W; c0 += EPI_COLS) {
        unsigned r[S - OV][EPI_COLS];
#pragma unroll
        for (int gi = 0; gi < S - OV; ++gi) tmem_ld8(lane_base + (unsigned)((l0 + gi) * TN + cbeg + c0), r[gi]);
        tmem_wait_ld();
        // values of this chunk, then all old values (accumulate), then the
        // stores: the loads of one chunk are in flight together
        double v[EPI_COLS], mv[EPI_COLS], od[EPI_COLS], om[EPI_COLS];
        bool wd[EPI_COLS], wm[EPI_COLS];
#pragma unroll
        for (int cc = 0; cc < EPI_COLS; ++cc) {
          const int jc = cbeg + c0 + cc;  // column within the tile
          const int j = tl.J * TN + jc;
          wd[cc] = rowok && j < jn && !(tl.diag && i > j);
          wm[cc] = wd[cc] && i != j && !nosym && !g.nomirror;
          long long L = 0;
#pragma unroll
          for (int gi = 0; gi < S - OV; ++gi) L = L * (1ll << g.beta) + __float2int_rn(__uint_as_float(r[gi][cc]));
          const long long I64 = P[c0 + cc] * mulP + L * mulL;
          v[cc] = i64_ldexp(I64, Xi + s_colexp[tc & 1][jc]);
          mv[cc] = __longlong_as_double(__double_as_longlong(v[cc]) ^
                                        ((sign * phi_i * s_colph[tc & 1][jc]) < 0 ? (long long)0x8000000000000000ull
                                                                                   : 0ll));
          od[cc] = 0.0;
          om[cc] = 0.0;
        }
        if (accumulate) {
#pragma unroll
          for (int cc = 0; cc < EPI_COLS; ++cc) {
            const long long j = tl.J * TN + cbeg + c0 + cc;
            if (wd[cc]) od[cc] = __ldcg(O + j * ldo + i);
            if (wm[cc]) om[cc] = __ldcg(O + (long long)i * ldo + j);
          }
#pragma unroll
          for (int cc = 0; cc < EPI_COLS; ++cc) {
            const long long j = tl.J * TN + cbeg + c0 + cc;
            if (wd[cc]) O[j * ldo + i] = od[cc] + v[cc];
            if (wm[cc]) O[(long long)i * ldo + j] = om[cc] + mv[cc];
          }
        } else {
          // overwrite: no FP64 add (the FP64 pipe is the slow one on this part)
#pragma unroll
          for (int cc = 0; cc < EPI_COLS; ++cc) {
            const long long j = tl.J * TN + cbeg + c0 + cc;
            if (wd[cc]) O[j * ldo + i] = v[cc];
            if (wm[cc]) O[(long long)i * ldo + j] = mv[cc];
          }
        }
      }
      // every TMEM load of this tile has completed (tcgen05.wait::ld)
      tc_fence_before();
      mbar_arrive(acc_done(tc & 1));
    }
  }
  // every role has left its loop: all MMAs this CTA issued have been drained
  // by the epilogue (or the CTA gave up after a bounded wait)
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512) : "memory");
  }
}

// Self-test of the bounded wait: one thread waits on an mbarrier that nothing
// arrives on, through the same wait loop as the products above but with a
// bound of `limit` iterations; when it runs out the kernel sets the status
// word (code 105), stores the clock cycles it waited, and returns, so the
// context stays usable.
__global__ void k_wait_selftest(int* status, unsigned limit, long long* cycles)
{
  __shared__ __align__(8) unsigned long long bar;
  if (threadIdx.x != 0) return;
  const unsigned a = smem_u32(&bar);
  mbar_init(a, 1);
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  const long long c0 = clock64();
  if (!mbar_wait(a, 0, limit)) set_status(status, 105);
  *cycles = clock64() - c0;
}

}  // namespace

cudaError_t launch_wait_selftest(int* status, unsigned limit, long long* cycles, cudaStream_t st)
{
  k_wait_selftest<<<1, 32, 0, st>>>(status, limit, cycles);
  count_launch();
  return cudaGetLastError();
}

unsigned wait_limit() { return WAIT_LIMIT; }

// ------------------------------------------------------------------ host
typedef CUresult (*PFN_encodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                    const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                    CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static PFN_encodeTiled get_encode()
{
  static PFN_encodeTiled fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !p)
      throw std::runtime_error("cuTensorMapEncodeTiled unavailable");
    fn = (PFN_encodeTiled)p;
  }
  return fn;
}

// a slice array as (K element, plane row, digit plane); a box is KB elements
// x box_rows rows x all S planes
static void encode_map(CUtensorMap* m, void* base, long long plane_rows, int S, int K_stride, int box_rows)
{
  cuuint64_t dims[3] = {(cuuint64_t)K_stride, (cuuint64_t)plane_rows, (cuuint64_t)S};
  cuuint64_t strides[2] = {(cuuint64_t)K_stride * 2, (cuuint64_t)K_stride * 2 * (cuuint64_t)plane_rows};
  cuuint32_t box[3] = {(cuuint32_t)KB, (cuuint32_t)box_rows, (cuuint32_t)S};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = get_encode()(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, base, dims, strides, box, estr,
                            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw std::runtime_error("cuTensorMapEncodeTiled failed");
}

// Choose the digit width: largest beta whose leading weight groups (T <= 5)
// sum exactly in FP32 for a reduction of length 2K, then S for >= 36 bits.
static void choose_digits(int Kmax, int& beta, int& S)
{
  long long K2 = 2ll * std::max(1, Kmax);
  for (beta = 7; beta >= 3; --beta) {
    long long d1 = (1ll << beta) + 1, dl = 1ll << (beta - 1);
    bool ok = true;
    for (int T = 2; T <= 5; ++T) {
      long long b = 0;
      for (int s = 1; s < T; ++s) {
        int t = T - s;
        b += (s == 1 ? d1 : dl) * (t == 1 ? d1 : dl);
      }
      if (b * K2 > (1ll << 24)) ok = false;
    }
    if (ok) break;
  }
  S = (36 + beta - 1) / beta;
  if (S > MAX_S) S = MAX_S;
}

SplitOpts split_plan_opts(const SplitPlan* p)
{
  SplitOpts o;
  o.tn = p->tn;
  o.nacc = p->nacc;
  o.stages = p->nstages;
  o.digits = p->S;
  o.sched = p->sched;
  return o;
}

SplitPlan* split_plan_create(const Space& s, const std::vector<GemmJobDev>& jobs_in, int family,
                             const SplitOpts& opts)
{
  (void)s;
  SplitPlan* p = new SplitPlan();
  p->family = family;
  // defaults: the ladder products have long K (MMA-bound tiles): 64-column
  // tiles; the Pandya-space products have short K (epilogue-bound tiles):
  // 32-column tiles; eight epilogue warps.  (The second number of a tile
  // shape, 1 or 2, is its name in the tuning tables: the accumulator ring
  // sizes itself from the tile width.)
  p->tn = family == 0 ? 64 : 32;
  p->nacc = family == 0 ? 1 : 2;
  if (opts.tn == 64 && (opts.nacc == 0 || opts.nacc == 1)) {
    p->tn = 64;
    p->nacc = 1;
  } else if (opts.tn == 32 && (opts.nacc == 0 || opts.nacc == 2)) {
    p->tn = 32;
    p->nacc = 2;
  } else if (opts.tn != 0 || opts.nacc != 0) {
    delete p;
    throw std::invalid_argument("split plan: tile shape must be 64 x 1 or 32 x 2");
  }
  if (opts.sched < 0 || opts.sched > 1 || opts.stages < 0) {
    delete p;
    throw std::invalid_argument("split plan: bad schedule or stage count");
  }
  p->stages_opt = opts.stages;
  p->sched = opts.sched;
  p->epiw = 8;
  int Kmax = 1;
  for (const GemmJobDev& j : jobs_in) Kmax = std::max(Kmax, j.K);
  choose_digits(Kmax, p->beta, p->S);
  // a requested digit count keeps the digit width (set by exactness) and
  // changes the precision: beta * S bits per operand row
  if (opts.digits != 0) {
    if (opts.digits < 5 || opts.digits > MAX_S) {
      delete p;
      throw std::invalid_argument("split plan: digits must be 5, 6 or 7");
    }
    if (p->beta * opts.digits > 42) {
      delete p;
      throw std::invalid_argument("split plan: digits x digit width above 42 bits");
    }
    p->S = opts.digits;
  }
  long long erow = 0;
  int kstride = KB;
  std::vector<SplitTile> tiles;
  std::vector<int> order(jobs_in.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return jobs_in[a].m > jobs_in[b].m; });
  for (const GemmJobDev& j : jobs_in) {
    SplitJob sj{};
    sj.a_off = j.a_off;
    sj.b_off = j.b_off;
    sj.out_off = j.out_off;
    sj.m = j.m;
    sj.K = j.K;
    sj.lda = j.lda;
    sj.ldb = j.ldb;
    sj.ldo = j.ldo;
    sj.kidx_off = j.kidx_off;
    sj.w_off = j.w_off;
    sj.phase_off = j.phase_off;
    sj.bsel = j.bsel;
    sj.sign = j.sign;
    sj.accumulate = j.accumulate;
    sj.bscale = j.bscale;
    sj.nosym = j.nosym ? 1 : 0;
    sj.n = j.nosym ? j.n : j.m;
    sj.m_pad = (std::max(sj.m, sj.n) + TILE_M - 1) / TILE_M * TILE_M;
    sj.K_pad = std::max(KB, (j.K + KB - 1) / KB * KB);
    sj.nkb = sj.K_pad / KB;
    sj.nkt = sj.nosym ? sj.nkb : 2 * sj.nkb;
    if (sj.nosym && (sj.sign != 0 || sj.phase_off >= 0))
      throw std::invalid_argument("a plain split job takes no sign or phases (fold a sign into bscale)");
    sj.exp_base = erow;
    erow += sj.m_pad;
    kstride = std::max(kstride, sj.K_pad);
    p->jobs.push_back(sj);
  }
  for (int jix : order) {
    const SplitJob& sj = p->jobs[jix];
    if (sj.m == 0 || sj.n == 0 || sj.K == 0) continue;
    const int per = TILE_M / p->tn;  // column tiles per 128-row block
    const int nJ = (sj.n + p->tn - 1) / p->tn;
    if (sj.nosym) {
      const int nI = (sj.m + TILE_M - 1) / TILE_M;
      for (int I = 0; I < nI; ++I)
        for (int J = 0; J < nJ; ++J) tiles.push_back({jix, I, J, 0});
    } else {
      const int nI = sj.m_pad / TILE_M;
      for (int I = 0; I < nI; ++I)
        for (int J = per * I; J < nJ; ++J) tiles.push_back({jix, I, J, J < per * (I + 1) ? 1 : 0});
    }
  }
  if (erow > (1ll << 31) - TILE_M) throw std::runtime_error("split digit planes exceed 2^31 rows");
  // every nonempty job pads to TILE_M rows, so a plane has at least TILE_M
  erow = std::max(erow, (long long)TILE_M);
  p->K_stride = kstride;
  p->total_exp_rows = erow;
  p->njobs = (int)p->jobs.size();
  p->ntiles = (int)tiles.size();
  auto dm = [](size_t bytes) {
    void* q = nullptr;
    if (cudaMalloc(&q, std::max<size_t>(bytes, 16)) != cudaSuccess) throw std::runtime_error("cudaMalloc");
    return q;
  };
  // persistent grid: one CTA per SM; each CTA works through its own run of
  // tiles, dealt round-robin in size order (sched 0) or by longest-first
  // greedy assignment of the tiles' K-block counts (sched 1)
  {
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    p->grid = std::max(1, std::min(nsm, p->ntiles));
  }
  std::vector<int> cta_first(p->grid + 1, 0);
  {
    const int G = p->grid;
    std::vector<int> owner(tiles.size());
    if (p->sched == 0) {
      for (size_t t = 0; t < tiles.size(); ++t) owner[t] = (int)(t % G);
    } else {
      std::vector<int> ord(tiles.size());
      for (size_t t = 0; t < ord.size(); ++t) ord[t] = (int)t;
      auto cost = [&](int t) { return (long long)p->jobs[tiles[t].job].nkt + 4; };
      std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return cost(a) > cost(b); });
      std::vector<std::pair<long long, int>> heap;  // (load, cta), min-heap
      for (int b = 0; b < G; ++b) heap.push_back({0, b});
      auto gt = [](const std::pair<long long, int>& x, const std::pair<long long, int>& y) { return x > y; };
      std::make_heap(heap.begin(), heap.end(), gt);
      for (int t : ord) {
        std::pop_heap(heap.begin(), heap.end(), gt);
        heap.back().first += cost(t);
        owner[t] = heap.back().second;
        std::push_heap(heap.begin(), heap.end(), gt);
      }
    }
    // tiles of one CTA contiguous, in their original (size) order
    std::vector<SplitTile> sorted;
    sorted.reserve(tiles.size());
    std::vector<std::vector<int>> lists(G);
    for (size_t t = 0; t < tiles.size(); ++t) lists[owner[t]].push_back((int)t);
    for (int b = 0; b < G; ++b) {
      cta_first[b] = (int)sorted.size();
      for (int t : lists[b]) sorted.push_back(tiles[t]);
    }
    cta_first[G] = (int)sorted.size();
    tiles.swap(sorted);
  }
  try {
    p->d_jobs = (SplitJob*)dm(sizeof(SplitJob) * std::max(1, p->njobs));
    p->d_tiles = (SplitTile*)dm(sizeof(SplitTile) * std::max(1, p->ntiles));
    p->d_cta = (int*)dm(sizeof(int) * cta_first.size());
    cudaMemcpy(p->d_jobs, p->jobs.data(), sizeof(SplitJob) * p->njobs, cudaMemcpyHostToDevice);
    cudaMemcpy(p->d_tiles, tiles.data(), sizeof(SplitTile) * p->ntiles, cudaMemcpyHostToDevice);
    cudaMemcpy(p->d_cta, cta_first.data(), sizeof(int) * cta_first.size(), cudaMemcpyHostToDevice);
    size_t abytes = (size_t)p->S * erow * kstride * 2;
    // gamma / delta (the second half of a doubled K) only for symmetrised jobs
    bool any_sym = false, any_plain = false;
    for (const SplitJob& sj : p->jobs) {
      any_sym = any_sym || !sj.nosym;
      any_plain = any_plain || sj.nosym;
    }
    if (any_sym && any_plain) throw std::invalid_argument("a split plan holds plain or symmetrised jobs, not both");
    p->plain = any_plain;
    for (int a = 0; a < (any_sym ? 4 : 2); ++a) {
      p->arr[a] = (__nv_bfloat16*)dm(abytes);
      cudaMemset(p->arr[a], 0, abytes);
    }
    if (!any_sym) {
      p->arr[2] = p->arr[1];
      p->arr[3] = p->arr[0];
      p->shared_gd = true;
    }
    p->d_rexpA = (int*)dm(sizeof(int) * std::max(1ll, erow));
    p->d_rexpB = (int*)dm(sizeof(int) * std::max(1ll, erow));
    p->d_jobmax = (int*)dm(sizeof(int) * 2 * std::max(1, p->njobs));
    p->d_flags = (int*)dm(sizeof(int) * 4 * std::max(1, p->njobs));
    std::vector<int> flags(4 * p->njobs, 0);
    for (int gs = 0; gs < 2; ++gs)
      for (int j = 0; j < p->njobs; ++j) {
        const SplitJob& sj = p->jobs[j];
        int sign = sj.sign != 0 ? sj.sign : (gs == 0 ? 1 : -1);
        // plain jobs have no second K half: gamma / delta stay unwritten.
        // Without row phases gamma is beta or -beta: the MMA reads beta and,
        // for -beta, negates its A operand (instruction descriptor bit 13)
        flags[2 * p->njobs * gs + 2 * j] = sj.nosym ? 0 : sj.phase_off >= 0 ? 1 : sign != 1 ? 2 : 0;
        flags[2 * p->njobs * gs + 2 * j + 1] = !sj.nosym && sj.phase_off >= 0 ? 1 : 0;
      }
    cudaMemcpy(p->d_flags, flags.data(), sizeof(int) * flags.size(), cudaMemcpyHostToDevice);
    // slicing blocks: only the (row group, column chunk) blocks each job has;
    // the digit pass visits jobs in the reverse order of the exponent pass, so
    // it starts on the operands the exponent pass read last (still in L2)
    std::vector<int4> rb, db;
    for (int j = 0; j < p->njobs; ++j) {
      const SplitJob& sj = p->jobs[j];
      if (sj.m == 0) continue;
      for (int y = 0; y < sj.m_pad / 32; ++y)
        for (int x = 0; x < (std::max(sj.K, 1) + 255) / 256; ++x) rb.push_back(make_int4(j, y, x, 0));
    }
    for (int j = p->njobs - 1; j >= 0; --j) {
      const SplitJob& sj = p->jobs[j];
      if (sj.m == 0) continue;
      for (int y = 0; y < sj.m_pad / 32; ++y)
        for (int x = 0; x < sj.K_pad / KB; ++x) db.push_back(make_int4(j, y, x, 0));
    }
    p->n_rblk = (int)rb.size();
    p->n_dblk = (int)db.size();
    p->d_rblk = (int4*)dm(sizeof(int4) * std::max<size_t>(1, rb.size()));
    p->d_dblk = (int4*)dm(sizeof(int4) * std::max<size_t>(1, db.size()));
    cudaMemcpy(p->d_rblk, rb.data(), sizeof(int4) * rb.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(p->d_dblk, db.data(), sizeof(int4) * db.size(), cudaMemcpyHostToDevice);
    // A-operand role of alpha, beta, gamma (TILE_M-row boxes); B-operand
    // role of alpha, beta, delta (tn-row boxes)
    for (int a = 0; a < 3; ++a) encode_map(&p->maps[a], p->arr[a], erow, p->S, kstride, TILE_M);
    const int brole[3] = {0, 1, 3};
    for (int a = 0; a < 3; ++a) encode_map(&p->maps[3 + a], p->arr[brole[a]], erow, p->S, kstride, p->tn);
  } catch (...) {
    split_plan_destroy(p);
    throw;
  }
  int dev = 0, maxsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  size_t stage = (size_t)p->S * (TILE_M + p->tn) * KB * 2;
  p->nstages = (int)std::min<size_t>(6, ((size_t)maxsm - 3072) / stage);
  if (p->stages_opt > 0) p->nstages = std::min(p->nstages, p->stages_opt);
  if (p->nstages < 2) {
    split_plan_destroy(p);
    throw std::runtime_error("not enough shared memory for the split GEMM pipeline (or fewer than 2 stages asked)");
  }
  p->smem = 1024 + p->nstages * stage + (2 * p->nstages + 5) * 8 + 16;
  return p;
}

void split_plan_destroy(SplitPlan* p)
{
  if (!p) return;
  cudaFree(p->d_jobs);
  cudaFree(p->d_tiles);
  cudaFree(p->d_cta);
  for (int a = 0; a < (p->shared_gd ? 2 : 4); ++a) cudaFree(p->arr[a]);
  cudaFree(p->d_rexpA);
  cudaFree(p->d_rexpB);
  cudaFree(p->d_jobmax);
  cudaFree(p->d_flags);
  cudaFree(p->d_rblk);
  cudaFree(p->d_dblk);
  delete p;
}

// per-job use of the gamma / delta arrays for a launch sign (precomputed for
// both signs at plan creation): [0, 2 njobs) for sign +1, then for sign -1
static const int* flags_for(const SplitPlan* p, int gsign) { return p->d_flags + (gsign == 1 ? 0 : 2 * p->njobs); }

template <int S>
static cudaError_t launch_s(SplitPlan* p, const double* A, const double* B0, const double* B1, double* O,
                            const int* kidx, const double* kw, const int* phase, int* status, int gsign,
                            double gbscale, cudaStream_t st)
{
  cudaError_t e;
  {
    ProfScope ps(p->family == 0 ? "split_slice_ladder" : "split_slice_zbar", st);
    e = cudaMemsetAsync(p->d_jobmax, 0, sizeof(int) * 2 * p->njobs, st);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(p->d_rexpA, 0, sizeof(int) * std::max(1ll, p->total_exp_rows), st);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(p->d_rexpB, 0, sizeof(int) * std::max(1ll, p->total_exp_rows), st);
    if (e != cudaSuccess) return e;
    if (p->n_rblk > 0) {
      auto kr = p->plain ? k_split_rowexp<true> : k_split_rowexp<false>;
      kr<<<p->n_rblk, 256, 0, st>>>(p->d_jobs, p->d_rblk, A, B0, B1, kidx, kw, gbscale, p->d_rexpA, p->d_rexpB,
                                    p->d_jobmax);
      count_launch();
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    if (p->n_dblk > 0) {
      auto kd = p->plain ? k_split_digits<S, true> : k_split_digits<S, false>;
      kd<<<p->n_dblk, 256, 0, st>>>(p->d_jobs, p->d_dblk, A, B0, B1, kidx, kw, phase, gbscale, gsign,
                                                    p->d_rexpA, p->d_rexpB, p->d_jobmax, flags_for(p, gsign),
                                                    p->beta, p->K_stride, p->total_exp_rows, p->arr[0],
                                                    p->arr[1], p->arr[2], p->arr[3]);
      count_launch();
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
  }
  {
    ProfScope ps(p->family == 0 ? "split_gemm_ladder" : "split_gemm_zbar", st);
    GemmArgs ga;
    ga.jobs = p->d_jobs;
    ga.tiles = p->d_tiles;
    ga.cta_first = p->d_cta;
    ga.ntiles = p->ntiles;
    ga.rexpA = p->d_rexpA;
    ga.rexpB = p->d_rexpB;
    ga.jobmax = p->d_jobmax;
    ga.flags = flags_for(p, gsign);
    ga.phase = phase;
    ga.out = O;
    ga.status = status;
    ga.S = S;
    ga.beta = p->beta;
    ga.nstages = p->nstages;
    ga.gsign = gsign;
    ga.accum = p->accum_override;
    ga.nomirror = p->mirror ? 0 : 1;
    if (p->tn == 64) {
      auto kern = k_split_gemm<S, 64, 8>;
      e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p->smem);
      if (e != cudaSuccess) return e;
      kern<<<p->grid, 64 + 32 * 8, p->smem, st>>>(p->maps[0], p->maps[1], p->maps[2], p->maps[3], p->maps[4],
                                                   p->maps[5], ga);
    } else {
      auto kern = k_split_gemm<S, 32, 8>;
      e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p->smem);
      if (e != cudaSuccess) return e;
      kern<<<p->grid, 64 + 32 * 8, p->smem, st>>>(p->maps[0], p->maps[1], p->maps[2], p->maps[3], p->maps[4],
                                                   p->maps[5], ga);
    }
    count_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

void split_plan_set_accumulate(SplitPlan* p, int mode) { p->accum_override = mode; }
void split_plan_set_mirror(SplitPlan* p, int mirror) { p->mirror = mirror ? 1 : 0; }

cudaError_t launch_symgemm_split(SplitPlan* p, const double* A, const double* B0, const double* B1, double* O,
                                 const int* kidx, const double* kw, const int* phase, int* dev_status, int gsign,
                                 double gbscale, cudaStream_t st)
{
  if (p->ntiles == 0) return cudaSuccess;
  switch (p->S) {
    case 5: return launch_s<5>(p, A, B0, B1, O, kidx, kw, phase, dev_status, gsign, gbscale, st);
    case 6: return launch_s<6>(p, A, B0, B1, O, kidx, kw, phase, dev_status, gsign, gbscale, st);
    case 7: return launch_s<7>(p, A, B0, B1, O, kidx, kw, phase, dev_status, gsign, gbscale, st);
    default: return cudaErrorNotSupported;
  }
}

}  // namespace imsrg
