// Kernel launchers of the GB300 IMSRG(2) commutator (host-callable).
#pragma once

#include <cuda_runtime.h>

#include "space.hpp"

namespace imsrg {

// device copy of a SymGemmJob (see space.hpp)
struct GemmJobDev {
  long long a_off, b_off, out_off;
  int m, K, lda, ldb, ldo;
  int kidx_off, w_off, phase_off;
  int bsel;        // 0: B0, 1: B1
  int sign;        // +-1, or 0: the launch's sign
  int accumulate;  // 1: Out += ..., 0: Out = ...
  double bscale;   // times the launch's scale
  // plain product (split form only): Out (+)= A B^T with A m x K and B n x K,
  // no symmetrisation, no phases, every tile; 0: the symmetrised m x m form
  int nosym;
  int n;
};

// kernels_terms.cu
//
// Launchers marked (grouped) also run nz pairs of the same structure at once
// (batches): pair z's operands sit at byte offsets zo[z * kZRoles + role] from
// the pointers passed (pair 0's); zo = nullptr, nz = 1 is one pair.
enum ZRole { ZR_X, ZR_Y, ZR_Z, ZR_XF, ZR_YF, ZR_W2, ZR_XB, ZR_YT, ZR_YFL, ZR_ZB, kZRoles };
// (grouped)
cudaError_t launch_comm111_110(const Space& s, const double* X, const double* Y, double* Z, bool do111, bool do110,
                               cudaStream_t st, const long long* zo = nullptr, int nz = 1);
// (grouped)
cudaError_t launch_comm220(const Space& s, const double* X, const double* Y, double* Z, int hX, cudaStream_t st,
                           const long long* zo = nullptr, int nz = 1);
// (grouped)
cudaError_t launch_comm121(const Space& s, const int* dev_holes, const double* X, const double* Y, double* Z, int hZ,
                           cudaStream_t st, const long long* zo = nullptr, int nz = 1);
// (grouped with Mz)
cudaError_t launch_comm221_1b(const Space& s, const double* X, const double* Y, double* Z, int hX, int hZ,
                              const double* Mz, cudaStream_t st, const long long* zo = nullptr, int nz = 1);
// (grouped)
cudaError_t launch_comm122(const Space& s, const double* X, const double* Y, double* Z, double* W2, int hZ,
                           const int* sym_tiles, int nsym_tiles, cudaStream_t st, const long long* zo = nullptr,
                           int nz = 1, bool sym = true);
// loads launch_comm122's kernels on the current device (they are otherwise
// loaded at their first launch under lazy module loading)
cudaError_t load_comm122_kernels();
// (hi, lo) float-pair copy of an arena (integer instructions); (grouped, with
// the roles of A and Af)
cudaError_t launch_to_ff(const Space& s, const double* A, float2* Af, cudaStream_t st, const long long* zo = nullptr,
                         int nz = 1, int rsrc = ZR_X, int rdst = ZR_XF);
// split-form comm122ss from the (hi, lo) copies Xf, Yf of X and Y
// (grouped)
// sym = false: W2 only (the Z update is folded into the inverse Pandya kernel)
cudaError_t launch_comm122_df(const Space& s, const double* X, const double* Y, double* Z, const float2* Xf,
                              const float2* Yf, float2* W2, int hZ, const int* sym_tiles, int nsym_tiles,
                              cudaStream_t st, const long long* zo = nullptr, int nz = 1, bool sym = true);
// the same without the W2 round trip: tile pairs (ch, a, b), a <= b, each
// forming both W2 tiles in shared memory and updating Z(a, b) and Z(b, a)
// (grouped)
cudaError_t launch_comm122_fused_df(const Space& s, const double* X, const double* Y, double* Z, const float2* Xf,
                                    const float2* Yf, int hZ, const int* tiles, int ntiles, cudaStream_t st,
                                    const long long* zo = nullptr, int nz = 1);
// (grouped)
cudaError_t launch_pandya_fwd(const Space& s, const double* X, const double* Y, int hY, double* Xb, double* Yt,
                              double* Yf, bool df, cudaStream_t st, const long long* zo = nullptr, int nz = 1);
cudaError_t launch_pandya_inv(const Space& s, const double* Zb, double* Z, int hZ, const int* tiles, int ntiles,
                              cudaStream_t st);
// split form: blocks of orbit quadruples (Space::invq_tasks), double-float sums
// (grouped)
cudaError_t launch_pandya_inv_ff(const Space& s, const double* Zb, double* Z, int hZ, const int* tasks, int ntasks,
                                 const int* clist, const int* coff, const unsigned char* csort, int smem,
                                 cudaStream_t st, const long long* zo = nullptr, int nz = 1);
// shared-memory budget of one quadruple block (dynamic part)
constexpr int kInvqBudget = 36864;

// kernels_invd.cu: the inverse Pandya transform from per-space descriptors
// (both forms; FP64 or double-float J' sums)
struct InvdPlan {
  std::vector<int4> blocks;  // per block: first staged index, staged count, first result, result count
  std::vector<int2> wblk;    // per block: first weight row, row count
  std::vector<int2> wrow;    // per 6j weight row: first sixj_wval / sixj_wf index, offset | length << 20
  std::vector<int> sidx;     // Zbar element (and sign bits) of every staged value, in address order
  std::vector<unsigned short> sslot;  // its slot in the block's shared memory
  std::vector<int4> dA;      // per result: staged weight rows of both sums, Z element, mirror element (-1: none)
  std::vector<int2> dB;      // per result: staged offsets, counts and combination bits
  int stage_max = 0;         // most staged values + weights in one block (shared-memory words)
};
struct InvdDev {
  const int4* blocks = nullptr;
  const int2* wblk = nullptr;
  const int2* wrow = nullptr;
  const int* sidx = nullptr;
  const unsigned short* sslot = nullptr;
  const int4* dA = nullptr;
  const int2* dB = nullptr;
  int nblocks = 0, stage_max = 0;
  bool staged_weights = false;  // the 6j weight rows are staged per block (else read from the table)
  int ilp = 1;                  // results each thread keeps in flight (1, 2 or 4)
  bool covers_all = false;      // one result per upper-triangle Z element (comm122ss's W2 can be folded in)
};
// blocks of at most stage_max staged values (and, staging weights, as many
// weights) and res_max results
void build_invd(const Space& s, InvdPlan& out, int stage_max, int res_max, bool stage_weights);
// (grouped)
// W2 / w2mode: comm122ss's W2 folded into the same update (Z -= W2 + hZ W2^T;
// 1: (hi, lo) float pairs, 2: FP64), only when d.covers_all and not grouped
cudaError_t launch_pandya_inv_desc(const Space& s, const InvdDev& d, bool df, const double* Zb, double* Z, int hZ,
                                   cudaStream_t st, const long long* zo = nullptr, int nz = 1,
                                   const void* W2 = nullptr, int w2mode = 0);
// single-operator Pandya transform into the Xbar panel layout (xb_off)
cudaError_t launch_pandya_single(const Space& s, const double* Z, int herm, int transpose, double* out,
                                 cudaStream_t st);
// Generator::Update for a single-reference space (white / atan / wegner /
// imaginary-time functions, Epstein-Nesbet or Moller-Plesset denominators):
// Eta is overwritten; mono is norb^2 doubles of scratch
enum { GEN_WHITE = 0, GEN_ATAN = 1, GEN_WEGNER = 2, GEN_IMAGINARY_TIME = 3 };
// qtransfer-atan_n: type GEN_QTRANSFER_BASE + n (qtransfer-atan is n = 1)
constexpr int GEN_QTRANSFER_BASE = 100;
enum { DENOM_EPSTEIN_NESBET = 0, DENOM_MOLLER_PLESSET = 1 };
constexpr int kDeltaAll = -12345;  // denominator_delta_index that adds the delta everywhere
struct GenParams {
  int type = GEN_WHITE, partitioning = DENOM_EPSTEIN_NESBET, delta_index = -1;
  double cutoff = 1e-6, delta = 0.0;
};
cudaError_t launch_generator(const Space& s, const double* H, double* Eta, double* mono, const GenParams& p,
                             cudaStream_t st);
cudaError_t launch_axpy(double* y, const double* x, double a, long long n, cudaStream_t st);
cudaError_t launch_scale(double* y, double a, long long n, cudaStream_t st);
// y += a x and the norm pieces of x (as launch_norm: partial[0..nchunks) the
// two-body chunks, partial[nchunks] the one-body part); x must have zero padding
cudaError_t launch_axpy_norm(const Space& s, double* y, const double* x, double a, const long long* chunk_off,
                             const int* chunk_len, const double* chunk_w, int nchunks, double* partial,
                             cudaStream_t st);
cudaError_t launch_norm(const Space& s, const double* A, const long long* chunk_off, const int* chunk_len,
                        const double* chunk_w, int nchunks, double* partial, cudaStream_t st);

// kernels_tensor.cu: the scalar-tensor commutator [X, Y] (X scalar, Y a
// reduced tensor of layout t); each adds its term into Z (layout t)
struct TensorLayout;
cudaError_t launch_tensor_111(const Space& s, const double* X, const double* Y, double* Z, cudaStream_t st);
cudaError_t launch_tensor_121(const Space& s, const TensorLayout& t, const int* dev_holes, const double* X,
                              const double* Y, int hY, double* Z, int hZ, cudaStream_t st);
// YT: scratch of layout t (Y with its blocks transposed, written here)
cudaError_t launch_tensor_122(const Space& s, const TensorLayout& t, const double* X, const double* Y, int hX,
                              double* YT, double* Z, cudaStream_t st);
// XW, WX: scratch of the space's arena length; D (= Mpp - Mhh), Mhh: scratch
// arenas of layout t
cudaError_t launch_tensor_222_221(const Space& s, const TensorLayout& t, const double* X, const double* Y,
                                  double* XW, double* WX, double* D, double* Mhh, double* Z, int hZ, cudaStream_t st);
// Xbar: the transposed single-operator Pandya transform of X (xb layout);
// Ybar, Zbar: scratch of t's yb_total and zb_total doubles
cudaError_t launch_tensor_ph(const Space& s, const TensorLayout& t, const double* Xbar, const double* Y, int hX,
                             int hY, double* Ybar, double* Zbar, double* Z, int hZ, cudaStream_t st);
// Operator::Norm of a tensor of layout t: partial[0 .. nrm2_off.size()] are
// the two-body chunks' weighted sums of squares, then the one-body one
cudaError_t launch_tensor_norm(const TensorLayout& t, const double* A, double* partial, cudaStream_t st);
// split form: the operands the split products read (Y with its blocks
// transposed, the tensor Pandya panels transposed and half-swapped, X bar
// half-swapped); the ladder's remainder (Mhh, Z2 += D, the one-body part) once
// D = Mpp - Mhh is in place; the inverse tensor Pandya transform of Zbar
cudaError_t launch_tensor_split_operands(const Space& s, const TensorLayout& t, const double* Y, int hY,
                                         const double* Xbar, double* YT, double* YbT, double* YbTF, double* XbF,
                                         cudaStream_t st);
cudaError_t launch_tensor_222_221_split(const Space& s, const TensorLayout& t, const double* X, const double* Y,
                                        double* D, double* Mhh, double* Z, int hZ, cudaStream_t st);
cudaError_t launch_tensor_inverse_pandya(const Space& s, const TensorLayout& t, const double* Zbar, double* Z, int hZ,
                                         cudaStream_t st);

// kernels_gemm.cu
int symgemm_fp64_tile();
cudaError_t launch_symgemm_fp64(const GemmJobDev* jobs, const int* pairs, int npairs, const double* A,
                                const double* B0, const double* B1, double* O, const int* kidx, const double* kw,
                                const int* phase, int gsign, double gbscale, cudaStream_t st);

// kernels_split.cu (Ozaki-style sliced BF16 products on tcgen05)
struct SplitPlan;
// Tile shape and schedule of a plan: tn x nacc in {64 x 1, 32 x 2} (tile
// columns, TMEM accumulator sets; 0 = the family's default), pipeline stages
// (0 = as many as shared memory holds), schedule 0 = tiles dealt round-robin
// to the persistent CTAs in size order, 1 = longest-first greedy (LPT) lists
// per CTA on the tiles' K-block counts.
struct SplitOpts {
  int tn = 0, nacc = 0, stages = 0, sched = 0;
  int digits = 0;  // digits per operand (5..7; 0: enough for 36 bits at the width exactness allows)
};
SplitPlan* split_plan_create(const Space& s, const std::vector<GemmJobDev>& jobs, int family,
                             const SplitOpts& opts = SplitOpts());
// the options a plan was built with (defaults resolved)
SplitOpts split_plan_opts(const SplitPlan* p);
void split_plan_destroy(SplitPlan* p);
// -1: each job's own accumulate flag; 0: overwrite the output; 1: accumulate
void split_plan_set_accumulate(SplitPlan* p, int mode);
// 0: symmetrised jobs store only their upper triangle (for a reader of the
// upper triangle alone, e.g. the descriptor inverse Pandya kernel); 1: both
void split_plan_set_mirror(SplitPlan* p, int mirror);
// one bounded mbarrier wait of `limit` iterations that runs out (no arrival):
// status = 105, *cycles = the SM clock cycles it waited (device pointer)
cudaError_t launch_wait_selftest(int* status, unsigned limit, long long* cycles, cudaStream_t st);
// the iteration bound of every wait in the split products
unsigned wait_limit();
cudaError_t launch_symgemm_split(SplitPlan* p, const double* A, const double* B0, const double* B1, double* O,
                                 const int* kidx, const double* kw, const int* phase, int* dev_status, int gsign,
                                 double gbscale, cudaStream_t st);

}  // namespace imsrg
