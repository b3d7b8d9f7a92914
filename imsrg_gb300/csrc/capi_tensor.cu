// extern "C" boundary, scalar-tensor commutator (include/imsrg_gb300.h):
// Commutator::CommutatorScalarTensor (src/Commutator.cc:432-500) and its
// IMSRG(2) terms on device operators.  X is a scalar operator, Y and Z are
// reduced tensors of the same rank (imsrg_op_create_tensor).  The ladder and
// Z bar products run in FP64 on the CUDA cores, or in the split form on the
// tensor cores (plain rectangular split products, kernels_split.cu).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <exception>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/imsrg_gb300.h"
#include "capi_internal.hpp"
#include "kernels.cuh"
#include "prof.hpp"

using namespace imsrg;

namespace {

int terr(int code, const std::string& msg) { return set_error(code, msg.c_str()); }

#define T_CUDA(expr)                                                                    \
  do {                                                                                  \
    cudaError_t _e = (expr);                                                            \
    if (_e != cudaSuccess) return terr(IMSRG_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e)); \
  } while (0)

int check_st(const imsrg_op* X, const imsrg_op* Y, const imsrg_op* Z)
{
  if (!X || !Y || !Z) return terr(IMSRG_ERR_ARG, "null operator");
  if (X->sp != Y->sp || X->sp != Z->sp) return terr(IMSRG_ERR_ARG, "operators belong to different model spaces");
  if (X->tl) return terr(IMSRG_ERR_UNSUPPORTED, "X must be a scalar operator");
  if (!Y->tl || Z->tl != Y->tl) return terr(IMSRG_ERR_ARG, "Y and Z must be tensor operators of the same rank");
  if (Z == Y) return terr(IMSRG_ERR_ARG, "Z must not alias Y");
  if ((X->herm != 1 && X->herm != -1) || (Y->herm != 1 && Y->herm != -1) || (Z->herm != 1 && Z->herm != -1))
    return terr(IMSRG_ERR_UNSUPPORTED, "operators must be hermitian or anti-hermitian");
  return IMSRG_OK;
}

int alloc(TensorLayout* tl, double*& p, long long n)
{
  if (p) return IMSRG_OK;
  void* q = nullptr;
  if (cudaMalloc(&q, (size_t)std::max(1LL, n) * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    return terr(IMSRG_ERR_NOMEM, "scalar-tensor scratch allocation failed");
  }
  tl->dev_allocs.push_back(q);
  p = (double*)q;
  return IMSRG_OK;
}

// scratch of one tensor layout (freed with the layout, i.e. with the space)
int scratch(imsrg_space* sp, TensorLayout* tl)
{
  std::lock_guard<std::mutex> g(sp->mu);
  int rc;
  if ((rc = alloc(tl, tl->d_mpp, tl->total)) || (rc = alloc(tl, tl->d_mhh, tl->total)) ||
      (rc = alloc(tl, tl->d_xbar, sp->s->xb_total)) || (rc = alloc(tl, tl->d_ybar, tl->yb_total)) ||
      (rc = alloc(tl, tl->d_zbar, tl->zb_total)) || (rc = alloc(tl, tl->d_xw, sp->s->arena)) ||
      (rc = alloc(tl, tl->d_wx, sp->s->arena)) || (rc = alloc(tl, tl->d_yt, tl->total)))
    return rc;
  return IMSRG_OK;
}

// ---------------------------------------------------------- split form
// plain split products of the ladder: term 1, D = Xb w Yc (A = X of the bra
// channel gathered by its ladder list, B = Y's block transposed), overwrite;
// term 2, D -= Yc w Xk (A = Y's block gathered by the ket channel's list,
// B = Xk, taken as hX Xk^T: the launch scale is hX), accumulate
std::vector<GemmJobDev> ladder_jobs(const Space& s, const TensorLayout& t, int term)
{
  std::vector<GemmJobDev> v;
  for (size_t b = 0; b < t.bra.size(); ++b) {
    const int chb = t.bra[b], chk = t.ket[b];
    const int nb = s.ch[chb].n(), nk = s.ch[chk].n();
    const int ch = term == 1 ? chb : chk;
    if (!nb || !nk || !t.lad_n[ch]) continue;
    GemmJobDev j{};
    j.nosym = 1;
    j.m = nb;
    j.n = nk;
    j.K = t.lad_n[ch];
    j.kidx_off = t.lad_koff[ch];
    j.w_off = t.lad_woff[ch];
    j.phase_off = -1;
    j.out_off = t.off[b];
    j.ldo = nb;
    j.lda = nb;
    j.ldb = nk;
    if (term == 1) {
      j.a_off = s.ch[chb].off;
      j.b_off = t.off[b];
      j.bscale = 1.0;
      j.accumulate = 0;
    } else {
      j.a_off = t.off[b];
      j.b_off = s.ch[chk].off;
      j.bscale = -1.0;
      j.accumulate = 1;
    }
    v.push_back(j);
  }
  return v;
}

// plain split products of Z bar (lo, hi) = M_left M_right, columns [0, n_hi)
// (head) and [n_hi, 2 n_hi) (tail), src/TensorCommutators.cc:1130-1190:
// part 1, K over the 2 nph_lo rows of X bar (lo): A = X bar (lo), B = the
// transposed panel Ybar(lo, hi) (head) or its half-swapped copy (tail, which
// carries hY and the ket phases; the job adds (-1)^(Jlo - Jhi)), overwrite;
// part 2, K over the 2 nph_hi rows of X bar (hi): A = the transposed panel
// Ybar(hi, lo), B = X bar (hi) (head) or its half-swapped copy (tail), scale
// -(-1)^(Jlo - Jhi) hY hX (the launch scale carries hY hX), accumulate
std::vector<GemmJobDev> zbar_jobs(const Space& s, const TensorLayout& t, int part)
{
  std::vector<GemmJobDev> v;
  for (size_t p = 0; p < t.zb_bra.size(); ++p) {
    const int lo = t.zb_bra[p], hi = t.zb_ket[p];
    const int nlo = s.cc[lo].n(), nhi = s.cc[hi].n();
    const int nph = part == 1 ? s.cc_nph[lo] : s.cc_nph[hi];
    if (!nlo || !nhi || !nph) continue;
    const long long y = part == 1 ? t.yb_lookup[(size_t)lo * s.nch + hi] : t.yb_lookup[(size_t)hi * s.nch + lo];
    if (y < 0) continue;
    const double f0 = ((lo / 6 - hi / 6) & 1) ? -1.0 : 1.0;
    for (int tail = 0; tail < 2; ++tail) {
      GemmJobDev j{};
      j.nosym = 1;
      j.m = nlo;
      j.n = nhi;
      j.K = 2 * nph;
      j.kidx_off = -1;
      j.w_off = -1;
      j.phase_off = -1;
      j.bsel = tail;
      j.out_off = t.zb_off[p] + (long long)tail * nhi * nlo;
      j.ldo = nlo;
      j.lda = nlo;
      j.ldb = nhi;
      if (part == 1) {
        j.a_off = s.xb_off[lo];
        j.b_off = y;
        j.bscale = tail ? f0 : 1.0;
        j.accumulate = 0;
      } else {
        j.a_off = y;
        j.b_off = s.xb_off[hi];
        j.bscale = -f0;
        j.accumulate = 1;
      }
      v.push_back(j);
    }
  }
  return v;
}

int split_ready(imsrg_space* sp, TensorLayout* tl)
{
  int rc = scratch(sp, tl);
  if (rc) return rc;
  std::lock_guard<std::mutex> g(sp->mu);
  const Space& s = *sp->s;
  if ((rc = alloc(tl, tl->d_ybt, tl->yb_total)) ||
      (rc = alloc(tl, tl->d_ybtf, tl->yb_total)) || (rc = alloc(tl, tl->d_xbf, s.xb_total)))
    return rc;
  try {
    if (!tl->sp_lad1) tl->sp_lad1 = split_plan_create(s, ladder_jobs(s, *tl, 1), 0);
    if (!tl->sp_lad2) tl->sp_lad2 = split_plan_create(s, ladder_jobs(s, *tl, 2), 0);
    if (!tl->sp_zb1) tl->sp_zb1 = split_plan_create(s, zbar_jobs(s, *tl, 1), 1);
    if (!tl->sp_zb2) tl->sp_zb2 = split_plan_create(s, zbar_jobs(s, *tl, 2), 1);
  } catch (std::exception& e) {
    return terr(IMSRG_ERR_NOMEM, std::string("split-precision plan: ") + e.what());
  }
  return IMSRG_OK;
}

// X bar and the split products' operands (Y transposed, Pandya panels)
int split_operands(const imsrg_op* X, const imsrg_op* Y, cudaStream_t st)
{
  TensorLayout* tl = Y->tl;
  const Space& s = *X->sp->s;
  T_CUDA(launch_pandya_single(s, X->d, X->herm, 1, tl->d_xbar, st));
  T_CUDA(launch_tensor_split_operands(s, *tl, Y->d, Y->herm, tl->d_xbar, tl->d_yt, tl->d_ybt, tl->d_ybtf, tl->d_xbf,
                                      st));
  return IMSRG_OK;
}

int t222_split(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, cudaStream_t st)
{
  TensorLayout* tl = Y->tl;
  const Space& s = *X->sp->s;
  ProfScope ps("comm222_pp_hh_221st", st);
  T_CUDA(cudaMemsetAsync(tl->d_mpp, 0, std::max<long long>(1, tl->total) * sizeof(double), st));
  T_CUDA(launch_symgemm_split(tl->sp_lad1, X->d, tl->d_yt, tl->d_yt, tl->d_mpp, s.work.kidx, s.work.kweight,
                              s.work.phase_tab, X->sp->d_status, 1, 1.0, st));
  T_CUDA(launch_symgemm_split(tl->sp_lad2, Y->d, X->d, X->d, tl->d_mpp, s.work.kidx, s.work.kweight,
                              s.work.phase_tab, X->sp->d_status, 1, (double)X->herm, st));
  T_CUDA(launch_tensor_222_221_split(s, *tl, X->d, Y->d, tl->d_mpp, tl->d_mhh, Z->d, Z->herm, st));
  return IMSRG_OK;
}

int tph_split(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, cudaStream_t st)
{
  TensorLayout* tl = Y->tl;
  const Space& s = *X->sp->s;
  ProfScope ps("comm222_phst", st);
  T_CUDA(cudaMemsetAsync(tl->d_zbar, 0, std::max<long long>(1, tl->zb_total) * sizeof(double), st));
  T_CUDA(launch_symgemm_split(tl->sp_zb1, tl->d_xbar, tl->d_ybt, tl->d_ybtf, tl->d_zbar, s.work.kidx,
                              s.work.kweight, s.work.phase_tab, X->sp->d_status, 1, 1.0, st));
  T_CUDA(launch_symgemm_split(tl->sp_zb2, tl->d_ybt, tl->d_xbar, tl->d_xbf, tl->d_zbar, s.work.kidx,
                              s.work.kweight, s.work.phase_tab, X->sp->d_status, 1, (double)(X->herm * Y->herm),
                              st));
  T_CUDA(launch_tensor_inverse_pandya(s, *tl, tl->d_zbar, Z->d, Z->herm, st));
  return IMSRG_OK;
}

// BCH_Transform's work arenas of a rank
int bch_scratch(imsrg_space* sp, TensorLayout* tl)
{
  std::lock_guard<std::mutex> g(sp->mu);
  int rc;
  if ((rc = alloc(tl, tl->d_bch_nested, tl->total)) || (rc = alloc(tl, tl->d_bch_next, tl->total))) return rc;
  return IMSRG_OK;
}

int check_prec(int precision)
{
  if (precision != IMSRG_PREC_FP64 && precision != IMSRG_PREC_SPLIT) return terr(IMSRG_ERR_ARG, "bad precision");
  return IMSRG_OK;
}

int t111(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, cudaStream_t st)
{
  ProfScope ps("comm111st", st);
  T_CUDA(launch_tensor_111(*X->sp->s, X->d, Y->d, Z->d, st));
  return IMSRG_OK;
}

int t121(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, cudaStream_t st)
{
  ProfScope ps("comm121st", st);
  T_CUDA(launch_tensor_121(*X->sp->s, *Y->tl, X->sp->d_holes, X->d, Y->d, Y->herm, Z->d, Z->herm, st));
  return IMSRG_OK;
}

int t122(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, cudaStream_t st)
{
  TensorLayout* tl = Y->tl;
  int rc = scratch(X->sp, tl);
  if (rc) return rc;
  ProfScope ps("comm122st", st);
  T_CUDA(launch_tensor_122(*X->sp->s, *tl, X->d, Y->d, X->herm, tl->d_yt, Z->d, st));
  return IMSRG_OK;
}

int t222(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, cudaStream_t st)
{
  TensorLayout* tl = Y->tl;
  int rc = scratch(X->sp, tl);
  if (rc) return rc;
  ProfScope ps("comm222_pp_hh_221st", st);
  T_CUDA(launch_tensor_222_221(*X->sp->s, *tl, X->d, Y->d, tl->d_xw, tl->d_wx, tl->d_mpp, tl->d_mhh, Z->d, Z->herm,
                               st));
  return IMSRG_OK;
}

int tph(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, cudaStream_t st)
{
  TensorLayout* tl = Y->tl;
  int rc = scratch(X->sp, tl);
  if (rc) return rc;
  ProfScope ps("comm222_phst", st);
  const Space& s = *X->sp->s;
  // X bar: DoPandyaTransformation(X, ..., "transpose") (src/TensorCommutators.cc:1067)
  T_CUDA(launch_pandya_single(s, X->d, X->herm, 1, tl->d_xbar, st));
  T_CUDA(cudaMemsetAsync(tl->d_zbar, 0, std::max<long long>(1, tl->zb_total) * sizeof(double), st));
  T_CUDA(launch_tensor_ph(s, *tl, tl->d_xbar, Y->d, X->herm, Y->herm, tl->d_ybar, tl->d_zbar, Z->d, Z->herm, st));
  return IMSRG_OK;
}

int z_herm_st(int hx, int hy) { return hx == hy ? -1 : 1; }

}  // namespace

extern "C" {

int imsrg_comm111st(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, void* stream)
{
  int rc = check_st(X, Y, Z);
  return rc ? rc : t111(X, Y, Z, (cudaStream_t)stream);
}

int imsrg_comm121st(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, void* stream)
{
  int rc = check_st(X, Y, Z);
  return rc ? rc : t121(X, Y, Z, (cudaStream_t)stream);
}

int imsrg_comm122st(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, void* stream)
{
  int rc = check_st(X, Y, Z);
  return rc ? rc : t122(X, Y, Z, (cudaStream_t)stream);
}

int imsrg_comm222_pp_hh_221st(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, int precision, void* stream)
{
  int rc = check_st(X, Y, Z);
  if (rc || (rc = check_prec(precision))) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  if (precision == IMSRG_PREC_FP64) return t222(X, Y, Z, st);
  if ((rc = split_ready(X->sp, Y->tl)) || (rc = split_operands(X, Y, st)) || (rc = t222_split(X, Y, Z, st)))
    return rc;
  return end_status(X->sp, st);
}

int imsrg_comm222_phst(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, int precision, void* stream)
{
  int rc = check_st(X, Y, Z);
  if (rc || (rc = check_prec(precision))) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  if (precision == IMSRG_PREC_FP64) return tph(X, Y, Z, st);
  if ((rc = split_ready(X->sp, Y->tl)) || (rc = split_operands(X, Y, st)) || (rc = tph_split(X, Y, Z, st)))
    return rc;
  return end_status(X->sp, st);
}

int imsrg_commutator_scalar_tensor(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, int precision, void* stream)
{
  if (!X || !Y || !Z) return terr(IMSRG_ERR_ARG, "null operator");
  if (Z == X || Z == Y) return terr(IMSRG_ERR_ARG, "Z must not alias X or Y");
  int rc = check_prec(precision);
  if (rc) return rc;
  Z->herm = z_herm_st(X->herm, Y->herm);
  if ((rc = check_st(X, Y, Z))) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  if (precision == IMSRG_PREC_SPLIT && (rc = split_ready(X->sp, Y->tl))) return rc;
  bool on[5];
  tensor_terms_on(on);  // Commutator::comm_term_on, as CommutatorScalarTensor consults it
  ProfScope ps("CommutatorScalarTensor", st);
  T_CUDA(cudaMemsetAsync(Z->d, 0, Z->len * sizeof(double), st));
  if ((on[0] && (rc = t111(X, Y, Z, st))) || (on[1] && (rc = t121(X, Y, Z, st))) ||
      (on[2] && (rc = t122(X, Y, Z, st))))
    return rc;
  if (precision == IMSRG_PREC_FP64) {
    if ((on[3] && (rc = t222(X, Y, Z, st))) || (on[4] && (rc = tph(X, Y, Z, st)))) return rc;
  } else if (on[3] || on[4]) {
    if ((rc = split_operands(X, Y, st)) || (on[3] && (rc = t222_split(X, Y, Z, st))) ||
        (on[4] && (rc = tph_split(X, Y, Z, st))))
      return rc;
    return end_status(X->sp, st);
  }
  return IMSRG_OK;
}

}  // extern "C"

namespace imsrg {

// Operator::Norm of a tensor operator (src/Operator.cc:1610-1646 with
// TwoBodyME::Norm, src/TwoBodyME.cc:703-725)
int tensor_norm_dev(const imsrg_op* op, double* out, cudaStream_t st)
{
  TensorLayout* tl = op->tl;
  const size_t n2 = tl->nrm2_off.size();
  T_CUDA(launch_tensor_norm(*tl, op->d, tl->d_nrm_partial, st));
  T_CUDA(cudaMemcpyAsync(tl->h_nrm_partial.data(), tl->d_nrm_partial, (n2 + 1) * sizeof(double),
                         cudaMemcpyDeviceToHost, st));
  T_CUDA(cudaStreamSynchronize(st));
  double s2 = 0.0;
  for (size_t c = 0; c < n2; ++c) s2 += tl->h_nrm_partial[c];
  *out = std::sqrt(tl->h_nrm_partial[n2] + s2);
  return IMSRG_OK;
}

// BCH::Standard_BCH_Transform (src/BCH.cc:87-201) of a tensor operator by a
// scalar Omega: the same series and stopping rule as the scalar form, with
// the nested commutators [Omega, .] from CommutatorScalarTensor
int tensor_bch_transform(const imsrg_op* OpIn, const imsrg_op* Omega, imsrg_op* OpOut, double threshold,
                         int precision, int* n_nested, cudaStream_t st)
{
  TensorLayout* tl = OpIn->tl;
  imsrg_space* sp = OpIn->sp;
  if (n_nested) *n_nested = 0;
  int rc;
  double nx = 0, ny = 0;
  if ((rc = tensor_norm_dev(OpIn, &nx, st)) || (rc = norm_dev(Omega, &ny, st))) return rc;
  if ((rc = imsrg_op_copy(OpOut, OpIn, st))) return rc;
  if (!(nx > threshold)) return IMSRG_OK;
  if ((rc = bch_scratch(sp, tl))) return rc;
  imsrg_op nested, next;
  nested.sp = next.sp = sp;
  nested.tl = next.tl = tl;
  nested.len = next.len = tl->total;
  nested.d = tl->d_bch_nested;
  next.d = tl->d_bch_next;
  T_CUDA(cudaMemcpyAsync(nested.d, OpOut->d, tl->total * sizeof(double), cudaMemcpyDeviceToDevice, st));
  nested.herm = OpOut->herm;
  double epsilon = nx * std::exp(-2 * ny) * threshold / (2 * ny);
  double fden = 1.0;
  for (int i = 1; i <= 40; ++i) {
    if ((rc = imsrg_commutator_scalar_tensor(Omega, &nested, &next, precision, st))) return rc;
    std::swap(nested.d, next.d);
    std::swap(nested.herm, next.herm);
    fden /= i;
    T_CUDA(launch_axpy(OpOut->d, nested.d, fden, tl->total, st));
    if (n_nested) *n_nested = i;
    epsilon *= i + 1;
    double nn = 0;
    if ((rc = tensor_norm_dev(&nested, &nn, st))) return rc;
    if (nn < epsilon) break;
  }
  return IMSRG_OK;
}

}  // namespace imsrg
