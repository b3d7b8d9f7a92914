// extern "C" boundary, scalar-tensor commutator (include/imsrg_gb300.h):
// Commutator::CommutatorScalarTensor (src/Commutator.cc:432-500) and its
// IMSRG(2) terms on device operators.  X is a scalar operator, Y and Z are
// reduced tensors of the same rank (imsrg_op_create_tensor).
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <string>

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
      (rc = alloc(tl, tl->d_wx, sp->s->arena)))
    return rc;
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
  ProfScope ps("comm122st", st);
  T_CUDA(launch_tensor_122(*X->sp->s, *Y->tl, X->d, Y->d, Y->herm, Z->d, st));
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

int imsrg_comm222_pp_hh_221st(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, void* stream)
{
  int rc = check_st(X, Y, Z);
  return rc ? rc : t222(X, Y, Z, (cudaStream_t)stream);
}

int imsrg_comm222_phst(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, void* stream)
{
  int rc = check_st(X, Y, Z);
  return rc ? rc : tph(X, Y, Z, (cudaStream_t)stream);
}

int imsrg_commutator_scalar_tensor(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, void* stream)
{
  if (!X || !Y || !Z) return terr(IMSRG_ERR_ARG, "null operator");
  if (Z == X || Z == Y) return terr(IMSRG_ERR_ARG, "Z must not alias X or Y");
  Z->herm = z_herm_st(X->herm, Y->herm);
  int rc = check_st(X, Y, Z);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  ProfScope ps("CommutatorScalarTensor", st);
  T_CUDA(cudaMemsetAsync(Z->d, 0, Z->len * sizeof(double), st));
  if ((rc = t111(X, Y, Z, st)) || (rc = t121(X, Y, Z, st)) || (rc = t122(X, Y, Z, st)) || (rc = t222(X, Y, Z, st)) ||
      (rc = tph(X, Y, Z, st)))
    return rc;
  return IMSRG_OK;
}

}  // extern "C"
