// Internal definitions of the opaque C-ABI handles (imsrg_space, imsrg_op),
// shared by the translation units that implement include/imsrg_gb300.h.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "kernels.cuh"
#include "space.hpp"
#include "tensor.hpp"

using imsrg::GemmJobDev;
using imsrg::Space;
using imsrg::SplitPlan;

struct imsrg_op;
struct imsrg_space;

namespace imsrg {
// sets the calling thread's imsrg_last_error() message and returns code
int set_error(int code, const char* msg);
// CommutatorScalarScalar into Z (overwritten), Operator::Norm (synchronises
// st), and the kernels' error word (synchronises st; IMSRG_ERR_KERNEL if set)
int commutator_dev(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, int prec, cudaStream_t st);
int norm_dev(const imsrg_op* op, double* out, cudaStream_t st);
int status_dev(imsrg_space* sp, cudaStream_t st);
// imsrg_comm122ss_noalloc's set-up on the current device (noalloc.cu)
int noalloc_setup(imsrg_space* sp, int device);
// the status read that ends a commutator or term entry point: status_dev, or
// nothing when the space defers it to imsrg_space_check_status
int end_status(imsrg_space* sp, cudaStream_t st);
// tensor operators (capi_tensor.cu): Operator::Norm, and BCH_Transform by a
// scalar Omega
int tensor_norm_dev(const imsrg_op* op, double* out, cudaStream_t st);
int tensor_bch_transform(const imsrg_op* OpIn, const imsrg_op* Omega, imsrg_op* OpOut, double threshold,
                         int precision, int* n_nested, cudaStream_t st);
// the commutator of a group of same-structure pairs, one launch per kernel
// for the whole group (either form): usable only with every term switched on
bool batch_phases_usable();
// the scalar-tensor term switches: comm111st, comm121st, comm122st,
// comm222_pp_hh_221st (comm222_pp_hhst and comm221st), comm222_phst
void tensor_terms_on(bool on[5]);
// the ladder and Zbar products of same-structure pairs as one launch each
// (split plans, or FP64 job lists over every pair)
struct GroupedProducts;
GroupedProducts* grouped_products_create(const std::vector<const imsrg_op*>& X, const std::vector<const imsrg_op*>& Y,
                                         const std::vector<imsrg_op*>& Z, int prec, std::string* why);
void grouped_products_destroy(GroupedProducts* g);
int grouped_ladder(GroupedProducts* g, cudaStream_t st);
int grouped_zbar(GroupedProducts* g, cudaStream_t st);
// the per-pair phases of the same pairs as one launch per kernel
int group_pre(GroupedProducts* g, cudaStream_t st);
int group_mid(GroupedProducts* g, cudaStream_t st);
int group_post(GroupedProducts* g, cudaStream_t st);
}  // namespace imsrg

struct imsrg_space {
  Space* s = nullptr;
  bool dev_ready = false;
  int device = -1;            // CUDA device the tables (and every operator) live on
  bool defer_status = false;  // imsrg_space_defer_status
  double* noalloc_w2 = nullptr;  // device address of the no-alloc entry's static W2 array on that device
  std::mutex mu;
  std::vector<void*> allocs;
  int* d_holes = nullptr;
  // FP64 symmetrised products
  GemmJobDev* d_ladder_jobs = nullptr;
  int* d_ladder_pairs = nullptr;
  int n_ladder_pairs = 0;
  std::vector<GemmJobDev> ladder_jobs, zbar_jobs;
  GemmJobDev* d_zbar_jobs = nullptr;
  int* d_zbar_pairs = nullptr;
  int n_zbar_pairs = 0;
  // other tile lists
  int* d_sym122 = nullptr;
  int n_sym122 = 0;
  int* d_sym122u = nullptr;  // tile pairs a <= b (fused split-form comm122ss)
  int n_sym122u = 0;
  int* d_pinv = nullptr;
  int n_pinv = 0;
  int* d_invq = nullptr;  // quadruple blocks of the split-form inverse Pandya transform
  int n_invq = 0;
  int* d_cls_list = nullptr;
  int* d_cls_off = nullptr;
  unsigned char* d_cls_sort = nullptr;
  std::vector<std::pair<int64_t, int64_t>> zbar_zero;  // Zbar regions with no ph kets
  // norm chunks
  long long* d_norm_off = nullptr;
  int* d_norm_len = nullptr;
  double* d_norm_w = nullptr;
  int n_norm = 0;
  double* d_norm_partial = nullptr;
  std::vector<double> h_norm_partial;
  // scratch
  double *d_xb = nullptr, *d_yt = nullptr, *d_yf = nullptr, *d_zb = nullptr, *d_w2 = nullptr;
  float2 *d_xf = nullptr, *d_yff = nullptr;  // (hi, lo) copies of X and Y for the double-float comm122ss
  int* d_status = nullptr;
  // split-precision plans
  SplitPlan* split_ladder = nullptr;
  SplitPlan* split_zbar = nullptr;
  // BCH work operators (d_prod: BCH_Product result when Z aliases X or Y)
  double *d_nested = nullptr, *d_next = nullptr, *d_prod = nullptr;
  // generator scratch: monopoles V(ab, ab) of H, norb^2
  double* d_mono = nullptr;
  // tuning (imsrg_space_set_tuning, or this space's entry of the tuning file)
  imsrg::SplitOpts opt_ladder, opt_zbar;
  int inv_split = 0;  // split form's inverse Pandya: 0 quadruple blocks (double-float), 1 descriptors
                      // (double-float), 2 descriptors (FP64)
  int inv_fp64 = 0;   // FP64 form's inverse Pandya: 0 channel tiles, 1 descriptors (FP64)
  int invq_budget = imsrg::kInvqBudget;
  int invd_stage = 2048, invd_res = 2048;
  int invd_weights = 0;  // descriptor kernel: 1 stages the 6j weight rows per block
  int invd_ilp = 1;      // descriptor kernel: results in flight per thread (1, 2, 4)
  int comm122_fused = 0;  // split-form comm122ss: 1 forms W2 tiles in shared memory (no W2 round trip)
  std::string tuning_source = "default";
  // inverse Pandya descriptors (built on first use)
  imsrg::InvdDev invd;
  bool invd_ready = false;
  std::vector<void*> invd_allocs;
  // second stream of CommutatorScalarScalar (work independent of the ladder
  // product) and the events that fork it from and join it to the caller's
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;

  template <class T>
  T* track(T* p)
  {
    allocs.push_back((void*)p);
    return p;
  }
  ~imsrg_space()
  {
    if (split_ladder) split_plan_destroy(split_ladder);
    if (split_zbar) split_plan_destroy(split_zbar);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    if (side) cudaStreamDestroy(side);
    for (void* p : allocs) cudaFree(p);
    for (void* p : invd_allocs) cudaFree(p);
    delete s;
  }
};

struct imsrg_op {
  imsrg_space* sp = nullptr;
  double* d = nullptr;
  int herm = 1;
  long long len = 0;  // arena length in doubles
  // reduced tensor operators (imsrg_op_create_tensor): their layout; nullptr
  // for the scalar operators of the IMSRG(2) scalar commutator
  imsrg::TensorLayout* tl = nullptr;
};

