// imsrg_comm122ss_noalloc: comm122ss (plain FP64 form) that allocates no
// device memory.
//
// Who needs it: callers that cannot call cudaMalloc at the point where they
// evaluate the term -- code running under a fixed device-memory budget or a
// caching allocator that owns all device memory, code inside a region where
// allocation is not allowed (e.g. while other work holds the allocator), or
// hosts that hand the library only pre-allocated buffers.  The regular
// imsrg_comm122ss allocates its W2 intermediate (an arena-sized scratch) on
// first use; this variant keeps W2 in a library-owned static device array.
//
// The array: g_w2_scratch, 2^21 doubles (16 MiB), file-scope __device__, held
// by every GPU that loads the library until the process exits.  It bounds the
// model spaces this entry point accepts (arena length <= 2^21 doubles, i.e.
// emax <= 6 for the O16 reference); larger spaces are rejected with
// IMSRG_ERR_ARG.  Every call shares the array and leaves its contents behind;
// the W2 kernel overwrites every element it later reads, so nothing needs
// clearing.  Calls that overlap on the GPU (different streams, no ordering)
// race on the array.
//
// Set-up happens when the space's device tables are built (its first
// operator, imsrg_op_create), with the space's device current: host code never
// passes g_w2_scratch itself to a kernel (in host code that name is a
// host-side stand-in, not a device address), so the device address is looked
// up there with cudaGetSymbolAddress, once per device, and the comm122ss
// kernels are loaded.  Under lazy module loading that step is what commits
// the array's 16 MiB on the device; the entry point itself then neither
// allocates nor loads anything.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/imsrg_gb300.h"
#include "capi_internal.hpp"
#include "kernels.cuh"

namespace {

constexpr long long kScratchDoubles = 1ll << 21;  // 16 MiB
__device__ __align__(256) double g_w2_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_sym_mu;
double* g_sym_addr[kMaxDevices] = {};

}  // namespace

namespace imsrg {

// the set-up of imsrg_comm122ss_noalloc on the current device (device), run
// while a space's device tables are built
int noalloc_setup(imsrg_space* sp, int device)
{
  if (device < 0 || device >= kMaxDevices) return set_error(IMSRG_ERR_ARG, "device ordinal out of range");
  std::lock_guard<std::mutex> g(g_sym_mu);
  if (!g_sym_addr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_w2_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      return set_error(IMSRG_ERR_CUDA, "cudaGetSymbolAddress of the comm122ss scratch failed");
    }
    e = load_comm122_kernels();
    if (e != cudaSuccess) {
      cudaGetLastError();
      return set_error(IMSRG_ERR_CUDA, "loading the comm122ss kernels failed");
    }
    g_sym_addr[device] = (double*)p;
  }
  sp->noalloc_w2 = g_sym_addr[device];
  return IMSRG_OK;
}

}  // namespace imsrg

extern "C" int imsrg_comm122ss_noalloc(const imsrg_space* s, const double* X, const double* Y, double* Z, int hZ,
                                       void* stream)
{
  if (!s || !X || !Y || !Z) return imsrg::set_error(IMSRG_ERR_ARG, "null argument");
  if (hZ != 1 && hZ != -1) return imsrg::set_error(IMSRG_ERR_UNSUPPORTED, "Z must be hermitian or anti-hermitian");
  if (!s->dev_ready || !s->noalloc_w2)
    return imsrg::set_error(IMSRG_ERR_ARG,
                            "the space has no device tables yet: create an operator on it first (imsrg_op_create)");
  if (s->s->arena > kScratchDoubles)
    return imsrg::set_error(IMSRG_ERR_ARG,
                            "model space too large for imsrg_comm122ss_noalloc: arena above 2^21 doubles (16 MiB)");
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return imsrg::set_error(IMSRG_ERR_CUDA, "cudaGetDevice failed");
  }
  if (dev != s->device)
    return imsrg::set_error(IMSRG_ERR_ARG,
                            "the current CUDA device is not the one the space's tables live on: make it current");
  cudaError_t e =
      imsrg::launch_comm122(*s->s, X, Y, Z, s->noalloc_w2, hZ, s->d_sym122, s->n_sym122, (cudaStream_t)stream);
  if (e != cudaSuccess) return imsrg::set_error(IMSRG_ERR_CUDA, cudaGetErrorString(e));
  return IMSRG_OK;
}
