// Split-precision symmetrised channel products (placeholder until the tcgen05
// kernel lands): reports "not supported".
#include <cuda_runtime.h>

#include "kernels.cuh"

namespace imsrg {

struct SplitPlan {
  int family = 0;
};

SplitPlan* split_plan_create(const Space&, const std::vector<GemmJobDev>&, int family)
{
  SplitPlan* p = new SplitPlan();
  p->family = family;
  return p;
}

void split_plan_destroy(SplitPlan* p) { delete p; }

cudaError_t launch_symgemm_split(SplitPlan*, const double*, const double*, const double*, double*, const int*,
                                 const double*, const int*, int*, cudaStream_t)
{
  return cudaErrorNotSupported;
}

}  // namespace imsrg
