// extern "C" boundary, batched commutators (include/imsrg_gb300.h): many
// independent CommutatorScalarScalar calls of uneven size replayed as one
// CUDA graph.  Capturing removes the per-kernel launch latency that dominates
// commutators at small emax (a few microseconds of work per kernel).
//
// Two graph shapes:
//  - grouped (either form, every term on, one model space per pair): pairs of
//    the same structure form a group, and each group is one chain of
//    launches in which every kernel of the commutator runs once for all the
//    group's pairs (the grid's z runs over pairs; the two dense products are
//    one persistent grid over the tiles of every pair), so the pairs share
//    the GPU inside each launch instead of taking it in turn;
//  - branches (otherwise): pairs grouped by model space (a space's scratch
//    serialises the pairs that share it), one branch per space running whole
//    commutators.
#include <cuda_runtime.h>

#include <map>
#include <string>
#include <vector>

#include "../../include/imsrg_gb300.h"
#include "capi_internal.hpp"
#include "prof.hpp"

using namespace imsrg;

struct imsrg_batch {
  std::vector<const imsrg_op*> X, Y;
  std::vector<imsrg_op*> Z;
  std::vector<imsrg_space*> spaces;  // one per group
  std::vector<std::vector<int>> groups;
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> joins;
  cudaEvent_t fork = nullptr;
  cudaStream_t cap = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int prec = IMSRG_PREC_FP64;
  size_t kernel_nodes = 0;
  // grouped shape: products per structure group, their streams and joins
  bool grouped = false;
  std::vector<GroupedProducts*> products;
  std::vector<cudaStream_t> gstreams;
  std::vector<cudaEvent_t> gjoins;

  ~imsrg_batch()
  {
    for (GroupedProducts* g : products) grouped_products_destroy(g);
    for (cudaEvent_t e : gjoins) cudaEventDestroy(e);
    for (cudaStream_t s : gstreams) cudaStreamDestroy(s);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    for (cudaEvent_t e : joins) cudaEventDestroy(e);
    if (fork) cudaEventDestroy(fork);
    for (cudaStream_t s : streams) cudaStreamDestroy(s);
    if (cap) cudaStreamDestroy(cap);
  }
};

namespace {

int berr(int code, const std::string& msg) { return set_error(code, msg.c_str()); }

#define BATCH_CUDA(expr)                                                                \
  do {                                                                                  \
    cudaError_t _e = (expr);                                                            \
    if (_e != cudaSuccess) return berr(IMSRG_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e)); \
  } while (0)

// grouped shape: every structure group is one chain on its own stream --
// the group's per-pair phases and products each as one launch over its pairs
int record_grouped(imsrg_batch* b)
{
  BATCH_CUDA(cudaEventRecord(b->fork, b->cap));
  for (size_t g = 0; g < b->products.size(); ++g) {
    cudaStream_t s = b->gstreams[g];
    GroupedProducts* gp = b->products[g];
    BATCH_CUDA(cudaStreamWaitEvent(s, b->fork, 0));
    int rc;
    if ((rc = group_pre(gp, s)) || (rc = grouped_ladder(gp, s)) || (rc = group_mid(gp, s)) ||
        (rc = grouped_zbar(gp, s)) || (rc = group_post(gp, s)))
      return rc;
    BATCH_CUDA(cudaEventRecord(b->gjoins[g], s));
    BATCH_CUDA(cudaStreamWaitEvent(b->cap, b->gjoins[g], 0));
  }
  return IMSRG_OK;
}

// the grouped shape's product groups: pairs of equal structure and hermiticity
int setup_grouped(imsrg_batch* b)
{
  std::map<std::vector<long long>, std::vector<int>> keyed;
  for (size_t i = 0; i < b->X.size(); ++i) {
    const Space& s = *b->X[i]->sp->s;
    keyed[{s.emax, s.norb, s.nch, s.arena, b->X[i]->herm, b->Y[i]->herm}].push_back((int)i);
  }
  for (auto& kv : keyed) {
    std::vector<const imsrg_op*> X, Y;
    std::vector<imsrg_op*> Z;
    for (int i : kv.second) {
      X.push_back(b->X[i]);
      Y.push_back(b->Y[i]);
      Z.push_back(b->Z[i]);
    }
    std::string why;
    GroupedProducts* g = grouped_products_create(X, Y, Z, b->prec, &why);
    if (!g) return berr(IMSRG_ERR_UNSUPPORTED, why);
    b->products.push_back(g);
    cudaStream_t s = nullptr;
    cudaEvent_t e = nullptr;
    BATCH_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    b->gstreams.push_back(s);
    BATCH_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    b->gjoins.push_back(e);
  }
  return IMSRG_OK;
}

// the graph's branches: fork from the capture stream, every group's pairs in
// order on the group's stream, join back
int record(imsrg_batch* b)
{
  if (b->grouped) return record_grouped(b);
  BATCH_CUDA(cudaEventRecord(b->fork, b->cap));
  for (size_t g = 0; g < b->groups.size(); ++g) {
    cudaStream_t s = b->streams[g];
    BATCH_CUDA(cudaStreamWaitEvent(s, b->fork, 0));
    for (int i : b->groups[g]) {
      int rc = commutator_dev(b->X[i], b->Y[i], b->Z[i], b->prec, s);
      if (rc) return rc;
    }
    BATCH_CUDA(cudaEventRecord(b->joins[g], s));
    BATCH_CUDA(cudaStreamWaitEvent(b->cap, b->joins[g], 0));
  }
  return IMSRG_OK;
}

}  // namespace

extern "C" {

int imsrg_batch_create(int n, const imsrg_op* const* X, const imsrg_op* const* Y, imsrg_op* const* Z, int precision,
                       imsrg_batch** out)
{
  if (!out || n <= 0 || !X || !Y || !Z) return berr(IMSRG_ERR_ARG, "bad arguments");
  if (precision != IMSRG_PREC_FP64 && precision != IMSRG_PREC_SPLIT) return berr(IMSRG_ERR_ARG, "bad precision");
  *out = nullptr;
  imsrg_batch* b = new imsrg_batch();
  b->prec = precision;
  std::map<imsrg_space*, int> gid;
  for (int i = 0; i < n; ++i) {
    if (!X[i] || !Y[i] || !Z[i]) {
      delete b;
      return berr(IMSRG_ERR_ARG, "null operator in batch");
    }
    for (int j = 0; j < i; ++j)
      if (Z[j] == Z[i]) {
        delete b;
        return berr(IMSRG_ERR_ARG, "two pairs of a batch write the same Z");
      }
    b->X.push_back(X[i]);
    b->Y.push_back(Y[i]);
    b->Z.push_back(Z[i]);
    imsrg_space* sp = X[i]->sp;
    auto it = gid.find(sp);
    if (it == gid.end()) {
      it = gid.emplace(sp, (int)b->groups.size()).first;
      b->groups.emplace_back();
      b->spaces.push_back(sp);
    }
    b->groups[it->second].push_back(i);
  }
  // one eager pass: allocates every space's scratch and plans (nothing may
  // allocate while the graph is captured) and checks the arguments
  for (int i = 0; i < n; ++i) {
    int rc = commutator_dev(X[i], Y[i], Z[i], precision, nullptr);
    if (rc) {
      delete b;
      return rc;
    }
  }
  cudaError_t e = cudaStreamSynchronize(nullptr);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
  for (size_t g = 0; e == cudaSuccess && g < b->groups.size(); ++g) {
    cudaStream_t s = nullptr;
    cudaEvent_t j = nullptr;
    e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess) b->streams.push_back(s);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&j, cudaEventDisableTiming);
    if (e == cudaSuccess) b->joins.push_back(j);
  }
  if (e != cudaSuccess) {
    delete b;
    return berr(IMSRG_ERR_CUDA, std::string("batch setup: ") + cudaGetErrorString(e));
  }
  if (precision == IMSRG_PREC_SPLIT)
    for (imsrg_space* sp : b->spaces) {
      int rc = status_dev(sp, nullptr);
      if (rc) {
        delete b;
        return rc;
      }
    }
  // the grouped shape when it applies; the branch shape otherwise
  if (batch_phases_usable() && (int)b->groups.size() == n) {
    b->grouped = true;
    if (setup_grouped(b) != IMSRG_OK) {
      for (GroupedProducts* g : b->products) grouped_products_destroy(g);
      b->products.clear();
      b->grouped = false;
    }
  }
  // the phase timers record events and read them back: not inside a graph
  const bool prof_was_on = prof_enabled();
  imsrg_profiler_enable(0);
  e = cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) {
    imsrg_profiler_enable(prof_was_on);
    delete b;
    return berr(IMSRG_ERR_CUDA, std::string("cudaStreamBeginCapture: ") + cudaGetErrorString(e));
  }
  int rc = record(b);
  cudaGraph_t g = nullptr;
  e = cudaStreamEndCapture(b->cap, &g);
  imsrg_profiler_enable(prof_was_on);
  b->graph = g;
  if (rc || e != cudaSuccess) {
    std::string why = rc ? "" : std::string("cudaStreamEndCapture: ") + cudaGetErrorString(e);
    cudaGetLastError();
    delete b;
    return rc ? rc : berr(IMSRG_ERR_CUDA, why);
  }
  e = cudaGraphInstantiate(&b->exec, b->graph, 0);
  if (e != cudaSuccess) {
    delete b;
    return berr(IMSRG_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
  }
  size_t nn = 0;
  if (cudaGraphGetNodes(b->graph, nullptr, &nn) == cudaSuccess && nn) {
    std::vector<cudaGraphNode_t> nodes(nn);
    if (cudaGraphGetNodes(b->graph, nodes.data(), &nn) == cudaSuccess)
      for (cudaGraphNode_t nd : nodes) {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++b->kernel_nodes;
      }
  }
  *out = b;
  return IMSRG_OK;
}

void imsrg_batch_destroy(imsrg_batch* b) { delete b; }

int imsrg_batch_launch(imsrg_batch* b, void* stream)
{
  if (!b) return berr(IMSRG_ERR_ARG, "null batch");
  BATCH_CUDA(cudaGraphLaunch(b->exec, (cudaStream_t)stream));
  g_kernel_launches.fetch_add((long long)b->kernel_nodes, std::memory_order_relaxed);
  return IMSRG_OK;
}

int imsrg_batch_sync(imsrg_batch* b, void* stream)
{
  if (!b) return berr(IMSRG_ERR_ARG, "null batch");
  BATCH_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  if (b->prec == IMSRG_PREC_SPLIT)
    for (imsrg_space* sp : b->spaces) {
      int rc = status_dev(sp, (cudaStream_t)stream);
      if (rc) return rc;
    }
  return IMSRG_OK;
}

int imsrg_batch_info(const imsrg_batch* b, int* n_pairs, int* n_branches, int* n_product_groups,
                     long long* kernel_nodes)
{
  if (!b) return berr(IMSRG_ERR_ARG, "null batch");
  if (n_pairs) *n_pairs = (int)b->X.size();
  if (n_branches) *n_branches = (int)b->groups.size();
  if (n_product_groups) *n_product_groups = b->grouped ? (int)b->products.size() : 0;
  if (kernel_nodes) *kernel_nodes = (long long)b->kernel_nodes;
  return IMSRG_OK;
}

}  // extern "C"
