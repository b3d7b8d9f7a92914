// extern "C" boundary, flow layer (include/imsrg_gb300.h): the White-type
// generators, BCH::BCH_Product and the Magnus-Euler IMSRG solver, on
// device-resident operators.  Everything here is composed from the C ABI's
// operator algebra, CommutatorScalarScalar and the BCH transform; the only
// kernels of its own are the generator's (kernels_terms.cu).  The host keeps
// the reference's control flow because every branch of it (series
// truncation, step size, Omega splitting) depends on an operator norm.
#include <cuda_runtime.h>

#include <unistd.h>

#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "../../include/imsrg_gb300.h"
#include "capi_internal.hpp"
#include "kernels.cuh"
#include "prof.hpp"

using namespace imsrg;

namespace {

int err(int code, const std::string& msg) { return set_error(code, msg.c_str()); }

#define FLOW_CUDA(expr)                                                                \
  do {                                                                                 \
    cudaError_t _e = (expr);                                                           \
    if (_e != cudaSuccess) return err(IMSRG_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e)); \
  } while (0)

#define FLOW_TRY(expr)          \
  do {                          \
    int _rc = (expr);           \
    if (_rc != IMSRG_OK) return _rc; \
  } while (0)

cudaStream_t S_(void* st) { return (cudaStream_t)st; }

int ensure_arena(imsrg_space* sp, double*& p)
{
  if (p) return IMSRG_OK;
  void* q = nullptr;
  if (cudaMalloc(&q, sp->s->arena * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    return err(IMSRG_ERR_NOMEM, "work operator allocation failed");
  }
  p = sp->track((double*)q);
  return IMSRG_OK;
}

double zero_body(const imsrg_op* op, cudaStream_t st, int* rc)
{
  double v = 0.0;
  if (cudaMemcpyAsync(&v, op->d, sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    *rc = err(IMSRG_ERR_CUDA, "reading ZeroBody failed");
  return v;
}

int generator_impl(const imsrg_op* H, imsrg_op* Eta, const GenParams& p, cudaStream_t st)
{
  imsrg_space* sp = H->sp;
  if (!sp->d_mono) {
    void* q = nullptr;
    if (cudaMalloc(&q, (size_t)sp->s->norb * sp->s->norb * sizeof(double)) != cudaSuccess) {
      cudaGetLastError();
      return err(IMSRG_ERR_NOMEM, "generator scratch allocation failed");
    }
    sp->d_mono = sp->track((double*)q);
  }
  ProfScope ps("UpdateEta", st);
  FLOW_CUDA(launch_generator(*sp->s, H->d, Eta->d, sp->d_mono, p, st));
  Eta->herm = -1;
  return IMSRG_OK;
}

// BCH::BCH_Product, src/BCH.cc:267-350 (factorized correction off, its default)
int bch_product_impl(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, double threshold, int prec, int* n_comm,
                     cudaStream_t st)
{
  static const double bern[9] = {1.0, -0.5, 1. / 6, 0.0, -1. / 30, 0.0, 1. / 42, 0, -1. / 30};
  static const double fact[9] = {1.0, 1.0, 2.0, 6.0, 24., 120., 720., 5040., 40320.};
  imsrg_space* sp = X->sp;
  const long long A = sp->s->arena;
  if (n_comm) *n_comm = 0;
  FLOW_TRY(ensure_arena(sp, sp->d_nested));
  FLOW_TRY(ensure_arena(sp, sp->d_next));
  const bool alias = (Z == X || Z == Y);
  if (alias) FLOW_TRY(ensure_arena(sp, sp->d_prod));
  ProfScope ps("BCH_Product", st);
  imsrg_op out, nested, next;
  out.sp = nested.sp = next.sp = sp;
  out.d = alias ? sp->d_prod : Z->d;
  out.herm = X->herm;  // Operator Z = X + Y keeps X's symmetry flags
  nested.d = sp->d_nested;
  next.d = sp->d_next;
  double nx = 0, ny = 0;
  FLOW_TRY(norm_dev(X, &nx, st));
  FLOW_TRY(norm_dev(Y, &ny, st));
  FLOW_CUDA(cudaMemcpyAsync(out.d, X->d, A * sizeof(double), cudaMemcpyDeviceToDevice, st));
  FLOW_CUDA(launch_axpy(out.d, Y->d, 1.0, A, st));
  FLOW_TRY(commutator_dev(Y, X, &nested, prec, st));  // [Y,X]
  int nc = 1;
  double nxy = 0;
  FLOW_TRY(norm_dev(&nested, &nxy, st));
  if (nxy * nx > threshold) {
    FLOW_TRY(commutator_dev(&nested, X, &next, prec, st));  // [[Y,X],X] = [X,[X,Y]]
    ++nc;
    FLOW_CUDA(launch_axpy(out.d, next.d, 1. / 12, A, st));
  }
  size_t k = 1;
  while (nxy > threshold) {
    if (k < 2 || k % 2 == 0) FLOW_CUDA(launch_axpy(out.d, nested.d, bern[k] / fact[k], A, st));
    ++k;
    if (k >= 9) break;
    if (2 * ny * nxy < threshold) break;
    FLOW_TRY(commutator_dev(Y, &nested, &next, prec, st));
    std::swap(nested.d, next.d);
    std::swap(nested.herm, next.herm);
    ++nc;
    FLOW_TRY(norm_dev(&nested, &nxy, st));
  }
  if (prec == IMSRG_PREC_SPLIT) FLOW_TRY(status_dev(sp, st));
  if (alias) FLOW_CUDA(cudaMemcpyAsync(Z->d, out.d, A * sizeof(double), cudaMemcpyDeviceToDevice, st));
  Z->herm = out.herm;
  if (n_comm) *n_comm = nc;
  return IMSRG_OK;
}

int gen_type(const char* t, int* out)
{
  if (!t) return err(IMSRG_ERR_ARG, "null generator type");
  static const char* names[] = {"white", "atan", "wegner", "imaginary-time"};
  for (int i = 0; i < 4; ++i)
    if (!std::strcmp(t, names[i])) {
      *out = i;
      return IMSRG_OK;
    }
  // qtransfer-atan and qtransfer-atan_<n> (src/Generator.cc:55, :63-69)
  if (!std::strcmp(t, "qtransfer-atan")) {
    *out = GEN_QTRANSFER_BASE + 1;
    return IMSRG_OK;
  }
  if (!std::strncmp(t, "qtransfer-atan_", 15)) {
    const int n = std::atoi(t + 15);
    if (n >= 1 && n <= 16) {
      *out = GEN_QTRANSFER_BASE + n;
      return IMSRG_OK;
    }
  }
  return err(IMSRG_ERR_UNSUPPORTED, std::string("generator type not on the GPU path: ") + t);
}

}  // namespace

// ------------------------------------------------------------------- solver
struct imsrg_solver {
  imsrg_space* sp = nullptr;
  const imsrg_op* H0 = nullptr;
  imsrg_op* Hs = nullptr;
  imsrg_op* Eta = nullptr;
  imsrg_op* Hsaved = nullptr;
  std::vector<imsrg_op*> omega;
  // IMSRGSolver(H) defaults, src/IMSRGSolver.cc:31-37
  double s = 0, ds = 0.1, ds_0 = 0.1, ds_max = 0.5, smax = 2.0, norm_domega = 0.1, omega_norm_max = 2.0;
  double eta_criterion = 1e-6;
  bool magnus_adaptive = true, hunter_gatherer = false;
  int istep = 0;
  // Generator() defaults, src/Generator.cc:18-20; BCH defaults, src/BCH.cc:16-17
  GenParams gen;
  double bch_transform_threshold = 1e-9, bch_product_threshold = 1e-4;
  struct Record {
    int istep;
    double s, e0, norm_eta, norm_omega;
  };
  std::vector<Record> history;
  // IMSRGSolver::SetScratchDir: split Omegas go to files instead of device
  // memory (src/IMSRGSolver.cc:44-83); max_omega_written as there
  std::string scratch;
  int n_written = 0, max_omega_written = 500;
  std::vector<std::string> files;
  // IMSRGSolver::method (src/IMSRGSolver.cc:201-234): 0 magnus_euler,
  // 1 magnus_modified_euler, 2 magnus_backoff, 3 flow_RK4; the back-off parameters and
  // state (src/IMSRGSolver.hh:73-78)
  int method = 0;
  double ds_backoff_factor = 0.5, ds_max_growth_factor = 1.2;
  bool soft_landing = false;
  imsrg_op* Htemp = nullptr;  // modified Euler's predicted H; RK4's stage H
  imsrg_op* Kstage = nullptr;  // RK4: [eta, H] of the current stage
  imsrg_op* Ksum = nullptr;    // RK4: K1 + 2 K2 + 2 K3 + K4
  // IMSRGSolver::AddOperator (src/IMSRGSolver.hh:94): flowing operators after
  // H(s), copies owned by the solver, each with RK4's stage operator, stage
  // [eta, O] and stage sum (allocated by the first RK4 solve)
  struct Flowing {
    imsrg_op *op = nullptr, *tmp = nullptr, *k = nullptr, *sum = nullptr;
  };
  std::vector<Flowing> flowing;

  ~imsrg_solver()
  {
    imsrg_op_destroy(Hs);
    imsrg_op_destroy(Eta);
    imsrg_op_destroy(Hsaved);
    imsrg_op_destroy(Htemp);
    imsrg_op_destroy(Kstage);
    imsrg_op_destroy(Ksum);
    for (Flowing& f : flowing) {
      imsrg_op_destroy(f.op);
      imsrg_op_destroy(f.tmp);
      imsrg_op_destroy(f.k);
      imsrg_op_destroy(f.sum);
    }
    for (imsrg_op* o : omega) imsrg_op_destroy(o);
    for (const std::string& f : files) std::remove(f.c_str());  // CleanupScratch
  }
};

namespace {

int new_zero_omega(imsrg_solver* sv, cudaStream_t st)
{
  imsrg_op* o = nullptr;
  FLOW_TRY(imsrg_op_create(sv->sp, -1, &o));
  sv->omega.push_back(o);
  (void)st;
  return IMSRG_OK;
}

// IMSRGSolver::NewOmega, src/IMSRGSolver.cc:44-83: with a scratch directory
// the finished Omega goes to a file (the reference's OMEGA_<pid><n> naming
// and binary layout) and its device operator is reused; without one a new
// device operator is kept
int new_omega(imsrg_solver* sv, cudaStream_t st)
{
  if (!sv->Hsaved) FLOW_TRY(imsrg_op_create(sv->sp, 1, &sv->Hsaved));
  FLOW_TRY(imsrg_op_copy(sv->Hsaved, sv->Hs, st));
  if (sv->scratch.empty()) return new_zero_omega(sv, st);
  if (sv->scratch.find("/dev/null") == std::string::npos) {
    char name[64];
    std::snprintf(name, sizeof(name), "/OMEGA_%06d%03d", (int)getpid(), sv->n_written);
    std::string path = sv->scratch + name;
    FLOW_TRY(imsrg_op_write_binary(sv->omega.back(), path.c_str(), st));
    sv->files.push_back(path);
    if (sv->n_written > sv->max_omega_written)
      return err(IMSRG_ERR_ARG, "more Omegas written than max_omega_written");
  }
  ++sv->n_written;
  FLOW_CUDA(cudaMemsetAsync(sv->omega.back()->d, 0, sv->sp->s->arena * sizeof(double), st));
  return IMSRG_OK;
}

// IMSRGSolver::GatherOmega, src/IMSRGSolver.cc:99-120
int gather_omega(imsrg_solver* sv, int prec, cudaStream_t st)
{
  if (sv->omega.size() < 2) {
    FLOW_TRY(new_zero_omega(sv, st));
    FLOW_TRY(imsrg_op_copy(sv->omega.back(), sv->omega[sv->omega.size() - 2], st));
  }
  imsrg_op* hunter = sv->omega.back();
  imsrg_op* gatherer = sv->omega[sv->omega.size() - 2];
  double nh = 0;
  FLOW_TRY(norm_dev(hunter, &nh, st));
  if (nh > 1e-6) FLOW_TRY(bch_product_impl(hunter, gatherer, gatherer, sv->bch_product_threshold, prec, nullptr, st));
  FLOW_CUDA(cudaMemsetAsync(hunter->d, 0, sv->sp->s->arena * sizeof(double), st));
  if (!sv->Hsaved) FLOW_TRY(imsrg_op_create(sv->sp, 1, &sv->Hsaved));
  FLOW_TRY(imsrg_op_copy(sv->Hsaved, sv->H0, st));
  for (size_t i = 0; i + 1 < sv->omega.size(); ++i)
    FLOW_TRY(imsrg_bch_transform(sv->Hsaved, sv->omega[i], sv->Hsaved, sv->bch_transform_threshold, prec, nullptr,
                                 st));
  return IMSRG_OK;
}

// IMSRGSolver::Solve_magnus_euler, src/IMSRGSolver.cc:236-321
int solve_magnus_euler(imsrg_solver* sv, int prec, cudaStream_t st)
{
  sv->istep = 0;
  FLOW_TRY(generator_impl(sv->Hs, sv->Eta, sv->gen, st));
  if (std::fabs(sv->omega_norm_max - sv->norm_domega) < 1e-6) sv->norm_domega += 1e-4;
  int rc = IMSRG_OK;
  double Elast = zero_body(sv->H0, st, &rc);
  if (rc) return rc;
  for (sv->istep = 1; sv->s < sv->smax; ++sv->istep) {
    double norm_eta = 0;
    FLOW_TRY(norm_dev(sv->Eta, &norm_eta, st));
    if (norm_eta < sv->eta_criterion) break;
    if (norm_eta > 1e12 || std::fabs(Elast) > 1e9) {
      // the reference multiplies H(s) by 1/0 and stops (:263-270)
      FLOW_TRY(imsrg_op_scale(sv->Hs, std::numeric_limits<double>::infinity(), st));
      return err(IMSRG_ERR_DIVERGED, "flow diverged: |eta| = " + std::to_string(norm_eta) +
                                         ", E0 = " + std::to_string(Elast));
    }
    double norm_omega = 0;
    FLOW_TRY(norm_dev(sv->omega.back(), &norm_omega, st));
    if (norm_omega > sv->omega_norm_max) {
      if (sv->hunter_gatherer)
        FLOW_TRY(gather_omega(sv, prec, st));
      else
        FLOW_TRY(new_omega(sv, st));
      norm_omega = 0;
    }
    if (sv->magnus_adaptive)
      sv->ds = std::min({sv->norm_domega / norm_eta, sv->norm_domega / norm_eta / (norm_omega + 1.0e-9),
                         (sv->omega_norm_max + 1e-5) / norm_eta, sv->ds_max});
    sv->ds = std::min(sv->ds, sv->smax - sv->s);
    sv->s += sv->ds;
    FLOW_TRY(imsrg_op_scale(sv->Eta, sv->ds, st));
    FLOW_TRY(bch_product_impl(sv->Eta, sv->omega.back(), sv->omega.back(), sv->bch_product_threshold, prec, nullptr,
                              st));
    const imsrg_op* Hin = sv->omega.size() + sv->n_written < 2 ? sv->H0 : sv->Hsaved;
    FLOW_TRY(imsrg_bch_transform(Hin, sv->omega.back(), sv->Hs, sv->bch_transform_threshold, prec, nullptr, st));
    FLOW_TRY(generator_impl(sv->Hs, sv->Eta, sv->gen, st));
    Elast = zero_body(sv->Hs, st, &rc);
    if (rc) return rc;
    sv->history.push_back({sv->istep, sv->s, Elast, norm_eta, norm_omega});
  }
  return IMSRG_OK;
}

// IMSRGSolver::Solve_magnus_modified_euler, src/IMSRGSolver.cc:449-504: the
// generator at the Euler-predicted H_temp = H + ds [eta, H] (Generator::
// AddToEta overwrites the elements Update wrote, so Eta becomes G(H_temp)),
// times ds / 2; no eta criterion, no Omega gathering
int solve_magnus_modified_euler(imsrg_solver* sv, int prec, cudaStream_t st)
{
  sv->istep = 0;
  FLOW_TRY(generator_impl(sv->Hs, sv->Eta, sv->gen, st));
  if (!sv->Htemp) FLOW_TRY(imsrg_op_create(sv->sp, 1, &sv->Htemp));
  int rc = IMSRG_OK;
  for (sv->istep = 1; sv->s < sv->smax; ++sv->istep) {
    double norm_eta = 0, norm_omega = 0;
    FLOW_TRY(norm_dev(sv->Eta, &norm_eta, st));
    FLOW_TRY(norm_dev(sv->omega.back(), &norm_omega, st));
    if (norm_omega > sv->omega_norm_max) {
      FLOW_TRY(new_omega(sv, st));
      norm_omega = 0;
    }
    sv->ds = std::min(std::min(sv->norm_domega / norm_eta, sv->norm_domega / norm_eta / (norm_omega + 1.0e-9)),
                      sv->ds_max);
    if (sv->s + sv->ds > sv->smax) sv->ds = sv->smax - sv->s;
    sv->s += sv->ds;
    FLOW_TRY(commutator_dev(sv->Eta, sv->Hs, sv->Htemp, prec, st));
    FLOW_TRY(imsrg_op_scale(sv->Htemp, sv->ds, st));
    FLOW_TRY(imsrg_op_axpy(sv->Htemp, 1.0, sv->Hs, st));
    sv->Htemp->herm = sv->Hs->herm;
    FLOW_TRY(generator_impl(sv->Htemp, sv->Eta, sv->gen, st));
    FLOW_TRY(imsrg_op_scale(sv->Eta, sv->ds * 0.5, st));
    FLOW_TRY(bch_product_impl(sv->Eta, sv->omega.back(), sv->omega.back(), sv->bch_product_threshold, prec, nullptr,
                              st));
    const imsrg_op* Hin = sv->omega.size() + sv->n_written < 2 ? sv->H0 : sv->Hsaved;
    FLOW_TRY(imsrg_bch_transform(Hin, sv->omega.back(), sv->Hs, sv->bch_transform_threshold, prec, nullptr, st));
    FLOW_TRY(generator_impl(sv->Hs, sv->Eta, sv->gen, st));
    const double e0 = zero_body(sv->Hs, st, &rc);
    if (rc) return rc;
    sv->history.push_back({sv->istep, sv->s, e0, norm_eta, norm_omega});
  }
  return IMSRG_OK;
}

// IMSRGSolver::Solve_magnus_backoff, src/IMSRGSolver.cc:324-447: Euler steps
// whose ds backs off (by ds_backoff_factor) while ds |eta| > pi/4 or when
// |eta| grew over the step, and grows (by ds_max_growth_factor, up to ds_max)
// otherwise, except in the soft-landing phase (|eta| < 20 eta_criterion)
int solve_magnus_backoff(imsrg_solver* sv, int prec, cudaStream_t st)
{
  sv->istep = 0;
  FLOW_TRY(generator_impl(sv->Hs, sv->Eta, sv->gen, st));
  int rc = IMSRG_OK;
  for (sv->istep = 1; sv->s < sv->smax; ++sv->istep) {
    double norm_eta = 0;
    FLOW_TRY(norm_dev(sv->Eta, &norm_eta, st));
    if (!sv->soft_landing && std::fabs(norm_eta) < sv->eta_criterion * 20.0) sv->soft_landing = true;
    if (norm_eta < sv->eta_criterion) break;
    while (sv->magnus_adaptive && sv->ds * norm_eta > M_PI_4) sv->ds = sv->ds * sv->ds_backoff_factor;
    double norm_omega = 0;
    FLOW_TRY(norm_dev(sv->omega.back(), &norm_omega, st));
    if (norm_omega > sv->omega_norm_max) {
      if (sv->hunter_gatherer)
        FLOW_TRY(gather_omega(sv, prec, st));
      else
        FLOW_TRY(new_omega(sv, st));
      norm_omega = 0;
    }
    sv->ds = std::min(sv->ds, sv->smax - sv->s);
    sv->s += sv->ds;
    FLOW_TRY(imsrg_op_scale(sv->Eta, sv->ds, st));
    FLOW_TRY(bch_product_impl(sv->Eta, sv->omega.back(), sv->omega.back(), sv->bch_product_threshold, prec, nullptr,
                              st));
    const imsrg_op* Hin = sv->omega.size() + sv->n_written < 2 ? sv->H0 : sv->Hsaved;
    FLOW_TRY(imsrg_bch_transform(Hin, sv->omega.back(), sv->Hs, sv->bch_transform_threshold, prec, nullptr, st));
    FLOW_TRY(generator_impl(sv->Hs, sv->Eta, sv->gen, st));
    if (sv->magnus_adaptive) {
      double norm_eta_new = 0;
      FLOW_TRY(norm_dev(sv->Eta, &norm_eta_new, st));
      if (norm_eta_new > norm_eta) {
        sv->ds = sv->ds * sv->ds_backoff_factor;
      } else if (!sv->soft_landing) {
        const double ds_new = std::min(sv->ds_max, sv->ds * sv->ds_max_growth_factor);
        if (ds_new > sv->ds) sv->ds = ds_new;
      }
    }
    const double e0 = zero_body(sv->Hs, st, &rc);
    if (rc) return rc;
    sv->history.push_back({sv->istep, sv->s, e0, norm_eta, norm_omega});
  }
  return IMSRG_OK;
}

// an operator of src's kind (scalar, or a reduced tensor of src's rank)
int create_like(const imsrg_op* src, imsrg_op** out)
{
  if (src->tl)
    return imsrg_op_create_tensor(src->sp, src->tl->lam, src->tl->trank, src->tl->parity, src->herm, out);
  return imsrg_op_create(src->sp, src->herm, out);
}

// [eta, O] for a scalar or tensor O, Commutator::Commutator's dispatch
// (src/Commutator.cc:106-160)
int flow_commutator(const imsrg_op* eta, const imsrg_op* O, imsrg_op* Z, int prec, cudaStream_t st)
{
  if (O->tl) return imsrg_commutator_scalar_tensor(eta, O, Z, prec, st);
  return commutator_dev(eta, O, Z, prec, st);
}

// IMSRGSolver::Solve_flow_RK4, src/IMSRGSolver.cc:505-636: the classical
// fixed-step RK4 rule for dH/ds = [eta(H), H] with steps of ds_max (the last
// one cut to end at smax), the generator re-evaluated at every stage's H;
// the operators added with AddOperator flow with the same stage generators
// (evaluated from H's stages only); no Omega, no goose-tank term (BCH's
// use_goose_tank_correction is off by default)
int solve_flow_rk4(imsrg_solver* sv, int prec, cudaStream_t st)
{
  sv->istep = 0;
  FLOW_TRY(generator_impl(sv->Hs, sv->Eta, sv->gen, st));
  if (!sv->Htemp) FLOW_TRY(imsrg_op_create(sv->sp, 1, &sv->Htemp));
  if (!sv->Kstage) FLOW_TRY(imsrg_op_create(sv->sp, 1, &sv->Kstage));
  if (!sv->Ksum) FLOW_TRY(imsrg_op_create(sv->sp, 1, &sv->Ksum));
  for (imsrg_solver::Flowing& f : sv->flowing) {
    if (!f.tmp) FLOW_TRY(create_like(f.op, &f.tmp));
    if (!f.k) FLOW_TRY(create_like(f.op, &f.k));
    if (!f.sum) FLOW_TRY(create_like(f.op, &f.sum));
  }
  // operator i of the flow: H(s) (i = 0) or an added one, with its stage
  // operator, stage [eta, O] and stage sum
  const size_t nops = sv->flowing.size() + 1;
  auto ops = [&](size_t i) {
    if (i == 0) return imsrg_solver::Flowing{sv->Hs, sv->Htemp, sv->Kstage, sv->Ksum};
    return sv->flowing[i - 1];
  };
  // weight of stage k's K in the sum, and the step fraction of the H that
  // feeds stage k + 1 (H + ds/2 K1, H + ds/2 K2, H + ds K3)
  const double wsum[4] = {1.0, 2.0, 2.0, 1.0};
  const double shift[3] = {0.5, 0.5, 1.0};
  int rc = IMSRG_OK;
  for (sv->istep = 1; sv->s < sv->smax; ++sv->istep) {
    double norm_eta = 0;
    FLOW_TRY(norm_dev(sv->Eta, &norm_eta, st));
    if (norm_eta < sv->eta_criterion) break;
    sv->ds = std::min(sv->ds_max, sv->smax - sv->s);
    sv->s += sv->ds;
    for (int k = 0; k < 4; ++k) {
      for (size_t i = 0; i < nops; ++i) {
        const imsrg_solver::Flowing f = ops(i);
        FLOW_TRY(flow_commutator(sv->Eta, k == 0 ? f.op : f.tmp, f.k, prec, st));
        if (k == 0)
          FLOW_TRY(imsrg_op_copy(f.sum, f.k, st));
        else
          FLOW_TRY(imsrg_op_axpy(f.sum, wsum[k], f.k, st));
        if (k < 3) {
          FLOW_TRY(imsrg_op_copy(f.tmp, f.op, st));
          FLOW_TRY(imsrg_op_axpy(f.tmp, shift[k] * sv->ds, f.k, st));
        }
      }
      if (k < 3) FLOW_TRY(generator_impl(sv->Htemp, sv->Eta, sv->gen, st));
    }
    for (size_t i = 0; i < nops; ++i) FLOW_TRY(imsrg_op_axpy(ops(i).op, sv->ds / 6.0, ops(i).sum, st));
    FLOW_TRY(generator_impl(sv->Hs, sv->Eta, sv->gen, st));
    const double e0 = zero_body(sv->Hs, st, &rc);
    if (rc) return rc;
    sv->history.push_back({sv->istep, sv->s, e0, norm_eta, 0.0});
  }
  return IMSRG_OK;
}

}  // namespace

extern "C" {

int imsrg_generator_update(const imsrg_op* H, imsrg_op* Eta, int type, int partitioning, double cutoff,
                           double delta, int delta_index, void* stream)
{
  if (!H || !Eta || H == Eta) return err(IMSRG_ERR_ARG, "bad operators");
  if (H->tl || Eta->tl) return err(IMSRG_ERR_UNSUPPORTED, "the generator takes scalar operators");
  if (H->sp != Eta->sp) return err(IMSRG_ERR_ARG, "operators belong to different model spaces");
  if ((type < IMSRG_GEN_WHITE || type > IMSRG_GEN_IMAGINARY_TIME) &&
      (type <= GEN_QTRANSFER_BASE || type > GEN_QTRANSFER_BASE + 16))
    return err(IMSRG_ERR_ARG, "bad generator type");
  if (partitioning != IMSRG_DENOM_EPSTEIN_NESBET && partitioning != IMSRG_DENOM_MOLLER_PLESSET)
    return err(IMSRG_ERR_ARG, "bad denominator partitioning");
  GenParams p;
  p.type = type;
  p.partitioning = partitioning;
  p.cutoff = cutoff;
  p.delta = delta;
  p.delta_index = delta_index;
  return generator_impl(H, Eta, p, S_(stream));
}

int imsrg_bch_product(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, double threshold, int precision,
                      int* n_commutators, void* stream)
{
  if (!X || !Y || !Z) return err(IMSRG_ERR_ARG, "null operator");
  if (X->sp != Y->sp || X->sp != Z->sp) return err(IMSRG_ERR_ARG, "operators belong to different model spaces");
  if (X->tl || Y->tl || Z->tl) return err(IMSRG_ERR_UNSUPPORTED, "BCH_Product of tensor operators is not on the GPU path");
  if ((X->herm != 1 && X->herm != -1) || (Y->herm != 1 && Y->herm != -1))
    return err(IMSRG_ERR_UNSUPPORTED, "X and Y must be hermitian or anti-hermitian");
  return bch_product_impl(X, Y, Z, threshold, precision, n_commutators, S_(stream));
}

int imsrg_solver_create(const imsrg_op* H0, imsrg_solver** out)
{
  if (!H0 || !out) return err(IMSRG_ERR_ARG, "bad arguments");
  if (H0->tl) return err(IMSRG_ERR_UNSUPPORTED, "the flow takes a scalar Hamiltonian");
  *out = nullptr;
  imsrg_solver* sv = new imsrg_solver();
  sv->sp = H0->sp;
  sv->H0 = H0;
  int rc;
  if ((rc = imsrg_op_create(sv->sp, H0->herm, &sv->Hs)) || (rc = imsrg_op_copy(sv->Hs, H0, nullptr)) ||
      (rc = imsrg_op_create(sv->sp, -1, &sv->Eta)) || (rc = new_zero_omega(sv, nullptr))) {
    delete sv;
    return rc;
  }
  if (cudaStreamSynchronize(nullptr) != cudaSuccess) {
    delete sv;
    return err(IMSRG_ERR_CUDA, "solver setup failed");
  }
  *out = sv;
  return IMSRG_OK;
}

void imsrg_solver_destroy(imsrg_solver* sv) { delete sv; }

int imsrg_solver_set(imsrg_solver* sv, const char* name, double v)
{
  if (!sv || !name) return err(IMSRG_ERR_ARG, "bad arguments");
  std::string n(name);
  if (n == "ds") sv->ds = sv->ds_0 = v;
  else if (n == "ds_max") sv->ds_max = v;
  else if (n == "smax") sv->smax = v;
  else if (n == "domega") sv->norm_domega = v;
  else if (n == "omega_norm_max") sv->omega_norm_max = v;
  else if (n == "eta_criterion") sv->eta_criterion = (double)(float)v;  // SetEtaCriterion(float)
  else if (n == "magnus_adaptive") sv->magnus_adaptive = v != 0;
  else if (n == "hunter_gatherer") sv->hunter_gatherer = v != 0;
  else if (n == "denominator_cutoff") sv->gen.cutoff = v;
  else if (n == "denominator_delta") sv->gen.delta = v;
  else if (n == "denominator_delta_index") sv->gen.delta_index = (int)v;
  else if (n == "bch_transform_threshold") sv->bch_transform_threshold = v;
  else if (n == "bch_product_threshold") sv->bch_product_threshold = v;
  else if (n == "max_omega_written") sv->max_omega_written = (int)v;
  else if (n == "method") {
    if (v != 0 && v != 1 && v != 2 && v != 3)
      return err(IMSRG_ERR_ARG, "method: 0 magnus_euler, 1 magnus_modified_euler, 2 magnus_backoff, 3 flow_RK4");
    sv->method = (int)v;
  }
  else if (n == "ds_backoff_factor") sv->ds_backoff_factor = v;
  else if (n == "ds_max_growth_factor") sv->ds_max_growth_factor = v;
  else return err(IMSRG_ERR_ARG, "unknown solver setting " + n);
  return IMSRG_OK;
}

int imsrg_solver_set_scratch_dir(imsrg_solver* sv, const char* dir)
{
  if (!sv || !dir) return err(IMSRG_ERR_ARG, "bad arguments");
  sv->scratch = dir;
  return IMSRG_OK;
}

int imsrg_solver_get(const imsrg_solver* sv, const char* name, double* v)
{
  if (!sv || !name || !v) return err(IMSRG_ERR_ARG, "bad arguments");
  std::string n(name);
  if (n == "s") *v = sv->s;
  else if (n == "ds") *v = sv->ds;
  else if (n == "ds_max") *v = sv->ds_max;
  else if (n == "smax") *v = sv->smax;
  else if (n == "domega") *v = sv->norm_domega;
  else if (n == "omega_norm_max") *v = sv->omega_norm_max;
  else if (n == "eta_criterion") *v = sv->eta_criterion;
  else if (n == "magnus_adaptive") *v = sv->magnus_adaptive;
  else if (n == "hunter_gatherer") *v = sv->hunter_gatherer;
  else if (n == "denominator_cutoff") *v = sv->gen.cutoff;
  else if (n == "denominator_delta") *v = sv->gen.delta;
  else if (n == "denominator_delta_index") *v = sv->gen.delta_index;
  else if (n == "bch_transform_threshold") *v = sv->bch_transform_threshold;
  else if (n == "bch_product_threshold") *v = sv->bch_product_threshold;
  else if (n == "n_omega") *v = (double)sv->omega.size();
  else if (n == "istep") *v = sv->istep;
  else if (n == "n_omega_written") *v = sv->n_written;
  else if (n == "max_omega_written") *v = sv->max_omega_written;
  else return err(IMSRG_ERR_ARG, "unknown solver setting " + n);
  return IMSRG_OK;
}

int imsrg_solver_set_generator(imsrg_solver* sv, const char* type, void* stream)
{
  if (!sv) return err(IMSRG_ERR_ARG, "null solver");
  int t = 0;
  FLOW_TRY(gen_type(type, &t));
  sv->gen.type = t;
  // IMSRGSolver::SetGenerator, src/IMSRGSolver.cc:157-183: a new generator
  // starts a new Omega once the current one is not empty
  cudaStream_t st = S_(stream);
  double no = 0;
  FLOW_TRY(norm_dev(sv->omega.back(), &no, st));
  if (no > 1e-6) {
    FLOW_CUDA(cudaMemsetAsync(sv->Eta->d, 0, sv->sp->s->arena * sizeof(double), st));
    if (sv->hunter_gatherer)
      FLOW_TRY(gather_omega(sv, IMSRG_PREC_FP64, st));
    else
      FLOW_TRY(new_omega(sv, st));
  }
  if (sv->magnus_adaptive) {
    sv->ds = sv->ds_0;
    sv->soft_landing = false;
  }
  return IMSRG_OK;
}

int imsrg_solver_set_denominator_partitioning(imsrg_solver* sv, const char* dp)
{
  if (!sv || !dp) return err(IMSRG_ERR_ARG, "bad arguments");
  // Generator::SetDenominatorPartitioning, src/Generator.cc:23-28
  if (!std::strcmp(dp, "MP_isospin")) return err(IMSRG_ERR_UNSUPPORTED, "MP_isospin partitioning is not on the GPU path");
  sv->gen.partitioning = !std::strcmp(dp, "Moller_Plesset") ? IMSRG_DENOM_MOLLER_PLESSET : IMSRG_DENOM_EPSTEIN_NESBET;
  return IMSRG_OK;
}

int imsrg_solver_solve(imsrg_solver* sv, int precision, void* stream)
{
  if (!sv) return err(IMSRG_ERR_ARG, "null solver");
  if (precision != IMSRG_PREC_FP64 && precision != IMSRG_PREC_SPLIT) return err(IMSRG_ERR_ARG, "bad precision");
  if (sv->method == 1) {
    ProfScope ps("Solve_magnus_modified_euler", S_(stream));
    return solve_magnus_modified_euler(sv, precision, S_(stream));
  }
  if (sv->method == 2) {
    ProfScope ps("Solve_magnus_backoff", S_(stream));
    return solve_magnus_backoff(sv, precision, S_(stream));
  }
  if (sv->method == 3) {
    ProfScope ps("Solve_flow_RK4", S_(stream));
    return solve_flow_rk4(sv, precision, S_(stream));
  }
  ProfScope ps("Solve_magnus_euler", S_(stream));
  return solve_magnus_euler(sv, precision, S_(stream));
}

int imsrg_solver_hs(imsrg_solver* sv, imsrg_op** out)
{
  if (!sv || !out) return err(IMSRG_ERR_ARG, "bad arguments");
  *out = sv->Hs;
  return IMSRG_OK;
}

int imsrg_solver_eta(imsrg_solver* sv, imsrg_op** out)
{
  if (!sv || !out) return err(IMSRG_ERR_ARG, "bad arguments");
  *out = sv->Eta;
  return IMSRG_OK;
}

int imsrg_solver_add_operator(imsrg_solver* sv, const imsrg_op* op, int* index, void* stream)
{
  if (!sv || !op) return err(IMSRG_ERR_ARG, "bad arguments");
  if (op->sp != sv->sp) return err(IMSRG_ERR_ARG, "the operator belongs to another model space");
  imsrg_solver::Flowing f;
  FLOW_TRY(create_like(op, &f.op));
  // the copy is complete on return, so the caller may free op
  int rc = imsrg_op_copy(f.op, op, S_(stream));
  if (!rc && cudaStreamSynchronize(S_(stream)) != cudaSuccess) rc = err(IMSRG_ERR_CUDA, "operator copy failed");
  if (rc) {
    imsrg_op_destroy(f.op);
    return rc;
  }
  sv->flowing.push_back(f);
  if (index) *index = (int)sv->flowing.size();
  return IMSRG_OK;
}

int imsrg_solver_get_operator(imsrg_solver* sv, int i, imsrg_op** out)
{
  if (!sv || !out) return err(IMSRG_ERR_ARG, "bad arguments");
  if (i < 0 || i > (int)sv->flowing.size()) return err(IMSRG_ERR_ARG, "operator index out of range");
  *out = i == 0 ? sv->Hs : sv->flowing[i - 1].op;
  return IMSRG_OK;
}

int imsrg_solver_omega(imsrg_solver* sv, int i, imsrg_op** out)
{
  if (!sv || !out) return err(IMSRG_ERR_ARG, "bad arguments");
  if (i < 0 || i >= (int)sv->omega.size()) return err(IMSRG_ERR_ARG, "Omega index out of range");
  *out = sv->omega[i];
  return IMSRG_OK;
}

int imsrg_solver_history(const imsrg_solver* sv, int cap, int* istep, double* s, double* e0, double* norm_eta,
                         double* norm_omega, int* n)
{
  if (!sv || !n) return err(IMSRG_ERR_ARG, "bad arguments");
  int m = (int)sv->history.size();
  *n = m;
  for (int i = 0; i < std::min(cap, m); ++i) {
    const auto& r = sv->history[i];
    if (istep) istep[i] = r.istep;
    if (s) s[i] = r.s;
    if (e0) e0[i] = r.e0;
    if (norm_eta) norm_eta[i] = r.norm_eta;
    if (norm_omega) norm_omega[i] = r.norm_omega;
  }
  return IMSRG_OK;
}

int imsrg_solver_transform(const imsrg_solver* sv, const imsrg_op* OpIn, imsrg_op* OpOut, int precision, void* stream)
{
  if (!sv || !OpIn || !OpOut) return err(IMSRG_ERR_ARG, "bad arguments");
  if (OpIn->sp != sv->sp || OpOut->sp != sv->sp) return err(IMSRG_ERR_ARG, "operator from another model space");
  if (OpIn->tl != OpOut->tl) return err(IMSRG_ERR_ARG, "OpIn and OpOut must have the same rank");
  cudaStream_t st = S_(stream);
  // IMSRGSolver::Transform_Partial(OpIn, 0), src/IMSRGSolver.cc:957-1002:
  // the Omegas written to scratch files first, then those in device memory
  FLOW_TRY(imsrg_op_copy(OpOut, OpIn, st));
  if (!sv->files.empty()) {
    imsrg_op* om = nullptr;
    FLOW_TRY(imsrg_op_create(sv->sp, -1, &om));
    int rc = IMSRG_OK;
    for (size_t i = 0; rc == IMSRG_OK && i < sv->files.size(); ++i) {
      rc = imsrg_op_read_binary(om, sv->files[i].c_str(), st);
      if (!rc) rc = imsrg_bch_transform(OpOut, om, OpOut, sv->bch_transform_threshold, precision, nullptr, st);
    }
    cudaStreamSynchronize(st);
    imsrg_op_destroy(om);
    if (rc) return rc;
  }
  for (imsrg_op* om : sv->omega)
    FLOW_TRY(imsrg_bch_transform(OpOut, om, OpOut, sv->bch_transform_threshold, precision, nullptr, st));
  return IMSRG_OK;
}

int imsrg_solver_inverse_transform(const imsrg_solver* sv, const imsrg_op* OpIn, imsrg_op* OpOut, int precision,
                                   void* stream)
{
  if (!sv || !OpIn || !OpOut) return err(IMSRG_ERR_ARG, "bad arguments");
  if (OpIn->sp != sv->sp || OpOut->sp != sv->sp) return err(IMSRG_ERR_ARG, "operator from another model space");
  if (OpIn->tl != OpOut->tl) return err(IMSRG_ERR_ARG, "OpIn and OpOut must have the same rank");
  cudaStream_t st = S_(stream);
  // IMSRGSolver::InverseTransform, src/IMSRGSolver.cc:939-952: Omegas in
  // reverse order, each negated
  imsrg_op* neg = nullptr;
  FLOW_TRY(imsrg_op_create(sv->sp, -1, &neg));
  int rc = imsrg_op_copy(OpOut, OpIn, st);
  for (size_t i = sv->omega.size(); rc == IMSRG_OK && i-- > 0;) {
    rc = imsrg_op_copy(neg, sv->omega[i], st);
    if (!rc) rc = imsrg_op_scale(neg, -1.0, st);
    if (!rc) rc = imsrg_bch_transform(OpOut, neg, OpOut, sv->bch_transform_threshold, precision, nullptr, st);
  }
  cudaStreamSynchronize(st);
  imsrg_op_destroy(neg);
  return rc;
}

}  // extern "C"
